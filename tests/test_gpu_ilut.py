"""ILUT on the GPU (fos_ilut_*) against the oracle's restatement of SPARSKIT ilut + lusol.

Given the same CSR matrix the GPU factors must equal the oracle's bit for bit in ilut's MSR
layout (inverted diagonal, L then U per row, the entries quick-split kept and in the same
positions); the sweeps (a fixed-order warp sum per row instead of lusol's sequential one)
within 1e-12.  Through the Euler preconditioner (P assembled on the GPU from its own
Jacobian, which matches the oracle's to rounding) psol within 1e-9, and a BDF run with ILUT
within 1e-10 of the oracle's."""
import numpy as np
import pytest

from fosolvers_gb300 import mesh as M
from fosolvers_gb300.euler import PREC_ILUT
from helpers import Case, perturbed, rel_err
from oracle import pyoracle as O
from test_oracle_kat import COO, _csr, _random_csr

pytestmark = pytest.mark.gpu


def gpu_ilu(n, a, ja1, ia1, lfil, droptol):
    """factor a 1-based CSR matrix with the GPU ILU class; returns the ILU object"""
    import torch
    from fosolvers_gb300.ilut import ILU
    p = ILU(n, lfil)
    dev = lambda x, t: torch.from_numpy(np.ascontiguousarray(x, t)).cuda()
    p.factor_csr(dev(np.asarray(ia1) - 1, np.int32), dev(np.asarray(ja1) - 1, np.int32),
                 dev(a, np.float64), droptol)
    return p


def assert_same_factors(p, ref):
    alu, jlu, ju = p.msr()
    ralu, rjlu, rju = ref
    assert np.array_equal(ju, rju)
    assert np.array_equal(jlu, rjlu[:len(jlu)]) and len(jlu) == len(rjlu)
    assert np.array_equal(alu[:p.n], ralu[:p.n])
    assert np.array_equal(alu[p.n + 1:], ralu[p.n + 1:len(alu)])


def oracle_ilut(n, a, ja1, ia1, lfil, droptol):
    ierr, alu, jlu, ju = O.ilut(n, a, ja1, ia1, lfil, droptol)
    assert ierr == 0
    used = int(jlu[n]) - 1
    return alu[:used], jlu[:used], ju


def test_ilu1_kat(cuda):
    """src/test/ILU1.f90:11-22 through the GPU ILU class: init(4, 7, 4), setCOO, fact(0),
    solve: x = [1, 3/2, 14/5, 11/4] within 1e-9, factors identical to the oracle's."""
    from fosolvers_gb300.ilut import ILU
    p = ILU(4, 4)
    assert p.lfil == 3
    p.set_coo(COO["iA"], COO["jA"], COO["A"])
    p.fact(0.0)
    x = p.solve([1.0, 2.0, 3.0, 4.0])
    assert np.linalg.norm(x - [1.0, 1.5, 2.8, 2.75]) <= 1e-9
    ao, jao, iao = _csr()
    assert_same_factors(p, oracle_ilut(4, ao, jao, iao, 4, 0.0))


@pytest.mark.parametrize("n,density,lfil,droptol,seed", [
    (40, 0.15, 39, 0.0, 1), (200, 0.05, 10, 1e-3, 2), (300, 0.03, 5, 1e-2, 3),
    (500, 0.02, 50, 1e-6, 4), (120, 0.3, 8, 1e-4, 5)])
def test_random_matrices_bitwise(cuda, n, density, lfil, droptol, seed):
    A, a, ja, ia = _random_csr(n, density, seed)
    ref = oracle_ilut(n, a, ja, ia, lfil, droptol)
    p = gpu_ilu(n, a, ja, ia, lfil, droptol)
    assert_same_factors(p, ref)
    y = np.random.default_rng(seed).normal(size=n)
    x = p.solve(y)
    xr = O.lusol(n, y, *ref)
    assert np.abs(x - xr).max() <= 1e-12 * np.abs(xr).max()


def test_long_rows_grow_the_working_capacity(cuda):
    """A dense last row and dense columns make rows longer than the first working capacity
    (256 entries of L and of U); the factorisation is redone with a larger one."""
    n = 600
    rng = np.random.default_rng(9)
    A = np.diag(10.0 + rng.random(n))
    A[-1, :] = rng.normal(size=n) * 0.01
    A[:, -1] = rng.normal(size=n) * 0.01
    A[-1, -1] = 20.0
    A[:, 0] += rng.normal(size=n) * 0.01
    ia = np.zeros(n + 1, np.int32)
    ja, a = [], []
    for i in range(n):
        c = np.flatnonzero(A[i])
        ja += list(c + 1)
        a += list(A[i, c])
        ia[i + 1] = ia[i] + len(c)
    ja, a, ia = np.array(ja, np.int32), np.array(a), ia + 1
    ref = oracle_ilut(n, a, ja, ia, n, 0.0)
    p = gpu_ilu(n, a, ja, ia, n, 0.0)
    from fosolvers_gb300 import _lib
    import ctypes as C
    info = (C.c_long * 6)()
    _lib.lib().fos_ilut_info(p.handle, info)
    assert info[2] > 256
    assert_same_factors(p, ref)


def test_zero_row_is_reported(cuda):
    a = np.array([2.0, 0.0, 3.0])
    ia = np.array([1, 2, 3, 4], np.int32)
    ja = np.array([1, 2, 3], np.int32)
    with pytest.raises(RuntimeError, match="zero row 2"):
        gpu_ilu(3, a, ja, ia, 2, 0.0)


@pytest.fixture(scope="module")
def euler(cuda):
    c = Case(M.make_workload("sine96", scale=8, seed=1), flags=PREC_ILUT)
    c.match_ilu_order()
    c.oracle.set_ilut(50, 1e-6)
    return c


def test_euler_P_factors_bitwise(euler):
    """fopbc's parameters (fill 50, drop 1e-6) on the oracle's P of the sine workload
    (3,072 cells, 15,360 unknowns): GPU factors of the same CSR equal the oracle's."""
    c = euler
    y = perturbed(c.y0, c.nC, 3)
    assert c.oracle.pset(0.0, y, None, 0, 5e-3) == (0, 1)
    a, ja, ia = c.oracle.pmat()
    p = gpu_ilu(5 * c.nC, a, ja, ia, 50, 1e-6)
    assert_same_factors(p, c.oracle.ilut_factors())


def test_euler_psol_with_ilut(euler):
    """pset/psol of a PREC_ILUT context (P assembled on the GPU) against the oracle's
    ILUT pset/psol in the same elimination order."""
    c = euler
    y = perturbed(c.y0, c.nC, 4)
    gamma = 5e-3
    assert c.oracle.pset(0.0, y, None, 0, gamma) == (0, 1)
    rc, _ = c.gpu.pset(0.0, y, None, 0, gamma)
    assert rc == 0
    rng = np.random.default_rng(8)
    for _ in range(2):
        r = rng.normal(size=c.N)
        z_ref, z = np.zeros_like(r), np.zeros_like(r)
        c.oracle.psol(0.0, None, None, r, z_ref, gamma)
        assert c.gpu.psol(0.0, y, None, r, z, gamma) == 0
        assert rel_err(z, z_ref) <= 1e-9


def test_bdf_with_ilut_matches_oracle(cuda):
    """BDF2 on the sine workload at 8^3 x 6 with GMRES(30) + ILUT(50, 1e-6) on both sides:
    the same Newton and Krylov counts, state within 1e-10."""
    import torch
    wl = M.make_workload("sine96", scale=8, seed=1)
    c = Case(wl, flags=PREC_ILUT)
    c.match_ilu_order()
    c.oracle.set_ilut(50, 1e-6)
    rhs, pset, psol = c.oracle.callbacks()
    y_ref = c.y0.copy()
    rc, st_ref = O.bdf_run(c.N, rhs, pset, psol, c.oracle.h, y_ref,
                           O.bdf_defaults(order=2, dt=wl.dt, nsteps=4, use_prec=1))
    assert rc == 0
    yr = torch.from_numpy(c.y0).cuda()
    yi = torch.empty_like(yr)
    c.gpu.to_internal(yr, yi)
    rc, st = c.gpu.bdf_run(yi, c.gpu.bdf_defaults(order=2, dt=wl.dt, nsteps=4, precond=1))
    assert rc == 0, st
    c.gpu.to_reference(yi, yr)
    torch.cuda.synchronize()
    print("ilut bdf", st, st_ref)
    assert st["n_lin_iters"] == st_ref["n_lin_iters"] and st["n_newton"] == st_ref["n_newton"]
    assert rel_err(yr.cpu().numpy(), y_ref) <= 1e-10
