"""Failure detection without a GPU fault: every failure is made on the host or by a bounded
wait that a test lets run out, the library reports it through its return codes, and the
context stays usable afterwards.

- ILUT dependency waits (fos_ilut_*): a short wait limit and a row that is never published
  (a flag nothing sets).  Every wait returns; the factorisation reports -6 and a solve
  leaves fos_ilut_status at -6 with NaN in the rows that waited; with the row published
  again, the same object factors and solves as the oracle does.
- Block ILU(0) zero pivot: a Jacobian whose first eliminated pivot block makes
  P = I - gamma/v J exactly singular, loaded with fos_euler_jac_set; pset returns 1, the
  recoverable code (the analogue of ilu0's ierr = k, ITSOL/ilut.f:1896,1911), and the
  driver returns 3 on it.
- Forced GMRES non-convergence: GMRES(1) without restarts, an unreachable linear tolerance
  and two Newton iterations on the bump at CFL ~5; the driver returns 1 and leaves the
  state at the last accepted step, like the oracle's driver."""
import time

import numpy as np
import pytest

from fosolvers_gb300 import mesh as M
from helpers import Case, rel_err
from oracle import pyoracle as O
from test_gpu_ilut import assert_same_factors, gpu_ilu, oracle_ilut
from test_oracle_kat import _random_csr

pytestmark = pytest.mark.gpu


def _chain_csr(n: int, seed: int):
    """A diagonally dominant matrix whose every row depends on the row above (L entry at
    i - 1) and on a few random earlier rows, 1-based CSR."""
    rng = np.random.default_rng(seed)
    rows = []
    for i in range(n):
        cols = {i: 4.0 + rng.random()}
        if i > 0:
            cols[i - 1] = -1.0 + 0.1 * rng.random()
        if i + 1 < n:
            cols[i + 1] = -1.0 + 0.1 * rng.random()
        for j in rng.integers(0, max(i, 1), size=2):
            if j < i - 1:
                cols[int(j)] = 0.1 * rng.normal()
        rows.append(sorted(cols.items()))
    ia = np.ones(n + 1, np.int32)
    ja, a = [], []
    for i, r in enumerate(rows):
        ja += [c + 1 for c, _ in r]
        a += [v for _, v in r]
        ia[i + 1] = ia[i] + len(r)
    return np.array(a), np.array(ja, np.int32), ia


def test_ilut_factor_wait_runs_out(cuda):
    from fosolvers_gb300.ilut import ILU
    import torch
    n = 3000
    a, ja, ia = _chain_csr(n, 1)
    dev = lambda x, t: torch.from_numpy(np.ascontiguousarray(x, t)).cuda()
    csr = (dev(ia - 1, np.int32), dev(ja - 1, np.int32), dev(a, np.float64))
    p = ILU(n, 10)
    p.set_wait_limit(polls=4096, withhold_row=100)
    t0 = time.perf_counter()
    with pytest.raises(RuntimeError, match="dependency wait ran out"):
        p.factor_csr(*csr, 0.0)
    assert time.perf_counter() - t0 < 60.0
    # every row published again, default limit: the same object factors as ilut does
    p.set_wait_limit(0, -1)
    p.factor_csr(*csr, 0.0)
    assert_same_factors(p, oracle_ilut(n, a, ja, ia, 10, 0.0))


def test_ilut_solve_wait_runs_out(cuda):
    import torch
    from fosolvers_gb300 import _lib
    n = 500
    A, a, ja, ia = _random_csr(n, 0.02, 4)
    p = gpu_ilu(n, a, ja, ia, 20, 1e-6)
    ref = oracle_ilut(n, a, ja, ia, 20, 1e-6)
    y = np.random.default_rng(2).normal(size=n)
    x_ref = O.lusol(n, y, *ref)
    p.set_wait_limit(polls=4096, withhold_row=0)
    yd = torch.from_numpy(y).cuda()
    xd = torch.empty_like(yd)
    t0 = time.perf_counter()
    p.solve_dev(yd, xd)
    torch.cuda.synchronize()
    assert time.perf_counter() - t0 < 60.0
    assert _lib.lib().fos_ilut_status(p.handle) == -6
    assert not np.isfinite(xd.cpu().numpy()).all()
    p.set_wait_limit(0, -1)
    x = p.solve(y)  # raises if the status is not 0
    assert np.abs(x - x_ref).max() <= 1e-12 * np.abs(x_ref).max()


def _exact_unit_gamma(inv_v: float):
    """gamma with gamma * inv_v == 1.0 exactly in binary64 (the factor's scale factor), or
    None (for a few values of inv_v no binary64 gamma gives exactly 1)."""
    g = 1.0 / inv_v
    for _ in range(64):
        prod = g * inv_v
        if prod == 1.0:
            return g
        g = np.nextafter(g, -np.inf if prod > 1.0 else np.inf)
    return None


@pytest.mark.parametrize("fp32", [False, True], ids=["fp64", "fp32"])
def test_block_ilu0_zero_pivot_is_recoverable(cuda, fp32):
    import torch
    from fosolvers_gb300.euler import ILU_COLOR, ILU_FP32
    c = Case(M.make_workload("sod16", scale=6), flags=ILU_COLOR | (ILU_FP32 if fp32 else 0))
    g = c.gpu
    assert g.pset(0.0, c.y0, None, 0, 1e-3) == (0, 1)
    rowptr, col, val = g.jacobian()
    # a row without L blocks (the first colour) has its own P_pp as pivot block; take one
    # whose cell volume admits a gamma with (gamma / v) exactly 1
    old2pos = g.ilu_order()
    pos2old = np.argsort(old2pos)
    p = gamma = None
    for q in range(c.nC):
        if col[rowptr[q]] != q:
            continue  # the row has L blocks
        gamma = _exact_unit_gamma(1.0 / float(c.grid.v[pos2old[q]]))  # 1/v as the context
        if gamma is not None:
            p = q
            break
    assert p is not None
    s = int(rowptr[p])  # the diagonal block comes first in such a row
    bad = val.copy()
    bad[s, 0, 0] = 1.0  # P_pp(0, 0) = 1 - (gamma / v) * 1 = 0 exactly
    g.set_jacobian(bad)
    rc, jcur = g.pset(0.0, c.y0, None, 1, gamma)
    assert rc == 1 and jcur == 0  # recoverable, J kept
    # a fresh assembly at the same gamma factors again
    assert g.pset(0.0, c.y0, None, 0, gamma) == (0, 1)
    r = np.random.default_rng(0).normal(size=c.N)
    z = np.zeros_like(r)
    assert g.psol(0.0, c.y0, None, r, z, gamma) == 0 and np.isfinite(z).all()
    # the driver on the singular set-up: returns 3 (zero pivot), state not advanced
    g.set_jacobian(bad)
    yr = torch.from_numpy(c.y0).cuda()
    y = torch.empty_like(yr)
    g.to_internal(yr, y)
    y_before = y.clone()
    opts = g.bdf_defaults(order=1, dt=gamma, nsteps=1, jac_reuse=1)
    rc, st = g.bdf_run(y, opts)
    assert rc == 3 and st["n_steps"] == 0
    assert torch.equal(y, y_before)


def test_forced_gmres_failure_returns_one_and_keeps_state(cuda):
    """GMRES(1), no restarts, lin_rtol 1e-30, no preconditioner, at most two Newton
    iterations, on the supersonic bump at CFL ~5: the Newton iteration cannot reach 1e-8.
    Both drivers return 1 after the same work and leave y at the initial (last accepted)
    state; afterwards the context runs normally."""
    import torch
    c = Case(M.make_workload("bump192", scale=12))
    wl = c.wl
    kw = dict(order=1, dt=wl.dt, nsteps=2, maxl=1, max_restarts=0, lin_rtol=1e-30,
              max_newton=2)
    c.match_ilu_order()
    rhs, pset, psol = c.oracle.callbacks()
    y_o = c.y0.copy()
    rc_o, st_o = O.bdf_run(c.N, rhs, pset, psol, c.oracle.h, y_o,
                           O.bdf_defaults(use_prec=0, **kw))
    assert rc_o == 1 and st_o["n_steps"] == 0 and st_o["fails"] == 1
    assert np.array_equal(y_o, c.y0)
    yr = torch.from_numpy(c.y0).cuda()
    y = torch.empty_like(yr)
    c.gpu.to_internal(yr, y)
    y0 = y.clone()
    rc, st = c.gpu.bdf_run(y, c.gpu.bdf_defaults(precond=0, **kw))
    assert rc == 1 and st["n_steps"] == 0 and st["fails"] == 1
    assert st["n_newton"] == st_o["n_newton"] and st["n_lin_iters"] == st_o["n_lin_iters"]
    assert torch.equal(y, y0)
    # the same context, normal options: the steps converge and match the oracle
    rc, st = c.gpu.bdf_run(y, c.gpu.bdf_defaults(order=1, dt=wl.dt, nsteps=2, precond=1))
    assert rc == 0
    y_o = c.y0.copy()
    rc_o, _ = O.bdf_run(c.N, rhs, pset, psol, c.oracle.h, y_o,
                        O.bdf_defaults(order=1, dt=wl.dt, nsteps=2, use_prec=1))
    assert rc_o == 0
    c.gpu.to_reference(y, yr)
    torch.cuda.synchronize()
    assert rel_err(yr.cpu().numpy(), y_o) <= 1e-10
