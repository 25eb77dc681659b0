"""The bench workload itself against the oracle: the unit cube of 96^3 hexahedra x 6 =
5,308,416 tetrahedra with seeded node jitter, the sinusoidal state, slip walls, BDF2 at
dt = 5e-4, Newton tolerance 1e-8, GMRES(30) with ILU(0).

- FP64 residual within 1e-11 of the oracle's rhs (foeuler.f90:349-375, Euler.f90:25-156),
  finite-difference Jv within 1e-6 of the oracle driver's;
- one ILU(0) apply (P factored in the same elimination order) within 1e-10;
- two BDF2 steps of the plain FP64 path within 1e-10 per conserved field, with the oracle's
  Newton and Krylov iteration counts;
- the FP32 forms (FP32 flux + FP32 colour-ordered ILU(0), alone and with the learned
  preconditioner in FGMRES) after the same two steps, against the FP64 oracle's state, in the
  relative l2 norm, per cell and per field; both stop Newton at ||G||_2 <= 1e-8 ||y_n||_2,
  and in the largest-field norm that tolerance alone separates two FP64 runs that differ
  only in their Krylov path (the yardstick below).

The oracle runs with OpenMP in its residual loops (atomic scatter, so its sums are not in a
fixed order); that changes its results at the 1e-16 level only."""
import os

import numpy as np
import pytest

from fosolvers_gb300 import mesh as M
from fosolvers_gb300.euler import FLUX_FP32, ILU_COLOR, ILU_FP32, FOEuler
from helpers import Case, cell_errors, field_errors, rel_err
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu

NSTEPS = 2
_state: dict = {}


@pytest.fixture(scope="module")
def full(cuda):
    c = Case(M.make_workload("sine96"))
    assert c.nC == 96 ** 3 * 6
    c.oracle.set_threads(os.cpu_count() or 1)
    yield c
    c.oracle.close()
    if c._gpu is not None:
        c._gpu.close()


def _oracle_steps(c: Case, rtol: float):
    key = ("oracle", rtol)
    if key not in _state:
        wl = c.wl
        c.match_ilu_order()
        rhs, pset, psol = c.oracle.callbacks()
        y = c.y0.copy()
        rc, st = O.bdf_run(c.N, rhs, pset, psol, c.oracle.h, y,
                           O.bdf_defaults(order=wl.order, dt=wl.dt, nsteps=NSTEPS,
                                          newton_rtol=rtol))
        assert rc == 0, st
        _state[key] = (y, st)
    return _state[key]


def _gpu_steps(c: Case, flags: int, precond: int, rtol: float, max_newton: int = 20):
    import torch
    wl = c.wl
    if flags == 0:
        ctx = c.gpu  # the FP64 context whose elimination order the oracle uses
    else:
        ctx = FOEuler(c.grid, c.iBC, wl.bc_type, wl.bc_param, wl.gamm, wl.r, flags=flags)
    gnn = None
    if precond == 2:
        from fosolvers_gb300.learned import DEFAULT_WEIGHTS, GNN
        gnn = GNN(seed=0)
        gnn.load(DEFAULT_WEIGHTS)
        ctx.attach_gnn(gnn)
    yr = torch.from_numpy(c.y0).cuda()
    y = torch.empty_like(yr)
    ctx.to_internal(yr, y)
    rc, st = ctx.bdf_run(y, ctx.bdf_defaults(order=wl.order, dt=wl.dt, nsteps=NSTEPS,
                                             precond=precond, newton_rtol=rtol,
                                             max_newton=max_newton))
    assert rc == 0, st
    ctx.to_reference(y, yr)
    torch.cuda.synchronize()
    out = yr.cpu().numpy()
    if flags != 0:
        ctx.close()
    if gnn is not None:
        gnn.close()
    return out, st


def test_fullsize_residual_and_jv(full):
    c = full
    y = c.y0
    ref = c.oracle_rhs(y)
    out = np.zeros_like(y)
    assert c.gpu.rhs(0.0, y, out) == 0
    err = rel_err(out, ref)
    print("residual", err)
    assert err <= 1e-11
    # the finite-difference Jv at the workload's gamma, FP64 increment
    import torch
    gamma = c.wl.dt * 2.0 / 3.0
    eps = float(np.sqrt(np.finfo(np.float64).eps))
    v = np.random.default_rng(3).normal(size=c.N)
    ynorm = float(np.linalg.norm(y))
    jref = np.empty_like(y)
    assert c.oracle.jv(y, ref, v, jref, 1.0, -gamma, ynorm, eps) == 0
    dev = lambda a: torch.from_numpy(a).cuda()
    yi, fi, vi, o, tmp = (torch.empty(c.N, dtype=torch.float64, device="cuda") for _ in range(5))
    c.gpu.to_internal(dev(y), yi)
    c.gpu.rhs_dev(0.0, yi, fi)
    c.gpu.to_internal(dev(v), vi)
    c.gpu.jv_dev(0.0, yi, fi, vi, o, 1.0, -gamma, ynorm, eps)
    c.gpu.to_reference(o, tmp)
    got = tmp.cpu().numpy()
    ejv = rel_err(got, jref)
    # the same product with ||v|| supplied by the caller (no norm pass)
    c.gpu.jv_dev_vnorm(0.0, yi, fi, vi, o, 1.0, -gamma, ynorm, float(np.linalg.norm(v)), eps)
    c.gpu.to_reference(o, tmp)
    ejv2 = rel_err(tmp.cpu().numpy(), jref)
    print("jv", ejv, ejv2)
    assert ejv <= 1e-6 and ejv2 <= 1e-6


def test_fullsize_ilu_apply(full):
    c = full
    gamma = c.wl.dt * 2.0 / 3.0
    c.match_ilu_order()
    assert c.oracle.pset(0.0, c.y0, None, 0, gamma) == (0, 1)
    rc, _ = c.gpu.pset(0.0, c.y0, None, 0, gamma)
    assert rc == 0
    r = np.random.default_rng(5).normal(size=c.N)
    z_ref, z = np.zeros_like(r), np.zeros_like(r)
    c.oracle.psol(0.0, None, None, r, z_ref, gamma)
    assert c.gpu.psol(0.0, c.y0, None, r, z, gamma) == 0
    err = rel_err(z, z_ref)
    print("ilu apply", err)
    assert err <= 1e-10


def test_fullsize_bdf2_fp64_matches_oracle(full):
    c = full
    y_ref, st_ref = _oracle_steps(c, 1e-8)
    y, st = _gpu_steps(c, 0, 1, 1e-8)
    err = rel_err(y, y_ref)
    print("fp64 bdf2", err, cell_errors(y, y_ref), st, st_ref)
    assert st["n_newton"] == st_ref["n_newton"]
    assert st["n_lin_iters"] == st_ref["n_lin_iters"]
    assert err <= 1e-10


@pytest.mark.parametrize("precond", [1, 2], ids=["ilu", "learned"])
def test_fullsize_fp32_forms_against_oracle(full, precond):
    """FP32 flux + FP32 colour ILU(0) (precond 1) and the same with the learned
    preconditioner in FGMRES (precond 2) against the FP64 oracle after two BDF2 steps at the
    workload's Newton tolerance 1e-8, and at 1e-9.

    Yardstick: the FP64 flux with the learned preconditioner -- the oracle's arithmetic on
    another Krylov path -- lands as far from the oracle in the largest-field norm as the
    Newton tolerance allows; the FP32 forms must stay within a small multiple of it, within
    1e-7 in the relative l2 norm (the norm of the Newton test) and within 3e-6 per cell.
    At 1e-9 the per-cell difference must fall.  (The FP32 flux's rounding puts a floor of
    about 2e-10 ||y|| under the Newton residual, so 1e-10 is out of its reach.)"""
    c = full
    flags = FLUX_FP32 | ILU_FP32 | ILU_COLOR
    y_ref, _ = _oracle_steps(c, 1e-8)
    if "fp64_learned" not in _state:
        _state["fp64_learned"] = _gpu_steps(c, ILU_COLOR, 2, 1e-8)
    y64, _ = _state["fp64_learned"]
    fe64 = field_errors(y64, y_ref)
    yard = max(fe64["rho"], fe64["rhou"], fe64["rhoE"])
    res = {}
    for rtol in (1e-8, 1e-9):
        yr, _ = _oracle_steps(c, rtol)
        y, st = _gpu_steps(c, flags, precond, rtol)
        fe = field_errors(y, yr)
        res[rtol] = {"field": max(fe["rho"], fe["rhou"], fe["rhoE"]), "fields": fe,
                     "cell": cell_errors(y, yr),
                     "l2": float(np.linalg.norm(y - yr) / np.linalg.norm(yr)), "stats": st}
        print(f"fp32 precond {precond} rtol {rtol:g}: {res[rtol]}")
    print(f"yardstick (FP64 flux, learned FGMRES, rtol 1e-8): field {yard:.3e}, "
          f"cell {cell_errors(y64, y_ref)}")
    r8 = res[1e-8]
    assert r8["l2"] <= 1e-7
    assert r8["cell"]["cell"] <= 3e-6
    assert r8["field"] <= max(5.0 * yard, 1e-6)
    assert res[1e-9]["cell"]["cell"] < r8["cell"]["cell"]
