"""The FP32 flux on the supersonic bump channel (static Mach 2 inflow, code 10, zero-gradient
outflow, slip walls; BDF1 at CFL ~5, Newton 1e-8, GMRES(30) with the FP32 colour-ordered
ILU(0)) -- the precision form of the bump workloads.

Plain FP32 rounds the large jumps at the shock in FP32, which puts the Newton residual's
floor above the 1e-8 tolerance.  FOS_FLUX_HYBRID evaluates the faces whose relative density
or pressure jump exceeds 5% (and the boundary faces) in FP64 and the rest in FP32; it must
converge every step, stay conservative, and land within 1e-6 of the FP64 oracle in every
conserved field.  Where no face crosses the threshold it must equal the plain FP32 flux
bit for bit."""
import numpy as np
import pytest

from fosolvers_gb300 import mesh as M
from fosolvers_gb300.euler import FLUX_FP32, FLUX_HYBRID, ILU_COLOR, ILU_FP32
from helpers import Case, cell_errors, field_errors, perturbed, rel_err
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu

HYB = FLUX_FP32 | FLUX_HYBRID | ILU_FP32 | ILU_COLOR


def _gpu_steps(c: Case, nsteps: int, **kw):
    import torch
    wl = c.wl
    yr = torch.from_numpy(c.y0).cuda()
    y = torch.empty_like(yr)
    c.gpu.to_internal(yr, y)
    rc, st = c.gpu.bdf_run(y, c.gpu.bdf_defaults(order=wl.order, dt=wl.dt, nsteps=nsteps,
                                                 precond=1, **kw))
    c.gpu.to_reference(y, yr)
    torch.cuda.synchronize()
    return rc, st, yr.cpu().numpy()


def test_hybrid_flux_residual_against_oracle(cuda):
    """One residual of the hybrid flux on a state with large jumps: within 2e-5 of the FP64
    oracle like the FP32 flux (the FP64 faces are at least as accurate); with the threshold
    above every jump the interior faces are the plain FP32 flux's, so every cell without a
    boundary face equals the plain FP32 residual bit for bit."""
    wl = M.make_workload("bump192", scale=24)
    c = Case(wl, flags=HYB)
    y = perturbed(c.y0, c.nC, 3, amp=0.3)  # jumps of up to ~60% between neighbours
    ref = c.oracle_rhs(y)
    out = np.zeros_like(y)
    assert c.gpu.rhs(0.0, y, out) == 0
    err = rel_err(out, ref)
    c32 = Case(wl, flags=FLUX_FP32 | ILU_FP32 | ILU_COLOR)
    out32 = np.zeros_like(y)
    assert c32.gpu.rhs(0.0, y, out32) == 0
    err32 = rel_err(out32, ref)
    print("hybrid residual", err, "fp32", err32)
    assert err <= 2e-5 and err <= err32
    c.gpu.set_flux_threshold(1e30)
    out_hi = np.zeros_like(y)
    assert c.gpu.rhs(0.0, y, out_hi) == 0
    g = c.grid
    inner = np.ones(c.nC, bool)
    inner[g.iEP[g.nPi:g.nPi + g.nPb, 0] - 1] = False  # cells with a boundary face
    assert inner.sum() > c.nC // 2
    a, b = out_hi.reshape(5, -1), out32.reshape(5, -1)
    assert np.array_equal(a[:, inner], b[:, inner])


def test_hybrid_flux_bump_converges_and_matches_oracle(cuda):
    """Four BDF1 steps at CFL ~5 on the 48 x 16 x 8 x 6 = 36,864-tet channel (where the plain
    FP32 flux stalls at about twice the Newton tolerance): every Newton iteration converges to
    1e-8 with the hybrid flux, and the state lies within 1e-6 of the FP64 oracle's per
    conserved field."""
    wl = M.make_workload("bump192", scale=48)
    c = Case(wl, flags=HYB)
    assert c.nC == 36864
    nsteps = 4
    rc, st, y = _gpu_steps(c, nsteps)
    assert rc == 0, st
    assert st["n_steps"] == nsteps
    c.match_ilu_order()
    rhs, pset, psol = c.oracle.callbacks()
    y_ref = c.y0.copy()
    rc_o, st_o = O.bdf_run(c.N, rhs, pset, psol, c.oracle.h, y_ref,
                           O.bdf_defaults(order=wl.order, dt=wl.dt, nsteps=nsteps))
    assert rc_o == 0
    fe = field_errors(y, y_ref)
    print("hybrid bump", fe, cell_errors(y, y_ref), st, st_o)
    assert max(fe["rho"], fe["rhou"], fe["rhoE"]) <= 1e-6
