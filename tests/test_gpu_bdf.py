"""End-to-end parity of the implicit inner loop: fixed-step BDF Newton--GMRES(30) with
block ILU(0), GPU against the oracle on the same mesh and initial state.

The plain FP64 GPU path must reproduce the oracle's per-cell conserved variables within
1e-10 (relative to the largest value of each conserved variable) after the workload's
steps; the FP32 flux + FP32 ILU form within 1e-6."""
import numpy as np
import pytest

from fosolvers_gb300 import mesh as M
from fosolvers_gb300.euler import FLUX_FP32, ILU_COLOR, ILU_FP32
from helpers import Case, field_errors, hex_workload, perturbed, rel_err, with_all_conditions
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu


def oracle_run(c: Case, nsteps=None, use_prec=1, **kw):
    wl = c.wl
    opts = O.bdf_defaults(order=wl.order, dt=wl.dt, nsteps=nsteps or wl.nsteps, use_prec=use_prec,
                          **kw)
    y = c.y0.copy()
    c.match_ilu_order()
    rhs, pset, psol = c.oracle.callbacks()
    rc, st = O.bdf_run(c.N, rhs, pset, psol, c.oracle.h, y, opts)
    assert rc == 0, st
    return y, st


def gpu_run(c: Case, nsteps=None, precond=1, **kw):
    import torch
    wl = c.wl
    yr = torch.from_numpy(c.y0).cuda()
    y = torch.empty_like(yr)
    c.gpu.to_internal(yr, y)
    opts = c.gpu.bdf_defaults(order=wl.order, dt=wl.dt, nsteps=nsteps or wl.nsteps, precond=precond,
                              **kw)
    rc, st = c.gpu.bdf_run(y, opts)
    assert rc == 0, st
    c.gpu.to_reference(y, yr)
    torch.cuda.synchronize()
    return yr.cpu().numpy(), st


def test_sod16_twenty_steps_matches_oracle(cuda):
    """16^3 x 6 tets, Sod, walls, BDF1 dt = 1e-3, 20 steps, GMRES(30) + ILU(0), 1e-8."""
    c = Case(M.make_workload("sod16"))
    y_ref, st_ref = oracle_run(c)
    y, st = gpu_run(c)
    err = rel_err(y, y_ref)
    print("sod16 parity", err, st, st_ref)
    assert st["n_steps"] == 20
    assert st["n_newton"] == st_ref["n_newton"]
    assert err <= 1e-10


@pytest.mark.parametrize("flags", [0, ILU_COLOR])
def test_sine_bdf2_matches_oracle(cuda, flags):
    c = Case(M.make_workload("sine96", scale=10, seed=2), flags=flags)
    y_ref, st_ref = oracle_run(c, nsteps=5)
    y, st = gpu_run(c, nsteps=5)
    assert rel_err(y, y_ref) <= 1e-10


@pytest.mark.parametrize("name,scale,nsteps,rtol", [("sine96", 16, 8, 1e-8), ("bump192", 24, 4, 1e-11)])
def test_predictor_matches_oracle(cuda, name, scale, nsteps, rtol):
    """CVODE's constant-step BDF predictor (fos_bdf_opts.predictor = 1): Newton starts from
    the extrapolation through the last q + 1 accepted states.  On the smooth sine state it
    saves Newton iterations; on the Mach 2 bump's start-up transient the extrapolation can
    fail, and the step is retried from y_n.  Both drivers take the same path: the state
    within 1e-10 of the oracle's, with the same Newton and Krylov counts on the smooth state
    (on the bump, about 22 Krylov iterations per Newton solve let the Jv rounding move a
    count by one, as in test_bump_cfl5_matches_oracle, so the Newton count is compared)."""
    c = Case(M.make_workload(name, scale=scale))
    y_ref, st_ref = oracle_run(c, nsteps=nsteps, newton_rtol=rtol, predictor=1)
    y, st = gpu_run(c, nsteps=nsteps, newton_rtol=rtol, predictor=1)
    print("predictor", name, st, st_ref)
    assert st["n_newton"] == st_ref["n_newton"]
    assert rel_err(y, y_ref) <= 1e-10
    if name == "sine96":
        assert st["n_lin_iters"] == st_ref["n_lin_iters"]
        _, st0 = oracle_run(c, nsteps=nsteps, newton_rtol=rtol, predictor=0)
        assert st_ref["n_newton"] < st0["n_newton"]


def test_bump_cfl5_matches_oracle(cuda):
    """Supersonic bump at CFL ~5 (static inflow, extrapolated outflow, walls).  With ~40
    Krylov iterations per Newton solve the finite-difference Jv rounding (~1e-8 relative)
    separates the two iterations within the Newton tolerance ball, so parity is checked at a
    Newton tolerance tightened to 1e-11 (both runs converge onto the same discrete solution)."""
    c = Case(M.make_workload("bump192", scale=24))
    y_ref, _ = oracle_run(c, nsteps=4, newton_rtol=1e-11)
    y, st = gpu_run(c, nsteps=4, newton_rtol=1e-11)
    assert rel_err(y, y_ref) <= 1e-10


@pytest.mark.parametrize("name,scale,precond,maxl", [("bump192", 24, 1, 5), ("sod16", 8, 0, 2)])
def test_restarted_gmres_matches_oracle(cuda, name, scale, precond, maxl):
    """GMRES(maxl) short enough that every solve restarts (the bump with ILU(0): about 35
    Krylov iterations per Newton solve; Sod unpreconditioned: 3): the first cycle's unscaled
    first vector, the correction kept for the restart residual, and the true-residual
    restart, against the oracle at a Newton tolerance of 1e-11."""
    c = Case(M.make_workload(name, scale=scale))
    kw = dict(nsteps=2, newton_rtol=1e-11, maxl=maxl, max_restarts=40)
    y_ref, st_ref = oracle_run(c, use_prec=precond, **kw)
    y, st = gpu_run(c, precond=precond, **kw)
    print("restarted", name, precond, maxl, st, st_ref)
    assert st["n_lin_iters"] > maxl * st["n_newton"]  # solves restarted
    assert st["n_jv"] > st["n_lin_iters"]  # restart residuals
    assert rel_err(y, y_ref) <= 1e-10


@pytest.mark.parametrize("pinned", [False, True])
def test_host_buffer_entry_points_match_device(cuda, pinned):
    """The host-buffer entry points on a pageable and on a page-locked array, copied plane
    by plane on the copy stream with the permutations overlapped: fos_bdf_run_host equals
    fos_bdf_run on the device bit for bit, and the rhs callback equals the one on a
    pageable copy."""
    import torch
    c = Case(M.make_workload("sine96", scale=8, seed=1), flags=FLUX_FP32 | ILU_FP32 | ILU_COLOR)
    y_dev, _ = gpu_run(c, nsteps=3)
    keep = []  # the tensors that own the host buffers

    def host(a):
        t = torch.from_numpy(a.copy())
        keep.append(t.pin_memory() if pinned else t)
        return keep[-1].numpy()

    yh = host(c.y0)
    opts = c.gpu.bdf_defaults(order=c.wl.order, dt=c.wl.dt, nsteps=3, precond=1)
    rc, st = c.gpu.bdf_run_host(yh, opts)
    assert rc == 0, st
    assert np.array_equal(yh, y_dev)
    y1 = perturbed(c.y0, c.nC, 5)
    f_ref = np.zeros_like(y1)
    assert c.gpu.rhs(0.0, y1.copy(), f_ref) == 0
    yin, fout = host(y1), host(np.zeros_like(y1))
    assert c.gpu.rhs(0.0, yin, fout) == 0
    assert np.array_equal(fout, f_ref)


def test_unpreconditioned_matches_oracle(cuda):
    c = Case(M.make_workload("sod16", scale=8))
    y_ref, _ = oracle_run(c, nsteps=5, use_prec=0)
    y, _ = gpu_run(c, nsteps=5, precond=0)
    assert rel_err(y, y_ref) <= 1e-10


def test_dropin_callbacks_under_reference_driver(cuda):
    """The oracle's BDF driver (standing in for CVODE) driving the GPU host callbacks
    fos_euler_rhs / pset / psol gives the oracle's own answer."""
    import ctypes as C
    from fosolvers_gb300 import _lib
    c = Case(M.make_workload("sod16", scale=8))
    y_ref, st_ref = oracle_run(c, nsteps=5)
    L = _lib.lib()
    y = c.y0.copy()
    opts = O.bdf_defaults(order=1, dt=1e-3, nsteps=5)
    rc, st = O.bdf_run(c.N, C.cast(L.fos_euler_rhs, C.c_void_p), C.cast(L.fos_euler_pset, C.c_void_p),
                       C.cast(L.fos_euler_psol, C.c_void_p), c.gpu.handle, y, opts)
    assert rc == 0
    assert rel_err(y, y_ref) <= 1e-10


@pytest.mark.parametrize("extra", [0, ILU_COLOR])
def test_fp32_form_within_1e6(cuda, extra):
    """FP32 Roe flux + FP32 ILU(0) factors/apply, FP64 Newton/orthogonalisation: state within
    1e-6 of the FP64 oracle after the Sod workload's 20 steps, per conserved field (density,
    momentum vector, energy), relative to the field's largest magnitude."""
    c = Case(M.make_workload("sod16"), flags=FLUX_FP32 | ILU_FP32 | extra)
    y_ref, _ = oracle_run(c)
    y, st = gpu_run(c)
    err = field_errors(y, y_ref)
    print("fp32 form sod16", err, st)
    assert max(err["rho"], err["rhou"], err["rhoE"]) <= 1e-6


def _bdf_case(name):
    if name == "hex10":
        return hex_workload(10, seed=2)
    if name == "conds6":
        wl = with_all_conditions(M.make_workload("sod16", scale=6))
    else:
        wl = with_all_conditions(hex_workload(8, seed=3))
    wl.order, wl.dt, wl.nsteps = 2, 2e-3, 6
    return wl


@pytest.mark.parametrize("name", ["hex10", "conds6", "conds-hex8"])
def test_cells_and_conditions_bdf2_match_oracle(cuda, name):
    """Hexahedral cells (six-face ELL rows, 7-block ILU rows, warped faces) and every
    condition type: FP64 within 1e-10 of the oracle's BDF run, and the FP32 flux +
    colour-ordered FP32 ILU(0) form within 1e-6 per conserved field."""
    c = Case(_bdf_case(name))
    y_ref, st_ref = oracle_run(c)
    y, st = gpu_run(c)
    print(name, "fp64", rel_err(y, y_ref), st, st_ref)
    assert rel_err(y, y_ref) <= 1e-10
    c32 = Case(_bdf_case(name), flags=FLUX_FP32 | ILU_FP32 | ILU_COLOR)
    y32, st32 = gpu_run(c32)
    err = field_errors(y32, y_ref)
    print(name, "fp32 form", err, st32)
    assert max(err["rho"], err["rhou"], err["rhoE"]) <= 1e-6


def test_learned_preconditioner_refuses_hex_grid(cuda):
    """The network reads four neighbour slots per cell: attaching it to a grid with
    hexahedra is an error at attach time, not a failure inside a run."""
    from fosolvers_gb300.learned import GNN
    c = Case(hex_workload(6))
    with pytest.raises(RuntimeError, match="tetrahedral grids only"):
        c.gpu.attach_gnn(GNN(seed=0))


@pytest.mark.parametrize("msbp", [5, 20])
def test_cvode_setup_policy_matches_oracle(cuda, msbp):
    """CVODE's preconditioner set-up policy (msbp > 1: at most msbp steps between psets, a
    fresh one on a > 30% gamma change or a Newton failure on a reused one) in both drivers:
    BDF2 on the sine workload at 8^3 x 6 for 12 steps, the same pset, Newton and Krylov
    counts, state within 1e-10."""
    wl = M.make_workload("sine96", scale=8, seed=1)
    c = Case(wl)
    y_ref, st_ref = oracle_run(c, nsteps=12, msbp=msbp)
    y, st = gpu_run(c, nsteps=12, msbp=msbp)
    print("msbp", msbp, st, st_ref)
    for k in ("n_pset", "n_newton", "n_lin_iters", "n_steps"):
        assert st[k] == st_ref[k], k
    assert st["n_pset"] < 12
    assert rel_err(y, y_ref) <= 1e-10


def test_resumed_calls_keep_the_setup_policy(cuda):
    """Twelve one-step calls with resume = 1 under CVODE's set-up policy (MSBP 5) make the
    same psets and reach the same state, bit for bit, as one twelve-step call: the set-up
    count carries across calls as CVODE's does across CVode calls.  A pset made outside the
    driver in between voids the kept set-up (the next step sets up again)."""
    import torch
    wl = M.make_workload("sine96", scale=8, seed=1)
    c = Case(wl)
    y_one, st_one = gpu_run(c, nsteps=12, msbp=5)
    yr = torch.from_numpy(c.y0).cuda()
    y = torch.empty_like(yr)
    c.gpu.to_internal(yr, y)
    n_pset = 0
    for k in range(12):
        rc, st = c.gpu.bdf_run(y, c.gpu.bdf_defaults(order=wl.order, dt=wl.dt, nsteps=1,
                                                     precond=1, msbp=5, resume=1 if k else 0),
                               t0=k * wl.dt)
        assert rc == 0
        n_pset += st["n_pset"]
    assert n_pset == st_one["n_pset"] < 12
    c.gpu.to_reference(y, yr)
    torch.cuda.synchronize()
    assert np.array_equal(yr.cpu().numpy(), y_one)
    # an outside pset between two resumed calls: the next call sets up afresh
    c.gpu.pset_dev(0.0, y, 0, 2.0 * wl.dt / 3.0)
    rc, st = c.gpu.bdf_run(y, c.gpu.bdf_defaults(order=wl.order, dt=wl.dt, nsteps=1, precond=1,
                                                 msbp=5, resume=1), t0=12 * wl.dt)
    assert rc == 0 and st["n_pset"] == 1
