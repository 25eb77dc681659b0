"""GPU residual and Jacobian-vector product against the oracle (same mesh, same state).

Tolerances: FP64 residual within 1e-11 of the oracle (relative to the largest entry of
each conserved block; the GPU sums faces in another order, forms sqrt(rho_m rho_n) as
sqrt(rho_m) sqrt(rho_n) and multiplies by 1/v); FD Jv within 1e-6 (the difference
quotient divides rounding noise by s ~ 1e-8); FP32 flux within 2e-5 of the FP64 oracle."""
import numpy as np
import pytest

from fosolvers_gb300 import mesh as M
from fosolvers_gb300.euler import FLUX_FP32
from helpers import Case, hex_workload, perturbed, rel_err, with_all_conditions

pytestmark = pytest.mark.gpu


def _cases():
    return {
        "sod16": lambda: M.make_workload("sod16"),
        "sine12": lambda: M.make_workload("sine96", scale=12, seed=3),
        "bump24": lambda: M.make_workload("bump192", scale=24),
        "hex10": lambda: hex_workload(10, seed=2),
    }


@pytest.fixture(scope="module")
def cases(cuda):
    return {k: Case(f()) for k, f in _cases().items()}


@pytest.mark.parametrize("name", ["sod16", "sine12", "bump24", "hex10"])
@pytest.mark.parametrize("seed", [None, 11])
def test_rhs_host_callback_matches_oracle(cases, name, seed):
    c = cases[name]
    y = c.y0 if seed is None else perturbed(c.y0, c.nC, seed)
    ref = c.oracle_rhs(y)
    out = np.zeros_like(y)
    assert c.gpu.rhs(0.0, y, out) == 0
    assert rel_err(out, ref) <= 1e-11


@pytest.mark.parametrize("name", ["tet6", "hex8"])
def test_rhs_all_condition_types(cuda, name):
    """Every non-UDF condition of setBC (foeuler.f90:217-325) on one box: static inflow
    (subsonic: interior momentum), total inflow, outflow (imposed p), far field,
    zero-gradient outflow, wall; tetrahedra and hexahedra (QUAD boundary faces), FP64 flux
    within 1e-11 and FP32 flux within 2e-5."""
    wl = with_all_conditions(M.make_workload("sod16", scale=6) if name == "tet6"
                             else hex_workload(8, seed=5))
    for flags, tol in ((0, 1e-11), (FLUX_FP32, 2e-5)):
        c = Case(wl, flags=flags)
        for seed in (None, 4):
            y = c.y0 if seed is None else perturbed(c.y0, c.nC, seed, amp=0.1)
            ref = c.oracle_rhs(y)
            out = np.zeros_like(y)
            assert c.gpu.rhs(0.0, y, out) == 0
            err = rel_err(out, ref)
            print(name, flags, seed, err)
            assert err <= tol


def test_rhs_bar_tet_unstructured(cuda):
    """The reference's own unstructured mesh (bar_tet, Gmsh), Sod state along x, walls."""
    from test_grid import bar_tet_mesh
    mesh = bar_tet_mesh()
    from fosolvers_gb300.euler import PolyFvGrid
    g = PolyFvGrid.from_mesh(mesh)
    st = M.sod_state(g.p)
    wl = M.Workload("bar", mesh, st, np.zeros(0, np.int32), np.zeros(0, np.int32),
                    np.zeros((0, 5)), 1, 1e-3, 1)
    c = Case(wl)
    # the workload state is in sorted element order already (cells first)
    y = perturbed(M.soa(st, c.nC), c.nC, 9)
    ref = c.oracle_rhs(y)
    out = np.zeros_like(y)
    assert c.gpu.rhs(0.0, y, out) == 0
    assert rel_err(out, ref) <= 1e-11


@pytest.mark.parametrize("name", ["sine12", "hex10"])
def test_rhs_device_entry_and_renumbering(cases, name):
    import torch
    c = cases[name]
    y = perturbed(c.y0, c.nC, 2)
    ref = c.oracle_rhs(y)
    yr = torch.from_numpy(y).cuda()
    yi, f, fr = torch.empty_like(yr), torch.empty_like(yr), torch.empty_like(yr)
    c.gpu.to_internal(yr, yi)
    c.gpu.rhs_dev(0.0, yi, f)
    c.gpu.to_reference(f, fr)
    torch.cuda.synchronize()
    assert rel_err(fr.cpu().numpy(), ref) <= 1e-11
    o2n = c.gpu.renumbering()
    assert np.array_equal(np.sort(o2n), np.arange(c.nC))
    assert c.gpu.info()["bandwidth"] < c.nC


@pytest.mark.parametrize("name", ["sine12", "hex10"])
def test_jv_matches_oracle_difference_quotient(cases, name):
    """Fused FD Jv: out = a v + b (f(y + s v) - f(y))/s, s = eps (1 + ||y||)/||v||."""
    import torch
    c = cases[name]
    rng = np.random.default_rng(0)
    y = perturbed(c.y0, c.nC, 5)
    v = rng.normal(size=y.size)
    eps = np.sqrt(np.finfo(float).eps)
    s = eps * (1 + np.linalg.norm(y)) / np.linalg.norm(v)
    fy = c.oracle_rhs(y)
    ref = (c.oracle_rhs(y + s * v) - fy) / s
    gamma = 2e-3
    dev = lambda a: torch.from_numpy(a).cuda()
    yi, fi, vi, out, tmp = (torch.empty(y.size, dtype=torch.float64, device="cuda") for _ in range(5))
    c.gpu.to_internal(dev(y), yi)
    c.gpu.rhs_dev(0.0, yi, fi)
    c.gpu.to_internal(dev(v), vi)
    c.gpu.jv_dev(0.0, yi, fi, vi, out, 1.0, -gamma, float(np.linalg.norm(y)), eps)
    c.gpu.to_reference(out, tmp)
    got = tmp.cpu().numpy()
    assert rel_err(got, v - gamma * ref) <= 1e-6
    c.gpu.jv_dev(0.0, yi, fi, vi, out, 0.0, 1.0, float(np.linalg.norm(y)), eps)
    c.gpu.to_reference(out, tmp)
    assert rel_err(tmp.cpu().numpy(), ref) <= 1e-6


def test_nonfinite_state_is_recoverable(cases):
    c = cases["sod16"]
    y = c.y0.copy()
    y[5] = np.nan
    out = np.zeros_like(y)
    assert c.gpu.rhs(0.0, y, out) == 1  # CVODE convention: > 0 = recoverable


@pytest.mark.parametrize("name", ["sod16", "sine12", "bump24", "hex10"])
def test_fp32_flux_against_fp64_oracle(name):
    wl = _cases()[name]()
    c = Case(wl, flags=FLUX_FP32)
    y = perturbed(c.y0, c.nC, 21)
    ref = c.oracle_rhs(y)
    out = np.zeros_like(y)
    assert c.gpu.rhs(0.0, y, out) == 0
    err = rel_err(out, ref)
    print(f"fp32 flux {name}: rel err {err:.3e}")
    assert err <= 2e-5
