"""A foeuler case directory end to end on the GPU: Gmsh mesh, condition table, initial
condition, run control and gas files in; fixed BDF2 steps with GMRES(30) + ILU(0) in FP64;
rst_<k>.vtk files out.  The final state must match the oracle's BDF run of the same case
within 1e-10 (per conserved variable, relative to its largest value), and the written files
must carry that state."""
import numpy as np
import pytest

from fosolvers_gb300 import mesh as M
from fosolvers_gb300.case import primitives, run_case, workload_from_case
from fosolvers_gb300.meshio import read_vtk
from helpers import Case, rel_err
from oracle import pyoracle as O
from test_meshio import _write_case

pytestmark = pytest.mark.gpu


def test_case_directory_matches_oracle_and_writes_results(cuda, tmp_path):
    m = M.box_mesh(10, 6, 6, jitter=0.1, seed=4, extent=(1.0, 0.6, 0.6))
    dt = 2e-5  # CFL ~ 0.07 on 347 m/s at h = 0.1
    # subsonic duct-like set-up in SI units: total-pressure inflow at x-min, static-pressure
    # outflow at x-max, walls elsewhere
    _write_case(tmp_path, m, [(M.GID_XMIN, 11, [1.05e5, 300.0, 1.0, 0.0, 0.0]),
                              (M.GID_XMAX, 20, [0.95e5])],
                ic=(1.0e5, 300.0, 0.0, 0.0, 0.0), sim=(6 * dt, 3 * dt))
    out = tmp_path / "out"
    res = run_case(tmp_path, out, dt=dt, order=2, log=lambda s: None)
    assert res["steps"] == 6 and res["outputs"] == 2

    wl = workload_from_case(tmp_path, dt=dt, order=2, nsteps=6)
    c = Case(wl)
    c.match_ilu_order()
    rhs, pset, psol = c.oracle.callbacks()
    y_ref = c.y0.copy()
    rc, st = O.bdf_run(c.N, rhs, pset, psol, c.oracle.h, y_ref,
                       O.bdf_defaults(order=2, dt=dt, nsteps=6, use_prec=1))
    assert rc == 0, st
    err = rel_err(res["y"], y_ref)
    print("case parity", err)
    assert err <= 1e-10
    # the flow moved: inflow total pressure above the initial static pressure
    assert np.abs(res["y"][c.nC:2 * c.nC]).max() > 0.0

    nC = c.nC
    for k in range(3):
        assert (out / f"rst_{k}.vtk").exists()
    mesh_out, data = read_vtk(out / "rst_2.vtk")
    assert mesh_out.nE == wl.mesh.nE
    rho, u, p, T = primitives(res["y"], nC, wl.r, wl.gamm)
    np.testing.assert_array_equal(data["cell"]["density"][:nC], rho)
    np.testing.assert_array_equal(data["cell"]["velocity"][:nC], u)
    np.testing.assert_array_equal(data["cell"]["pressure"][:nC], p)
    np.testing.assert_array_equal(data["cell"]["temperature"][:nC], T)


def test_adaptive_case_matches_oracle(cuda, tmp_path):
    """The same case with the variable-order, variable-step driver at RTOL 1e-6, ATOL 1e-6
    (SI state magnitudes ~1 to 1e5) from output time to output time: identical accepted-step
    count to the oracle's restatement over each interval, final state within 1e-9."""
    m = M.box_mesh(8, 5, 5, jitter=0.1, seed=7, extent=(1.0, 0.6, 0.6))
    t1 = 4e-4
    _write_case(tmp_path, m, [(M.GID_XMIN, 11, [1.05e5, 300.0, 1.0, 0.0, 0.0]),
                              (M.GID_XMAX, 20, [0.95e5])],
                ic=(1.0e5, 300.0, 0.0, 0.0, 0.0), sim=(t1, t1 / 2))
    res = run_case(tmp_path, tmp_path / "out", dt=1e-6, adaptive=True, rtol=1e-6, atol=1e-6,
                   newton_rtol=1e-10, log=lambda s: None)
    assert res["outputs"] == 2 and abs(res["t"] - t1) <= 1e-15

    wl = workload_from_case(tmp_path, dt=1e-6)
    c = Case(wl)
    c.match_ilu_order()
    rhs, pset, psol = c.oracle.callbacks()
    y_ref = c.y0.copy()
    n_acc, h = 0, 1e-6
    for (ta, tb) in ((0.0, t1 / 2), (t1 / 2, t1)):
        rc, st, ast = O.bdf_adaptive(c.N, rhs, pset, psol, c.oracle.h, y_ref, ta, tb,
                                     O.bdf_defaults(newton_rtol=1e-10),
                                     O.adapt_defaults(rtol=1e-6, atol=1e-6, h0=min(h, tb - ta)))
        assert rc == 0, ast
        n_acc += ast["n_accepted"]
        h = ast["h_last"]
    print("adaptive case", res["steps"], n_acc, rel_err(res["y"], y_ref))
    assert res["steps"] == n_acc
    assert rel_err(res["y"], y_ref) <= 1e-9


def _duct_case(tmp_path, t_final, t_int):
    """The reference's examples/foeuler/duct case directory (mesh, bc, ic and fl as the
    reference ships them, from tests/golden/duct.npz) with the run control shortened."""
    from test_meshio import write_duct_case
    case = write_duct_case(tmp_path / "duct")
    (case / "sim").write_text(f"{float(t_final)!r}  # final time [s]\n{float(t_int)!r}  # output interval [s]\n")
    return case


def test_duct_example_fixed_steps_match_oracle(cuda, tmp_path):
    """examples/foeuler/duct (65,483 tetrahedra; total-pressure inflow, code 11, on group 5;
    static-pressure outflow, code 20, on group 3; walls elsewhere; SI units, R = 287.058):
    six BDF2 steps at CFL 5 on the initial state with GMRES(30) + ILU(0) in FP64, written as
    rst_<k>.vtk every three steps; the state must match the oracle's within 1e-10 and the
    files must carry it."""
    from fosolvers_gb300.case import load_case
    ci = load_case(_duct_case(tmp_path, 1.0, 1.0))
    c_snd = np.sqrt(ci.gamm * ci.r * ci.ic["T0"])
    from fosolvers_gb300.euler import PolyFvGrid
    dt = 5.0 * float(np.cbrt(PolyFvGrid.from_mesh(ci.mesh).v).min()) / c_snd
    case = _duct_case(tmp_path, 6 * dt, 3 * dt)
    out = tmp_path / "out"
    res = run_case(case, out, dt=dt, order=2, log=lambda s: None)
    assert res["steps"] == 6 and res["outputs"] == 2 and res["cells"] == 65483

    wl = workload_from_case(case, dt=dt, order=2, nsteps=6)
    c = Case(wl)
    c.match_ilu_order()
    rhs, pset, psol = c.oracle.callbacks()
    y_ref = c.y0.copy()
    rc, st = O.bdf_run(c.N, rhs, pset, psol, c.oracle.h, y_ref,
                       O.bdf_defaults(order=2, dt=dt, nsteps=6, use_prec=1))
    assert rc == 0, st
    err = rel_err(res["y"], y_ref)
    print("duct parity", dt, err, res["stats"], st)
    assert err <= 1e-10
    nC = c.nC
    # the inflow drives the gas: momentum appears and the pressure leaves its initial value
    rho, u, p, T = primitives(res["y"], nC, wl.r, wl.gamm)
    assert np.abs(u).max() > 1e-3 and p.max() > 0.9e5
    for k in range(3):
        assert (out / f"rst_{k}.vtk").exists()
    mesh_out, data = read_vtk(out / "rst_2.vtk")
    assert mesh_out.nE == wl.mesh.nE
    np.testing.assert_array_equal(data["cell"]["density"][:nC], rho)
    np.testing.assert_array_equal(data["cell"]["velocity"][:nC], u)
    np.testing.assert_array_equal(data["cell"]["pressure"][:nC], p)
    np.testing.assert_array_equal(data["cell"]["temperature"][:nC], T)

