"""A foeuler case directory on the GPU: ``grid.msh``, ``bc``, ``ic``, ``sim`` and ``fl`` in,
``rst_<k>.vtk`` out -- the inputs and outputs of foeuler's ``init`` / ``writeState`` /
main program (src/foeuler/foeuler.f90:58-180, 332-345, 443-468), with the residual, the
Jacobian, the preconditioner and the BDF Newton--Krylov steps of libfosgpu.

Input files (the reference's list-directed reads, one value per line, text after the value
ignored):

* ``bc``  -- readCondTab (libfosolvers/fileIO/condTab.f90:4-21): number of conditions,
  maximum parameters; then per condition a separator line, the geometric group id, the
  condition type (foeuler.f90 BC_* codes) and the number of real parameters followed by
  one parameter per line;
* ``ic``  -- UDF switch (0: constant state), pressure, temperature, velocity x, y, z
  (foeuler.f90:82-100); the libmatheval UDF form is rejected, as the condition table's UDF
  types are at context creation;
* ``sim`` -- final time and output interval (foeuler.f90:102-105);
* ``fl``  -- specific gas constant and gamma (foeuler.f90:106-109).

The initial state is the reference's: rho = p0 / (r T0), rho u = rho u0,
rho E = rho (r T0 / (gamma - 1) + |u0|^2 / 2) (foeuler.f90:123-138).  Condition rows
are matched to elements by group id, first match wins (foeuler.f90:145-154).

Time stepping: the reference hands the step size to CVODE (adaptive order and step,
RTOL 1e-6, ATOL 1e-12).  Here either the device driver's variable-order, variable-step BDF
at those tolerances runs from output time to output time (``adaptive``), or fixed-size
BDF1/BDF2 steps with dt given or derived from a CFL number on the initial state; an output
file is written at every multiple of the output interval.

Output: ``rst_<k>.vtk`` with the grid (elements in the grid's order: cells, then facets)
and per-element density, velocity, pressure and temperature (foeuler.f90:332-345).  The
reference writes the boundary facets' ghost states; here a facet carries the state of the
cell behind it.
"""
from __future__ import annotations

import argparse
import math
import time
from dataclasses import dataclass
from pathlib import Path

import numpy as np

from .meshio import CELL_SHAPES, read_gmsh, write_vtk

FACET_SHAPES = (10, 11, 110)


def _values(path):
    """Lines of a list-directed input file: the first token of each line (None if blank)."""
    out = []
    for line in Path(path).read_text().splitlines():
        t = line.split()
        out.append(t[0] if t else None)
    return out


def _num(tok, what):
    if tok is None:
        raise ValueError(f"missing value: {what}")
    return float(tok.replace("d", "e").replace("D", "e"))


@dataclass
class CondTab:
    gid: np.ndarray     # (n,) geometric group ids
    type: np.ndarray    # (n,) condition codes
    param: np.ndarray   # (n, m) real parameters (row = condition)


def read_cond_tab(path) -> CondTab:
    v = _values(path)
    n, m = int(_num(v[0], "number of conditions")), int(_num(v[1], "maximum parameters"))
    gid, typ, par = np.zeros(n, np.int32), np.zeros(n, np.int32), np.zeros((n, max(m, 1)))
    i = 2
    for c in range(n):
        i += 1  # the separator line each condition starts with
        gid[c] = int(_num(v[i], "group id")); i += 1
        typ[c] = int(_num(v[i], "condition type")); i += 1
        k = int(_num(v[i], "number of parameters")); i += 1
        if k > m:
            raise ValueError(f"condition {c + 1} has {k} parameters, more than the maximum {m}")
        for j in range(k):
            par[c, j] = _num(v[i], "parameter"); i += 1
    return CondTab(gid, typ, par)


def read_ic(path) -> dict:
    v = [t for t in _values(path) if t is not None]
    if int(_num(v[0], "UDF switch")) != 0:
        raise NotImplementedError("initial conditions from user-defined functions (libmatheval) "
                                  "are not supported")
    return {"p0": _num(v[1], "p0"), "T0": _num(v[2], "T0"),
            "u0": np.array([_num(v[3], "u"), _num(v[4], "v"), _num(v[5], "w")])}


def read_sim(path):
    v = [t for t in _values(path) if t is not None]
    return _num(v[0], "final time"), _num(v[1], "output interval")


def read_fl(path):
    v = [t for t in _values(path) if t is not None]
    return _num(v[0], "gas constant"), _num(v[1], "gamma")


def grid_order(mesh) -> np.ndarray:
    """Mesh element index of each grid element: cells, then facets, then the rest, each in
    file order (the stable partition fos_grid_build applies)."""
    s = mesh.sE
    cells = np.flatnonzero(np.isin(s, CELL_SHAPES))
    facets = np.flatnonzero(np.isin(s, FACET_SHAPES))
    rest = np.flatnonzero(~np.isin(s, CELL_SHAPES + FACET_SHAPES))
    return np.concatenate([cells, facets, rest])


def sorted_mesh(mesh):
    """The mesh with its elements in grid order (cells, facets, rest), so element arrays
    (group ids, condition rows, element states) line up with the face arrays."""
    from .mesh import Mesh
    o = grid_order(mesh)
    return Mesh(pN=mesh.pN, sE=mesh.sE[o], nNE=mesh.nNE[o], iNE=mesh.iNE[o], gid=mesh.gid[o],
                nC=int(np.isin(mesh.sE, CELL_SHAPES).sum()), meta=dict(mesh.meta))


@dataclass
class CaseInput:
    mesh: object        # Mesh, elements in grid order
    bc: CondTab
    ic: dict
    t_final: float
    t_int: float
    r: float
    gamm: float


def load_case(case_dir) -> CaseInput:
    case = Path(case_dir)
    t_final, t_int = read_sim(case / "sim")
    r, gamm = read_fl(case / "fl")
    return CaseInput(sorted_mesh(read_gmsh(case / "grid.msh")), read_cond_tab(case / "bc"),
                     read_ic(case / "ic"), t_final, t_int, r, gamm)


def workload_from_case(case_dir, dt: float, order: int = 2, nsteps: int = 1):
    """The case as a Workload (uniform initial state on every element)."""
    from .mesh import Workload
    ci = load_case(case_dir)
    y = initial_state(ci.mesh.nE, ci.ic, ci.r, ci.gamm).reshape(5, -1)
    return Workload(name=str(case_dir), mesh=ci.mesh, elem_state=tuple(y), bc_gid=ci.bc.gid,
                    bc_type=ci.bc.type, bc_param=ci.bc.param, order=order, dt=dt, nsteps=nsteps,
                    gamm=ci.gamm, r=ci.r)


def initial_state(nC: int, ic: dict, r: float, gamm: float) -> np.ndarray:
    rho = ic["p0"] / r / ic["T0"]
    u0 = ic["u0"]
    E = rho * (1.0 / (gamm - 1.0) * r * ic["T0"] + 0.5 * float(u0 @ u0))
    return np.concatenate([np.full(nC, rho), np.full(nC, rho * u0[0]), np.full(nC, rho * u0[1]),
                           np.full(nC, rho * u0[2]), np.full(nC, E)])


def primitives(y: np.ndarray, nC: int, r: float, gamm: float):
    """density, velocity (nC, 3), pressure, temperature of an SoA state (syncState)."""
    q = y.reshape(5, nC)
    rho = q[0]
    u = (q[1:4] / rho).T
    p = (gamm - 1.0) * (q[4] - 0.5 * rho * (u * u).sum(1))
    return rho, u, p, p / (rho * r)


def write_state(path, mesh, grid, y, r, gamm):
    """rst file: the grid (elements in grid order), per-element density, velocity,
    pressure, temperature; facets carry the state of the cell behind them."""
    nC, nE = grid.nC, grid.nE
    rho, u, p, T = primitives(y, nC, r, gamm)
    owner = np.zeros(nE, np.int64)  # cell whose state an element shows
    owner[:nC] = np.arange(nC)
    b = grid.iEP[grid.nPi:grid.nPi + grid.nPb]
    owner[b[:, 1] - 1] = b[:, 0] - 1
    write_vtk(path, mesh, cell_data={"density": rho[owner], "velocity": u[owner],
                                     "pressure": p[owner], "temperature": T[owner]})


def run_case(case_dir, out_dir=None, dt=None, cfl=5.0, order=2, flags=0, precond=1,
             newton_rtol=1e-8, max_steps=None, write=True, log=print, adaptive=False,
             rtol=1e-6, atol=1e-12) -> dict:
    """Run a foeuler case directory to its final time on the GPU, with fixed BDF steps of
    size dt, or (adaptive) with the variable-order, variable-step driver at the local error
    tolerances foeuler gives CVODE (RTOL 1e-6, ATOL 1e-12; dt is then the first step).
    Returns the final SoA state (reference cell order) and run statistics."""
    import torch
    from .euler import FOEuler, PolyFvGrid
    case = Path(case_dir)
    out = Path(out_dir) if out_dir else case
    out.mkdir(parents=True, exist_ok=True)
    t0 = time.perf_counter()
    ci = load_case(case)
    mesh, bc, ic, r, gamm = ci.mesh, ci.bc, ci.ic, ci.r, ci.gamm
    t_final, t_int = ci.t_final, ci.t_int
    grid = PolyFvGrid.from_mesh(mesh)
    ibc = np.zeros(grid.nE, np.int32)
    for row, g in enumerate(bc.gid):
        ibc[(grid.gid == g) & (ibc == 0)] = row + 1
    ctx = FOEuler(grid, ibc, bc.type, bc.param, gamm, r, flags=flags)
    y = initial_state(grid.nC, ic, r, gamm)
    if dt is None:  # CFL on the initial state with h = V^(1/3)
        c = math.sqrt(gamm * r * ic["T0"]) + float(np.linalg.norm(ic["u0"]))
        dt = cfl * float(np.cbrt(grid.v).min()) / c
    setup = time.perf_counter() - t0
    if write:
        write_state(out / "rst_0.vtk", mesh, grid, y, r, gamm)
    yd = torch.from_numpy(y).cuda()
    yi = torch.empty_like(yd)
    ctx.to_internal(yd, yi)
    t, k_out, n_steps, tot = 0.0, 0, 0, {}
    t_next = t_int
    resume = 0
    h = dt
    while adaptive and t < t_final * (1.0 - 1e-12):
        t_stop = min(t_next, t_final)
        nk = ctx.bdf_defaults(precond=precond, newton_rtol=newton_rtol)
        ad = ctx.adapt_defaults(rtol=rtol, atol=atol, h0=min(h, t_stop - t))
        rc, st, ast = ctx.bdf_adaptive(yi, t, t_stop, nk, ad)
        if rc != 0:
            raise RuntimeError(f"adaptive BDF failed at t = {t:g} (rc {rc}): {ast}")
        t = t_stop
        h = ast["h_last"]
        n_steps += ast["n_accepted"]
        for key, val in list(st.items()) + list(ast.items()):
            if isinstance(val, (int, float)) and key.startswith("n_"):
                tot[key] = tot.get(key, 0) + val
        log(f"[i] t = {t:.6g}, {n_steps} steps (last h = {h:.4g}, order {ast['q_last']}), "
            f"Newton {st['n_newton']}, Krylov {st['n_lin_iters']}")
        k_out += 1
        if write:
            yo = torch.empty_like(yi)
            ctx.to_reference(yi, yo)
            write_state(out / f"rst_{k_out}.vtk", mesh, grid, yo.cpu().numpy(), r, gamm)
        t_next += t_int
    while not adaptive and t < t_final * (1.0 - 1e-12) and (max_steps is None or n_steps < max_steps):
        n = max(1, int(math.ceil((min(t_next, t_final) - t) / dt - 1e-9)))
        if max_steps is not None:
            n = min(n, max_steps - n_steps)
        opts = ctx.bdf_defaults(order=order, dt=dt, nsteps=n, precond=precond,
                                newton_rtol=newton_rtol, resume=resume)
        rc, st = ctx.bdf_run(yi, opts, t0=t)
        if rc != 0:
            raise RuntimeError(f"BDF steps failed at t = {t:g} (rc {rc}): {st}")
        resume = 1
        t += n * dt
        n_steps += n
        for key, val in st.items():
            if isinstance(val, (int, float)) and key.startswith("n_"):
                tot[key] = tot.get(key, 0) + val
        log(f"[i] t = {t:.6g}, {n_steps} steps of dt = {dt:.4g}, Newton {st['n_newton']}, "
            f"Krylov {st['n_lin_iters']}")
        if t + 1e-12 * max(t_final, 1.0) >= t_next:
            k_out += 1
            if write:
                yo = torch.empty_like(yi)
                ctx.to_reference(yi, yo)
                write_state(out / f"rst_{k_out}.vtk", mesh, grid, yo.cpu().numpy(), r, gamm)
            t_next += t_int
    yo = torch.empty_like(yi)
    ctx.to_reference(yi, yo)
    y_final = yo.cpu().numpy()
    ctx.close()
    return {"y": y_final, "t": t, "dt": dt, "steps": n_steps, "outputs": k_out,
            "cells": grid.nC, "setup_s": setup, "stats": tot}


def _main(argv=None):
    ap = argparse.ArgumentParser(prog="python -m fosolvers_gb300.case",
                                 description="run a foeuler case directory on the GPU")
    ap.add_argument("case_dir")
    ap.add_argument("--out", default=None, help="output directory (default: the case)")
    ap.add_argument("--dt", type=float, default=None)
    ap.add_argument("--cfl", type=float, default=5.0, help="CFL on the initial state if no --dt")
    ap.add_argument("--order", type=int, default=2, choices=[1, 2])
    ap.add_argument("--fp32", action="store_true", help="FP32 flux and ILU(0) (flags 1 | 4 | 8)")
    ap.add_argument("--max-steps", type=int, default=None)
    ap.add_argument("--adaptive", action="store_true",
                    help="variable-order, variable-step BDF at --rtol/--atol (foeuler's CVODE "
                         "tolerances by default); --dt or --cfl then sets the first step")
    ap.add_argument("--rtol", type=float, default=1e-6)
    ap.add_argument("--atol", type=float, default=1e-12)
    a = ap.parse_args(argv)
    flags = (1 | 4 | 8) if a.fp32 else 0
    res = run_case(a.case_dir, a.out, dt=a.dt, cfl=a.cfl, order=a.order, flags=flags,
                   max_steps=a.max_steps, adaptive=a.adaptive, rtol=a.rtol, atol=a.atol)
    print(f"done: t = {res['t']:g}, {res['steps']} steps, {res['outputs']} outputs, "
          f"{res['cells']} cells")


if __name__ == "__main__":
    _main()
