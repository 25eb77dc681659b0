"""Shared set-up for the parity tests: one workload -> reference face arrays, oracle
context and GPU context on the same mesh and initial state."""
from __future__ import annotations

import numpy as np

from fosolvers_gb300 import mesh as M
from fosolvers_gb300.euler import FOEuler, PolyFvGrid
from oracle import pyoracle as O


class Case:
    def __init__(self, wl: M.Workload, flags: int = 0, grid_from: str = "product"):
        self.wl = wl
        self.grid = PolyFvGrid.from_mesh(wl.mesh)
        self.g = self.grid.__dict__
        self.nC = self.grid.nC
        self.N = 5 * self.nC
        self.iBC = M.ibc_for(wl.mesh, wl.bc_gid)
        self.y0 = M.soa(wl.elem_state, self.nC)
        self.flags = flags
        self._oracle = None
        self._gpu = None
        self._gpu_has_factor = False

    @property
    def oracle(self) -> O.Euler:
        if self._oracle is None:
            self._oracle = O.Euler(self.g, self.iBC, self.wl.bc_type, self.wl.bc_param,
                                   self.wl.gamm, self.wl.r, self.wl.elem_state)
        return self._oracle

    @property
    def gpu(self) -> FOEuler:
        if self._gpu is None:
            self._gpu = FOEuler(self.grid, self.iBC, self.wl.bc_type, self.wl.bc_param,
                                self.wl.gamm, self.wl.r, flags=self.flags)
        return self._gpu

    def match_ilu_order(self):
        """ILU(0) depends on the cell order: factor the oracle in the GPU's order (the GPU
        sets its order up at the first pset, so run one on the initial state first)."""
        if not self._gpu_has_factor:
            self.gpu.pset(0.0, self.y0, None, 0, 1e-3)
            self._gpu_has_factor = True
        self.oracle.set_ilu_order(self.gpu.ilu_order())

    def oracle_rhs(self, y):
        f = np.zeros_like(y)
        rc = self.oracle.rhs(0.0, np.ascontiguousarray(y), f)
        assert rc == 0
        return f


def hex_workload(nx: int = 10, seed: int = 0) -> M.Workload:
    """nx x (nx - 2) x (nx - 4) jittered hexahedra (HEX cells, QUAD facets), the sinusoidal
    state, walls, BDF2 dt = 5e-4 x 6 steps: the six-face cell kernels' case."""
    m = M.box_mesh(nx, nx - 2, nx - 4, jitter=0.1, seed=seed, cells="hex")
    st = M.sine_state(m.centroids(), seed)
    return M.Workload(f"hex{nx}", m, st, np.zeros(0, np.int32), np.zeros(0, np.int32),
                      np.zeros((0, 5)), order=2, dt=5e-4, nsteps=6)


def with_all_conditions(wl: M.Workload) -> M.Workload:
    """Every non-UDF condition of setBC (foeuler.f90:217-325) on the six box sides: static
    inflow (subsonic: interior momentum), total inflow, outflow (imposed p), far field,
    zero-gradient outflow, wall."""
    wl.bc_gid = np.array([1, 2, 3, 4, 5, 6], np.int32)
    wl.bc_type = np.array([10, 11, 20, 30, 21, 0], np.int32)
    wl.bc_param = np.array([[1.0, 1.0, 0.3, 0.0, 0.0],
                            [1.2, 1.1, 0.5, 0.1, 0.0],
                            [0.9, 0, 0, 0, 0],
                            [1.0, 1.0, 0.2, 0.1, 0.05],
                            [0, 0, 0, 0, 0],
                            [0, 0, 0, 0, 0]])
    return wl


def perturbed(y: np.ndarray, nC: int, seed: int, amp: float = 0.05) -> np.ndarray:
    """Smooth-ish random perturbation that keeps rho and p positive."""
    rng = np.random.default_rng(seed)
    y = y.copy().reshape(5, nC)
    rho = y[0] * (1.0 + amp * rng.uniform(-1, 1, nC))
    u = y[1:4] / y[0] + amp * rng.uniform(-1, 1, (3, nC))
    p = (0.4) * (y[4] - 0.5 * (y[1:4] ** 2).sum(0) / y[0]) * (1.0 + amp * rng.uniform(-1, 1, nC))
    out = np.empty_like(y)
    out[0] = rho
    out[1:4] = rho * u
    out[4] = p / 0.4 + 0.5 * rho * (u ** 2).sum(0)
    return out.reshape(-1)


def rel_err(a: np.ndarray, b: np.ndarray) -> float:
    """max |a - b| / max |b| per conserved block, maximum over the 5 blocks."""
    a = a.reshape(5, -1)
    b = b.reshape(5, -1)
    return float(max(np.abs(a[q] - b[q]).max() / max(np.abs(b[q]).max(), 1e-300) for q in range(5)))


def field_errors(a: np.ndarray, b: np.ndarray) -> dict:
    """Errors per conserved field relative to the field's largest magnitude; momentum is one
    vector field (relative to max |rho u|), so near-zero transverse components are not
    normalised by their own tiny maximum."""
    a = a.reshape(5, -1)
    b = b.reshape(5, -1)
    mom = np.sqrt((b[1:4] ** 2).sum(0)).max()
    return {"rho": float(np.abs(a[0] - b[0]).max() / np.abs(b[0]).max()),
            "rhou": float(np.abs(a[1:4] - b[1:4]).max() / max(mom, 1e-300)),
            "rhoE": float(np.abs(a[4] - b[4]).max() / np.abs(b[4]).max()),
            "per_component": [float(np.abs(a[q] - b[q]).max()) for q in range(5)]}


def cell_errors(a: np.ndarray, b: np.ndarray) -> dict:
    """Per-cell relative errors: the largest ||a_c - b_c|| / ||b_c|| over cells (the 5-vector
    of conserved variables of cell c), and per field the largest |a - b| / |b| of density and
    energy (bounded away from zero; momentum components cross zero, so momentum enters
    through the cell vector only)."""
    a = a.reshape(5, -1)
    b = b.reshape(5, -1)
    nb = np.sqrt((b ** 2).sum(0))
    nd = np.sqrt(((a - b) ** 2).sum(0))
    return {"cell": float((nd / nb).max()),
            "rho": float((np.abs(a[0] - b[0]) / np.abs(b[0])).max()),
            "rhoE": float((np.abs(a[4] - b[4]) / np.abs(b[4])).max())}
