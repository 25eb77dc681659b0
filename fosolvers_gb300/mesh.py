"""Seeded synthetic tetrahedral meshes and initial states for the foeuler workloads.

The reference reads Gmsh files (fileIO/GMSH.f90); the workloads here are
generated instead, with the same element tables a Gmsh read produces:

* a box of nx x ny x nz hexahedra, each cut into the 6 tetrahedra of the Kuhn
  split (every tetrahedron contains the hexahedron's main diagonal), all hexes
  cut the same way so the faces conform; every tetrahedron is positively
  oriented, so the TET face tables (polyGrid.f90:236-247) give outward normals;
* interior nodes jittered uniformly by +-jitter*h per axis from a seeded
  numpy PCG64 generator (identical on x86 and Arm);
* optional bump-channel mapping of the bottom wall, y0(x) = 0.1 exp(-((x-1)/0.2)^2),
  blended linearly to the top wall;
* boundary triangles (TRI facets) on the six sides with group ids
  1..6 = x-min, x-max, y-min, y-max, z-min, z-max.

Elements are returned cells first, then facets (the order sortPolyGrid makes).
"""
from __future__ import annotations

from dataclasses import dataclass, field
from itertools import permutations

import numpy as np

TET, TRI, HEX, QUAD = 20, 10, 21, 11
GID_XMIN, GID_XMAX, GID_YMIN, GID_YMAX, GID_ZMIN, GID_ZMAX = 1, 2, 3, 4, 5, 6


@dataclass
class Mesh:
    pN: np.ndarray          # (nN, 3) float64 node positions
    sE: np.ndarray          # (nE,) int32 shape codes
    nNE: np.ndarray         # (nE,) int32 nodes per element
    iNE: np.ndarray         # (nE, m) int32 1-based node ids (row = element; m = 4, or 8 with hexes)
    gid: np.ndarray         # (nE,) int32 group ids
    nC: int
    dims: tuple = ()
    extent: tuple = ()
    meta: dict = field(default_factory=dict)

    @property
    def nE(self) -> int:
        return int(self.sE.shape[0])

    @property
    def nN(self) -> int:
        return int(self.pN.shape[0])

    def centroids(self) -> np.ndarray:
        idx = self.iNE - 1
        cnt = self.nNE[:, None].astype(np.float64)
        mask = (np.arange(idx.shape[1])[None, :] < self.nNE[:, None])
        pts = self.pN[np.where(mask, idx, 0)] * mask[..., None]
        return pts.sum(axis=1) / cnt


def _kuhn_tets() -> np.ndarray:
    """6 tets of the unit cube as corner indices (corner = a + 2b + 4c), positive volume."""
    corner = lambda a, b, c: a + 2 * b + 4 * c
    coords = np.array([[(k >> 0) & 1, (k >> 1) & 1, (k >> 2) & 1] for k in range(8)], float)
    tets = []
    for perm in permutations(range(3)):
        p = [0, 0, 0]
        path = [corner(*p)]
        for ax in perm:
            p[ax] = 1
            path.append(corner(*p))
        a, b, c, d = (coords[k] for k in path)
        if np.linalg.det(np.stack([b - a, c - a, d - a])) < 0:
            path[1], path[2] = path[2], path[1]
        tets.append(path)
    return np.array(tets, dtype=np.int64)


def box_mesh(nx: int, ny: int, nz: int, extent=(1.0, 1.0, 1.0), jitter: float = 0.1,
             seed: int = 0, bump: bool = False, cells: str = "tet") -> Mesh:
    """The box of nx x ny x nz hexahedra; cells="tet" cuts each into the 6 Kuhn
    tetrahedra with TRI facets, cells="hex" keeps the HEX cells (Gmsh node order:
    bottom face counter-clockwise, then the top face) with QUAD facets."""
    if cells not in ("tet", "hex"):
        raise ValueError(f"cells must be 'tet' or 'hex', not {cells!r}")
    Lx, Ly, Lz = extent
    hx, hy, hz = Lx / nx, Ly / ny, Lz / nz
    ix, iy, iz = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), np.arange(nz + 1), indexing="ij")
    # node id = i + (nx+1)*(j + (ny+1)*k)
    ix = ix.transpose(2, 1, 0).reshape(-1)
    iy = iy.transpose(2, 1, 0).reshape(-1)
    iz = iz.transpose(2, 1, 0).reshape(-1)
    pN = np.stack([ix * hx, iy * hy, iz * hz], axis=1).astype(np.float64)
    interior = (ix > 0) & (ix < nx) & (iy > 0) & (iy < ny) & (iz > 0) & (iz < nz)
    if jitter > 0.0:
        rng = np.random.default_rng(seed)
        nint = int(interior.sum())
        d = rng.uniform(-jitter, jitter, size=(nint, 3)) * np.array([hx, hy, hz])
        pN[interior] += d
    if bump:
        x, y = pN[:, 0], pN[:, 1]
        y0 = 0.1 * np.exp(-((x - 1.0) / 0.2) ** 2)
        pN[:, 1] = y0 + y / Ly * (Ly - y0)
    nid = lambda i, j, k: i + (nx + 1) * (j + (ny + 1) * k)
    # hexes in k-major, i-fastest order
    hk, hj, hi = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    hi, hj, hk = hi.reshape(-1), hj.reshape(-1), hk.reshape(-1)
    corners = np.stack([nid(hi + (k & 1), hj + ((k >> 1) & 1), hk + ((k >> 2) & 1))
                        for k in range(8)], axis=1)  # (nH, 8)
    if cells == "hex":
        return _hex_box(pN, corners, nid, nx, ny, nz, extent,
                        {"jitter": jitter, "seed": seed, "bump": bump, "cells": "hex"})
    kt = _kuhn_tets()
    tets = corners[:, kt].reshape(-1, 4)  # (6 nH, 4)
    # boundary triangles: quad (a, b, c, d) with the min->max diagonal, split as in the Kuhn tets
    tris, gids = [], []

    def side(fixed_axis, fixed_val, gid):
        axes = [a for a in range(3) if a != fixed_axis]
        n1 = [nx, ny, nz][axes[0]]
        n2 = [nx, ny, nz][axes[1]]
        u, v = np.meshgrid(np.arange(n1), np.arange(n2), indexing="ij")
        u, v = u.reshape(-1), v.reshape(-1)

        def node(du, dv):
            ijk = [None, None, None]
            ijk[fixed_axis] = np.full_like(u, fixed_val)
            ijk[axes[0]] = u + du
            ijk[axes[1]] = v + dv
            return nid(*ijk)

        p00, p10, p01, p11 = node(0, 0), node(1, 0), node(0, 1), node(1, 1)
        tris.append(np.stack([p00, p10, p11], axis=1))
        tris.append(np.stack([p00, p01, p11], axis=1))
        gids.append(np.full(2 * u.size, gid))

    side(0, 0, GID_XMIN); side(0, nx, GID_XMAX)
    side(1, 0, GID_YMIN); side(1, ny, GID_YMAX)
    side(2, 0, GID_ZMIN); side(2, nz, GID_ZMAX)
    tris = np.concatenate(tris)
    gids = np.concatenate(gids)
    nC, nF = tets.shape[0], tris.shape[0]
    iNE = np.zeros((nC + nF, 4), np.int32)
    iNE[:nC] = tets + 1
    iNE[nC:, :3] = tris + 1
    sE = np.concatenate([np.full(nC, TET, np.int32), np.full(nF, TRI, np.int32)])
    nNE = np.concatenate([np.full(nC, 4, np.int32), np.full(nF, 3, np.int32)])
    gid = np.concatenate([np.zeros(nC, np.int32), gids.astype(np.int32)])
    return Mesh(pN=pN, sE=sE, nNE=nNE, iNE=iNE, gid=gid, nC=nC, dims=(nx, ny, nz),
                extent=tuple(extent), meta={"jitter": jitter, "seed": seed, "bump": bump})


def _hex_box(pN, corners, nid, nx, ny, nz, extent, meta) -> Mesh:
    """HEX cells and QUAD side facets of the box; corner k of a hex is (k & 1, k >> 1 & 1,
    k >> 2) in its i, j, k offsets, so Gmsh order is corners 0, 1, 3, 2, 4, 5, 7, 6."""
    hexes = corners[:, [0, 1, 3, 2, 4, 5, 7, 6]]
    quads, gids = [], []

    def side(fixed_axis, fixed_val, gid):
        axes = [a for a in range(3) if a != fixed_axis]
        n1, n2 = [nx, ny, nz][axes[0]], [nx, ny, nz][axes[1]]
        u, v = np.meshgrid(np.arange(n1), np.arange(n2), indexing="ij")
        u, v = u.reshape(-1), v.reshape(-1)

        def node(du, dv):
            ijk = [None, None, None]
            ijk[fixed_axis] = np.full_like(u, fixed_val)
            ijk[axes[0]] = u + du
            ijk[axes[1]] = v + dv
            return nid(*ijk)

        quads.append(np.stack([node(0, 0), node(1, 0), node(1, 1), node(0, 1)], axis=1))
        gids.append(np.full(u.size, gid))

    side(0, 0, GID_XMIN); side(0, nx, GID_XMAX)
    side(1, 0, GID_YMIN); side(1, ny, GID_YMAX)
    side(2, 0, GID_ZMIN); side(2, nz, GID_ZMAX)
    quads = np.concatenate(quads)
    nC, nF = hexes.shape[0], quads.shape[0]
    iNE = np.zeros((nC + nF, 8), np.int32)
    iNE[:nC] = hexes + 1
    iNE[nC:, :4] = quads + 1
    sE = np.concatenate([np.full(nC, HEX, np.int32), np.full(nF, QUAD, np.int32)])
    nNE = np.concatenate([np.full(nC, 8, np.int32), np.full(nF, 4, np.int32)])
    gid = np.concatenate([np.zeros(nC, np.int32), np.concatenate(gids).astype(np.int32)])
    return Mesh(pN=pN, sE=sE, nNE=nNE, iNE=iNE, gid=gid, nC=nC, dims=(nx, ny, nz),
                extent=tuple(extent), meta=meta)


# ------------------------------------------------------------------ initial states
def conserved(rho, u, v, w, p, gamm):
    """(rho, rhou, rhov, rhow, rhoE) from primitives (foeuler.f90:133-135 with p = rho R T)."""
    return (rho, rho * u, rho * v, rho * w, p / (gamm - 1.0) + 0.5 * rho * (u * u + v * v + w * w))


def sod_state(x: np.ndarray, gamm: float = 1.4):
    """Sod shock tube along x: x < 0.5: rho = 1, p = 1; else rho = 0.125, p = 0.1; u = 0."""
    left = x[:, 0] < 0.5
    rho = np.where(left, 1.0, 0.125)
    p = np.where(left, 1.0, 0.1)
    z = np.zeros_like(rho)
    return conserved(rho, z, z, z, p, gamm)


def sine_state(x: np.ndarray, seed: int, gamm: float = 1.4, amp_rho: float = 0.05,
               amp_u: float = 0.1, nwaves: int = 4):
    """rho = 1 + amp sum_k sin(2 pi n_k.x + phi_k), n_k in [1,3]^3, phi_k ~ U[0, 2 pi);
    each velocity component the same form with amplitude amp_u (own n_k, phi_k); p = 1."""
    rng = np.random.default_rng(seed + 7919)

    def field(amp):
        n = rng.integers(1, 4, size=(nwaves, 3))
        phi = rng.uniform(0.0, 2.0 * np.pi, size=nwaves)
        s = np.zeros(x.shape[0])
        for k in range(nwaves):
            s += np.sin(2.0 * np.pi * (x @ n[k]) + phi[k])
        return amp * s

    rho = 1.0 + field(amp_rho)
    u, v, w = field(amp_u), field(amp_u), field(amp_u)
    p = np.ones_like(rho)
    return conserved(rho, u, v, w, p, gamm)


def freestream_state(n: int, rho=1.4, u=2.0, p=1.0, gamm: float = 1.4):
    z = np.zeros(n)
    return conserved(np.full(n, rho), np.full(n, u), z, z, np.full(n, p), gamm)


def soa(cons, nC: int) -> np.ndarray:
    """Stack conserved variables of the first nC elements into the SoA N_Vector layout."""
    return np.concatenate([np.asarray(c, np.float64)[:nC] for c in cons])


# ------------------------------------------------------------------ workloads
@dataclass
class Workload:
    name: str
    mesh: Mesh
    elem_state: tuple       # conserved variables for all nE elements (cells then facets)
    bc_gid: np.ndarray      # group id per condition row
    bc_type: np.ndarray     # condition codes
    bc_param: np.ndarray    # (nBC, 5) parameters
    order: int
    dt: float
    nsteps: int
    gamm: float = 1.4
    r: float = 1.0


def make_workload(name: str, scale: int | None = None, seed: int = 0) -> Workload:
    """The five workloads; `scale` overrides the hex count along x (for small cases)."""
    if name == "sod16":  # 16^3 x 6 tets, Sod, walls, BDF1 dt=1e-3 x 20
        n = scale or 16
        m = box_mesh(n, n, n, jitter=0.1, seed=seed)
        st = sod_state(m.centroids())
        return Workload(name, m, st, np.zeros(0, np.int32), np.zeros(0, np.int32),
                        np.zeros((0, 5)), order=1, dt=1e-3, nsteps=20)
    if name == "sine96":  # 96^3 x 6 = 5,308,416 tets, sinusoidal state, walls, BDF2 dt=5e-4 x 10
        n = scale or 96
        m = box_mesh(n, n, n, jitter=0.1, seed=seed)
        st = sine_state(m.centroids(), seed)
        return Workload(name, m, st, np.zeros(0, np.int32), np.zeros(0, np.int32),
                        np.zeros((0, 5)), order=2, dt=5e-4, nsteps=10)
    if name in ("bump192", "bump320"):
        nx, ny, nz = (192, 64, 32) if name == "bump192" else (320, 107, 53)
        if scale:
            f = scale / nx
            nx, ny, nz = scale, max(2, round(ny * f)), max(2, round(nz * f))
        m = box_mesh(nx, ny, nz, extent=(3.0, 1.0, 0.5), jitter=0.0, seed=seed, bump=True)
        st = freestream_state(m.nE)
        gamm = 1.4
        # inflow: static, supersonic (code 10): p, T, u; T = p/(rho R) with R = 1
        bc_gid = np.array([GID_XMIN, GID_XMAX], np.int32)
        bc_type = np.array([10, 21], np.int32)
        bc_param = np.array([[1.0, 1.0 / 1.4, 2.0, 0.0, 0.0], [0.0] * 5])
        h = 3.0 / nx
        c_max = 2.0 + np.sqrt(gamm * 1.0 / 1.4)
        dt = 5.0 * h / c_max  # CFL ~ 5 on the inflow state
        return Workload(name, m, st, bc_gid, bc_type, bc_param,
                        order=1 if name == "bump192" else 2, dt=dt,
                        nsteps=50 if name == "bump192" else 20, gamm=gamm)
    raise ValueError(f"unknown workload {name!r}")


def ibc_for(mesh: Mesh, bc_gid: np.ndarray) -> np.ndarray:
    """iBC per element: 1-based condition row whose gid matches, 0 = default wall
    (foeuler.f90:145-154)."""
    ibc = np.zeros(mesh.nE, np.int32)
    for row, g in enumerate(bc_gid):
        ibc[(mesh.gid == g) & (ibc == 0)] = row + 1
    return ibc
