"""Grid set-up parity: libfosgpu's face builder (fos_grid_build, host code) against
the oracle's restatement of polyGrid%up + getNeibPolyFvGrid + sortPolyFvGrid.
Pairs, order, normals, areas, centres, volumes and neighbour tables must agree.
CPU only (no device calls)."""
from pathlib import Path

import numpy as np
import pytest

from fosolvers_gb300 import mesh as M
from fosolvers_gb300.euler import PolyFvGrid
from oracle import pyoracle as O

GOLDEN = Path(__file__).resolve().parent / "golden"


def bar_tet_mesh() -> M.Mesh:
    d = np.load(GOLDEN / "bar_tet.npz")
    sE = d["sE"]
    return M.Mesh(pN=d["pN"], sE=sE, nNE=d["nNE"], iNE=d["iNE"], gid=np.zeros(sE.size, np.int32),
                  nC=int((sE == 20).sum()))


def _compare(mesh):
    g = PolyFvGrid.from_mesh(mesh)
    r = O.grid_build(mesh)
    for k in ("nC", "nE", "nP", "nPi", "nPb", "maxFace"):
        assert getattr(g, k) == r[k], k
    for k in ("iEP", "neib", "gid", "sE"):
        assert np.array_equal(getattr(g, k), r[k]), k
    for k in ("aP", "normP", "pP", "p"):
        np.testing.assert_allclose(getattr(g, k), r[k], rtol=0, atol=1e-14 * max(1.0, np.abs(r[k]).max()))
    # v4p expands the determinant in absolute coordinates (geometry.f90:61-82); the product
    # forms edge vectors first, so thin cells far from the origin differ by ~1e-13 relative
    np.testing.assert_allclose(g.v, r["v"], rtol=1e-11, atol=0)
    return g


@pytest.mark.parametrize("dims,seed", [((1, 1, 1), 0), ((4, 3, 5), 1), ((6, 6, 6), 2)])
def test_box_grid_matches_reference(dims, seed):
    g = _compare(M.box_mesh(*dims, jitter=0.1, seed=seed))
    nx, ny, nz = dims
    assert g.nC == 6 * nx * ny * nz
    assert g.nPb == 4 * (nx * ny + ny * nz + nx * nz)
    assert np.all(g.iEP[: g.nPi, 1] <= g.nC) and np.all(g.iEP[g.nPi:, 1] > g.nC)


@pytest.mark.parametrize("dims,seed", [((1, 1, 1), 0), ((4, 3, 5), 1)])
def test_hex_box_grid_matches_reference(dims, seed):
    """HEX cells and QUAD facets (hexahedron face table, quad face areas, six-tetrahedron
    volumes) against the oracle's restatement."""
    g = _compare(M.box_mesh(*dims, jitter=0.1, seed=seed, cells="hex"))
    nx, ny, nz = dims
    assert g.nC == nx * ny * nz and g.maxFace == 6
    assert g.nPb == 2 * (nx * ny + ny * nz + nx * nz)
    assert g.nPi == 3 * nx * ny * nz - (nx * ny + ny * nz + nx * nz)
    assert abs(g.v.sum() - 1.0) < 1e-13


def test_unjittered_hex_cells_are_closed():
    g = PolyFvGrid.from_mesh(M.box_mesh(4, 3, 2, jitter=0.0, cells="hex"))
    S = np.zeros((g.nC, 3))
    an = g.aP[:, None] * g.normP
    np.add.at(S, g.iEP[:, 0] - 1, an)
    inner = g.iEP[:, 1] <= g.nC
    np.add.at(S, g.iEP[inner, 1] - 1, -an[inner])
    assert np.abs(S).max() < 1e-15
    np.testing.assert_allclose(g.v, 1.0 / 24, rtol=1e-13)


def test_bump_grid_matches_reference():
    _compare(M.box_mesh(12, 4, 2, extent=(3.0, 1.0, 0.5), jitter=0.0, bump=True))


def test_bar_tet_grid_matches_reference():
    """The reference's own unstructured test mesh (src/test/data/bar_tet.vtk)."""
    g = _compare(bar_tet_mesh())
    assert g.nC == 14728 and g.nPb == 3336


def test_sod16_sizes():
    """16^3 x 6 tets: nC 24,576, nPb 3,072, nPi 47,616, nP 50,688."""
    g = PolyFvGrid.from_mesh(M.box_mesh(16, 16, 16, seed=0))
    assert (g.nC, g.nPb, g.nPi, g.nP) == (24576, 3072, 47616, 50688)


def test_cells_are_closed():
    """sum over a cell's faces of aP * outward normal = 0 and the volumes tile the box."""
    g = PolyFvGrid.from_mesh(M.box_mesh(5, 4, 3, seed=3))
    S = np.zeros((g.nC, 3))
    an = g.aP[:, None] * g.normP
    np.add.at(S, g.iEP[:, 0] - 1, an)
    inner = g.iEP[:, 1] <= g.nC
    np.add.at(S, g.iEP[inner, 1] - 1, -an[inner])
    assert np.abs(S).max() < 1e-15
    assert abs(g.v.sum() - 1.0) < 1e-13


def test_qsort_matches_reference_permutation(oracle_lib):
    """The product's pair ordering uses the reference quicksort (sort.f90): same permutation
    on keys with many ties."""
    rng = np.random.default_rng(5)
    a = rng.integers(0, 50, 2000).astype(np.int32)
    a0 = a.copy()
    perm = np.zeros_like(a)
    oracle_lib.og_qsort_perm(a.size, O.ip(a), O.ip(perm))
    assert np.array_equal(a, np.sort(a0))
    assert np.array_equal(a0[perm - 1], a)
