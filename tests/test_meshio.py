"""Mesh and case files on the host: Gmsh 2.2 / 4.1 reading (readGMSHPolyGrid semantics:
kept element types, geometric-entity group ids, element order as in the file), legacy VTK
writing and reading (writeVTKPolyX / readVTKPolyX semantics), the condition-table and
case-input readers, and the element order the face builder imposes."""
from pathlib import Path

import numpy as np
import pytest

from fosolvers_gb300 import mesh as M
from fosolvers_gb300 import meshio as IO
from fosolvers_gb300.case import (grid_order, initial_state, load_case, primitives,
                                  read_cond_tab, read_ic, read_fl, read_sim, sorted_mesh)
from fosolvers_gb300.euler import PolyFvGrid

import os

GOLDEN = Path(__file__).resolve().parent / "golden"
# a checkout of the reference source tree, when one is at hand (FOS_REFERENCE); the tests
# that read its files directly are skipped without it, the committed fixtures cover the rest
REFERENCE = Path(os.environ["FOS_REFERENCE"]) if os.environ.get("FOS_REFERENCE") else None


def duct_mesh() -> M.Mesh:
    """The reference's examples/foeuler/duct mesh, from tests/golden/duct.npz."""
    d = np.load(GOLDEN / "duct.npz")
    return M.Mesh(pN=d["pN"], sE=d["sE"], nNE=d["nNE"], iNE=d["iNE"], gid=d["gid"],
                  nC=int(d["nC"]))


def write_duct_case(case_dir: Path) -> Path:
    """The duct example's case directory (grid.msh as Gmsh 2.2, bc, ic, sim, fl)."""
    d = np.load(GOLDEN / "duct.npz")
    case_dir.mkdir(parents=True, exist_ok=True)
    IO.write_gmsh(case_dir / "grid.msh", duct_mesh(), version=2.2)
    for k in ("bc", "ic", "sim", "fl"):
        (case_dir / k).write_text(str(d[k]))
    return case_dir


@pytest.mark.parametrize("version", [2.2, 4.1])
def test_gmsh_round_trip_gives_identical_face_arrays(tmp_path, version):
    m = M.box_mesh(4, 3, 2, jitter=0.1, seed=3)
    p = tmp_path / "g.msh"
    IO.write_gmsh(p, m, version=version)
    r = IO.read_gmsh(p)
    assert r.nN == m.nN and r.nE == m.nE and r.nC == m.nC
    np.testing.assert_array_equal(r.pN, m.pN)  # repr() round-trips doubles exactly
    order = np.argsort(np.arange(m.nE))  # 2.2 keeps file order; 4.1 groups by block
    if version > 4:
        # blocks are written per (dim, gid, shape) in first-appearance order
        keys = [(3 if s in IO.CELL_SHAPES else 2, g, s) for s, g in zip(m.sE, m.gid)]
        first = {}
        for e, k in enumerate(keys):
            first.setdefault(k, len(first))
        order = np.array(sorted(range(m.nE), key=lambda e: (first[keys[e]], e)))
    np.testing.assert_array_equal(r.sE, m.sE[order])
    np.testing.assert_array_equal(r.gid, m.gid[order])
    np.testing.assert_array_equal(r.iNE[:, :4], m.iNE[order, :4])
    a, b = PolyFvGrid.from_mesh(m), PolyFvGrid.from_mesh(r)
    np.testing.assert_array_equal(a.iEP, b.iEP)
    np.testing.assert_array_equal(a.aP, b.aP)
    np.testing.assert_array_equal(a.normP, b.normP)


def test_gmsh_22_skips_unsupported_types_and_reads_entity_tags(tmp_path):
    text = """$MeshFormat
2.2 0 8
$EndMeshFormat
$Nodes
5
10 0 0 0
20 1 0 0
30 0 1 0
40 0 0 1
50 1 1 1
$EndNodes
$Elements
5
1 15 2 9 1 10
2 1 2 9 2 10 20
3 2 2 7 3 10 20 30
4 4 2 8 4 10 20 30 40
5 4 2 8 4 20 30 40 50
$EndElements
"""
    p = tmp_path / "t.msh"
    p.write_text(text)
    m = IO.read_gmsh(p)
    # the point (15) and the line (1) are skipped; sparse node tags map to 1..5 in order
    np.testing.assert_array_equal(m.sE, [IO.TRI, IO.TET, IO.TET])
    np.testing.assert_array_equal(m.gid, [3, 4, 4])  # the elementary (second) tag
    np.testing.assert_array_equal(m.iNE[0, :3], [1, 2, 3])
    np.testing.assert_array_equal(m.iNE[2], [2, 3, 4, 5])
    assert m.nC == 2
    # facet first in the file: the grid order puts the cells first
    np.testing.assert_array_equal(grid_order(m), [1, 2, 0])
    s = sorted_mesh(m)
    np.testing.assert_array_equal(s.sE, [IO.TET, IO.TET, IO.TRI])
    g = PolyFvGrid.from_mesh(m)
    np.testing.assert_array_equal(g.gid, s.gid)


def test_gmsh_rejects_binary_and_missing_sections(tmp_path):
    p = tmp_path / "b.msh"
    p.write_text("$MeshFormat\n2.2 1 8\n$EndMeshFormat\n")
    with pytest.raises(IO.MeshFileError):
        IO.read_gmsh(p)
    p.write_text("$MeshFormat\n2.2 0 8\n$EndMeshFormat\n$Nodes\n1\n1 0 0 0\n$EndNodes\n")
    with pytest.raises(IO.MeshFileError):
        IO.read_gmsh(p)


def test_reads_the_duct_example_mesh(tmp_path):
    """The reference's duct example (Gmsh 2.2): 13,704 nodes, 65,483 tetrahedra, 10,816
    boundary triangles in groups 1..7; the face arrays close every cell.  The mesh comes
    from the committed fixture, written back as Gmsh 2.2 and read again (the same arrays);
    with a reference checkout at hand the original file is read too."""
    m = IO.read_gmsh(write_duct_case(tmp_path) / "grid.msh")
    f = duct_mesh()
    for k in ("pN", "sE", "nNE", "iNE", "gid"):
        np.testing.assert_array_equal(getattr(m, k), getattr(f, k))
    if REFERENCE is not None and (REFERENCE / "examples/foeuler/duct/grid.msh").exists():
        r = IO.read_gmsh(REFERENCE / "examples/foeuler/duct/grid.msh")
        for k in ("pN", "sE", "nNE", "iNE", "gid"):
            np.testing.assert_array_equal(getattr(r, k), getattr(f, k))
    assert (m.nN, m.nC) == (13704, 65483)
    assert int((m.sE == IO.TRI).sum()) == 10816
    assert set(np.unique(m.gid)) == set(range(1, 8))
    g = PolyFvGrid.from_mesh(m)
    assert (g.nC, g.nPb) == (65483, 10816)
    assert np.all(g.v > 0)
    # closure: sum of aP n over each cell's faces vanishes
    acc = np.zeros((g.nC, 3))
    an = g.aP[:, None] * g.normP
    L, R = g.iEP[:, 0] - 1, g.iEP[:, 1] - 1
    np.add.at(acc, L, an)
    inner = R < g.nC
    np.add.at(acc, R[inner], -an[inner])
    assert np.abs(acc).max() <= 1e-12 * np.abs(an).max() * 10


MESH_SIMPLE = REFERENCE / "src/test/data/mesh_simple.vtk" if REFERENCE else None


@pytest.mark.skipif(MESH_SIMPLE is None or not MESH_SIMPLE.exists(),
                    reason="no reference checkout (FOS_REFERENCE)")
def test_reads_the_reference_simple_vtk_mesh():
    """src/test/readVTK1.f90:10-22: the four triangles of data/mesh_simple.vtk come out with
    1-based nodes (1,3,2), (1,4,3), (1,2,4), (2,3,4), all TRI with 3 nodes."""
    m, _ = IO.read_vtk(MESH_SIMPLE)
    np.testing.assert_array_equal(m.iNE[:, :3], [[1, 3, 2], [1, 4, 3], [1, 2, 4], [2, 3, 4]])
    assert np.all(m.sE == IO.TRI) and np.all(m.nNE == 3)


def test_vtk_round_trip_with_cell_and_point_data(tmp_path):
    m = M.box_mesh(3, 2, 2, jitter=0.05, seed=1)
    rng = np.random.default_rng(0)
    rho = rng.uniform(1, 2, m.nE)
    u = rng.normal(size=(m.nE, 3))
    pt = rng.normal(size=m.nN)
    p = tmp_path / "s.vtk"
    IO.write_vtk(p, m, cell_data={"density": rho, "velocity": u}, point_data={"phi": pt})
    text = p.read_text().splitlines()
    assert text[0] == "# vtk DataFile Version 3.0" and "DATASET UNSTRUCTURED_GRID" in text
    r, data = IO.read_vtk(p)
    np.testing.assert_array_equal(r.pN, m.pN)
    np.testing.assert_array_equal(r.sE, m.sE)
    np.testing.assert_array_equal(r.iNE[:, :4], m.iNE[:, :4])
    np.testing.assert_array_equal(data["cell"]["density"], rho)
    np.testing.assert_array_equal(data["cell"]["velocity"], u)
    np.testing.assert_array_equal(data["point"]["phi"], pt)
    with pytest.raises(ValueError):
        IO.write_vtk(p, m, cell_data={"bad": np.zeros(m.nE + 1)})


def _write_case(d: Path, mesh, conds, ic=(1.0e5, 300.0, 10.0, 0.0, 0.0), sim=(1e-3, 5e-4),
                fl=(287.058, 1.4)):
    """A case directory in the reference's input formats."""
    IO.write_gmsh(d / "grid.msh", mesh)
    m = max(len(c[2]) for c in conds)
    lines = [f"{len(conds)}   number of conditions", f"{m}   maximum parameters"]
    for gid, typ, par in conds:
        lines += ["", f"{gid}   group", f"{typ}   type", f"{len(par)}   parameters"]
        lines += [f"{x!r}" for x in par]
    (d / "bc").write_text("\n".join(lines) + "\n")
    (d / "ic").write_text("0   no UDF\n" + "\n".join(f"{x!r}   value" for x in ic) + "\n")
    (d / "sim").write_text(f"{sim[0]!r}   final time\n{sim[1]!r}   interval\n")
    (d / "fl").write_text(f"{fl[0]!r}   r\n{fl[1]!r}   gamma\n")


def test_case_inputs_and_initial_state(tmp_path):
    m = M.box_mesh(3, 3, 3, jitter=0.0, seed=0)
    _write_case(tmp_path, m, [(M.GID_XMIN, 11, [1.2e5, 310.0, 1.0, 0.0, 0.0]),
                              (M.GID_XMAX, 20, [0.9e5])])
    bc = read_cond_tab(tmp_path / "bc")
    np.testing.assert_array_equal(bc.gid, [M.GID_XMIN, M.GID_XMAX])
    np.testing.assert_array_equal(bc.type, [11, 20])
    np.testing.assert_array_equal(bc.param[0], [1.2e5, 310.0, 1.0, 0.0, 0.0])
    np.testing.assert_array_equal(bc.param[1], [0.9e5, 0, 0, 0, 0])
    ic = read_ic(tmp_path / "ic")
    assert read_sim(tmp_path / "sim") == (1e-3, 5e-4)
    r, g = read_fl(tmp_path / "fl")
    y = initial_state(10, ic, r, g)
    rho, u, p, T = primitives(y, 10, r, g)
    np.testing.assert_allclose(p, 1e5, rtol=1e-14)
    np.testing.assert_allclose(T, 300.0, rtol=1e-14)
    np.testing.assert_allclose(u[:, 0], 10.0, rtol=1e-14)
    ci = load_case(tmp_path)
    assert ci.mesh.nC == m.nC and ci.t_final == 1e-3
    (tmp_path / "ic").write_text("1\n1\n2\n3\n4\n5\n")
    with pytest.raises(NotImplementedError):
        read_ic(tmp_path / "ic")
