"""Regenerate the committed fixtures under tests/golden/ from a checkout of the reference
source tree, given as the first argument or in the FOS_REFERENCE environment variable (the
GPU machines and the tests only read the .npz files).

bar_tet.npz   the reference's own unstructured test mesh src/test/data/bar_tet.vtk
              (Gmsh-generated bar, 14,728 tetrahedra + 3,336 boundary triangles),
              converted from legacy VTK the way readVTKPolyX does (VTK.f90:4-81):
              points, cells (+1 to 1-based node ids), cell types 10 -> TET, 5 -> TRI.
              Element order is kept; gid is 0 (the VTK reader sets no group ids).
duct.npz      the reference's foeuler example examples/foeuler/duct: its Gmsh 2.2 mesh
              (13,704 nodes, 65,483 tetrahedra, 10,816 boundary triangles in groups 1..7)
              read with fosolvers_gb300.meshio.read_gmsh (readGMSHPolyGrid semantics), and
              the text of its bc, ic, sim and fl input files, so that a test can rebuild the
              case directory without the reference tree.
"""
from __future__ import annotations

import os
import sys
from pathlib import Path

import numpy as np

OUT = Path(__file__).resolve().parent


def reference_root() -> Path:
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("FOS_REFERENCE")
    if not root:
        raise SystemExit("usage: make_fixtures.py <reference checkout> (or set FOS_REFERENCE)")
    return Path(root)


def read_vtk(path: Path):
    tok = path.read_text().split()
    i = tok.index("POINTS")
    n = int(tok[i + 1])
    pts = np.array(tok[i + 3:i + 3 + 3 * n], dtype=np.float64).reshape(n, 3)
    i = tok.index("CELLS")
    m, total = int(tok[i + 1]), int(tok[i + 2])
    raw = np.array(tok[i + 3:i + 3 + total], dtype=np.int64)
    i = tok.index("CELL_TYPES")
    types = np.array(tok[i + 2:i + 2 + m], dtype=np.int64)
    conn, k = [], 0
    for _ in range(m):
        c = raw[k]
        conn.append(raw[k + 1:k + 1 + c] + 1)
        k += c + 1
    return pts, conn, types


def duct(ref: Path):
    sys.path.insert(0, str(OUT.parents[1]))
    from fosolvers_gb300.meshio import read_gmsh
    d = ref / "examples/foeuler/duct"
    m = read_gmsh(d / "grid.msh")
    texts = {k: np.array((d / k).read_text()) for k in ("bc", "ic", "sim", "fl")}
    np.savez_compressed(OUT / "duct.npz", pN=m.pN, sE=m.sE, nNE=m.nNE, iNE=m.iNE, gid=m.gid,
                        nC=np.int64(m.nC), **texts)
    print("duct:", m.pN.shape, m.nC, m.nE - m.nC)


def main():
    ref = reference_root()
    duct(ref)
    pts, conn, types = read_vtk(ref / "src/test/data/bar_tet.vtk")
    shape = {10: 20, 5: 10}
    sE = np.array([shape[int(t)] for t in types], np.int32)
    nNE = np.array([len(c) for c in conn], np.int32)
    iNE = np.zeros((len(conn), 4), np.int32)
    for e, c in enumerate(conn):
        iNE[e, :len(c)] = c
    np.savez_compressed(OUT / "bar_tet.npz", pN=pts, sE=sE, nNE=nNE, iNE=iNE)
    print("bar_tet:", pts.shape, np.bincount(sE)[[10, 20]])


if __name__ == "__main__":
    main()
