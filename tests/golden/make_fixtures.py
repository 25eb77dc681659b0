"""Regenerate the committed fixtures under tests/golden/ (run in a checkout that has
the reference source tree; the GPU machines only read the .npz files).

bar_tet.npz   the reference's own unstructured test mesh src/test/data/bar_tet.vtk
              (Gmsh-generated bar, 14,728 tetrahedra + 3,336 boundary triangles),
              converted from legacy VTK the way readVTKPolyX does (VTK.f90:4-81):
              points, cells (+1 to 1-based node ids), cell types 10 -> TET, 5 -> TRI.
              Element order is kept; gid is 0 (the VTK reader sets no group ids).
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

REF = Path(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
OUT = Path(__file__).resolve().parent


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


def main():
    pts, conn, types = read_vtk(REF / "src/test/data/bar_tet.vtk")
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
