"""Mesh and result files: Gmsh ASCII meshes in, legacy VTK out (and back in).

Restates the behaviour of the reference's readers and writers:

* ``read_gmsh`` -- readGMSHPolyGrid (libfosolvers/fileIO/GMSH.f90:4-157): Gmsh ASCII
  format 2.2 and 4.1, nodes and elements; element types 2 (3-node triangle), 3 (4-node
  quadrilateral), 9 (6-node triangle), 4 (4-node tetrahedron), 5 (8-node hexahedron) and
  11 (10-node tetrahedron) are kept, every other type is skipped; an element's group id is
  its geometric entity tag (format 2.2: the second tag; format 4.1: the block's entity
  tag).  Node tags may be sparse here (they are mapped to 1..nN in file order); the
  reference requires them to be 1..nN.
* ``write_vtk`` -- writeVTKPolyX / writeVTKHead / writeVTKScal / writeVTKVect
  (fileIO/VTK.f90:83-204): legacy ASCII ``UNSTRUCTURED_GRID`` with points, cells (0-based
  node ids, the 10-node tetrahedron with the two last mid-edge nodes swapped into VTK
  order), cell types, then per-element ``SCALARS`` / ``VECTORS`` after a ``CELL_DATA``
  header, or per-node ones after ``POINT_DATA``.
* ``read_vtk`` -- readVTKPolyX (fileIO/VTK.f90:3-81): points, cells and cell types of
  triangles, quadrilaterals, tetrahedra and hexahedra.

``write_gmsh`` (format 2.2 or 4.1) has no reference counterpart; it writes the meshes this
package generates so that a case directory can be made from them.

Element shape codes are the reference's (polyGrid.f90:10-21).
"""
from __future__ import annotations

from pathlib import Path

import numpy as np

from .mesh import Mesh

TRI, QUAD, TRI6, TET, HEX, TET10 = 10, 11, 110, 20, 21, 120
NODES = {TRI: 3, QUAD: 4, TRI6: 6, TET: 4, HEX: 8, TET10: 10}
CELL_SHAPES = (TET, HEX, TET10)
# Gmsh element type -> shape code (the types readGMSHPolyGrid translates)
GMSH_TO_SHAPE = {2: TRI, 3: QUAD, 9: TRI6, 4: TET, 5: HEX, 11: TET10}
SHAPE_TO_GMSH = {v: k for k, v in GMSH_TO_SHAPE.items()}
# VTK cell type <-> shape code (transShape in VTK.f90)
VTK_OF = {TRI: 5, QUAD: 9, TRI6: 22, TET: 10, HEX: 12, TET10: 24}
SHAPE_OF_VTK = {5: TRI, 9: QUAD, 10: TET, 12: HEX}
# the 10-node tetrahedron lists its last two mid-edge nodes in the other order in VTK
TET10_TO_VTK = np.array([0, 1, 2, 3, 4, 5, 6, 7, 9, 8])


class MeshFileError(ValueError):
    pass


def _tokens(lines, i):
    return lines[i].split()


def _assemble(pN, shapes, conn, gids) -> Mesh:
    """Mesh from parallel lists of kept elements (1-based node ids)."""
    if not shapes:
        raise MeshFileError("no supported elements in the file")
    nE = len(shapes)
    m = max(NODES[s] for s in shapes)
    iNE = np.zeros((nE, m), np.int32)
    for k, c in enumerate(conn):
        iNE[k, :len(c)] = c
    sE = np.asarray(shapes, np.int32)
    nNE = np.asarray([NODES[s] for s in shapes], np.int32)
    gid = np.asarray(gids, np.int32)
    nC = int(np.isin(sE, CELL_SHAPES).sum())
    return Mesh(pN=np.asarray(pN, np.float64), sE=sE, nNE=nNE, iNE=iNE, gid=gid, nC=nC)


def read_gmsh(path) -> Mesh:
    """Read a Gmsh ASCII mesh (format 2.2 or 4.1) into a Mesh (elements in file order)."""
    lines = Path(path).read_text().splitlines()
    n = len(lines)
    version = None
    i = 0
    node_index = {}
    pts = []
    shapes, conn, gids = [], [], []
    have_nodes = False
    while i < n:
        head = lines[i].strip()
        if head == "$MeshFormat":
            fields = _tokens(lines, i + 1)
            version = int(float(fields[0]))
            if len(fields) > 1 and fields[1] != "0":
                raise MeshFileError("binary Gmsh files are not supported")
            i += 2
        elif head == "$Nodes":
            if version is None:
                raise MeshFileError("$Nodes before $MeshFormat")
            if version == 2:
                nn = int(lines[i + 1])
                for k in range(nn):
                    f = lines[i + 2 + k].split()
                    node_index[int(f[0])] = len(pts) + 1
                    pts.append((float(f[1]), float(f[2]), float(f[3])))
                i += 2 + nn
            elif version == 4:
                nblocks = int(_tokens(lines, i + 1)[0])
                j = i + 2
                for _ in range(nblocks):
                    f = _tokens(lines, j)
                    cnt = int(f[3])
                    if int(f[2]) != 0:
                        raise MeshFileError("parametric node blocks are not supported")
                    tags = [int(lines[j + 1 + k]) for k in range(cnt)]
                    for k in range(cnt):
                        c = lines[j + 1 + cnt + k].split()
                        node_index[tags[k]] = len(pts) + 1
                        pts.append((float(c[0]), float(c[1]), float(c[2])))
                    j += 1 + 2 * cnt
                i = j
            else:
                raise MeshFileError(f"Gmsh format {version} is not supported (2.2 or 4.1)")
            have_nodes = True
        elif head == "$Elements":
            if not have_nodes:
                raise MeshFileError("reading elements before nodes")
            if version == 2:
                ne = int(lines[i + 1])
                for k in range(ne):
                    f = lines[i + 2 + k].split()
                    etype, ntag = int(f[1]), int(f[2])
                    shape = GMSH_TO_SHAPE.get(etype)
                    if shape is None:
                        continue
                    tags = f[3:3 + ntag]
                    nodes = f[3 + ntag:3 + ntag + NODES[shape]]
                    shapes.append(shape)
                    conn.append([node_index[int(x)] for x in nodes])
                    gids.append(int(tags[1]) if ntag >= 2 else (int(tags[0]) if ntag else 0))
                i += 2 + ne
            else:
                nblocks = int(_tokens(lines, i + 1)[0])
                j = i + 2
                for _ in range(nblocks):
                    f = _tokens(lines, j)
                    etag, etype, cnt = int(f[1]), int(f[2]), int(f[3])
                    shape = GMSH_TO_SHAPE.get(etype)
                    if shape is not None:
                        for k in range(cnt):
                            c = lines[j + 1 + k].split()
                            shapes.append(shape)
                            conn.append([node_index[int(x)] for x in c[1:1 + NODES[shape]]])
                            gids.append(etag)
                    j += 1 + cnt
                i = j
            break  # the reference stops reading after the element section
        else:
            i += 1
    if not have_nodes:
        raise MeshFileError("no $Nodes section")
    if not shapes:
        raise MeshFileError("element data not read")
    return _assemble(pts, shapes, conn, gids)


def write_gmsh(path, mesh: Mesh, version: float = 2.2) -> None:
    """Write a Mesh as a Gmsh ASCII file (format 2.2 or 4.1); group ids become the
    geometric entity tags (and physical tags in 2.2)."""
    nN, nE = mesh.nN, mesh.nE
    out = ["$MeshFormat", f"{'2.2' if version < 4 else '4.1'} 0 8", "$EndMeshFormat"]
    if version < 4:
        out.append("$Nodes")
        out.append(str(nN))
        out += [f"{k + 1} {x!r} {y!r} {z!r}" for k, (x, y, z) in enumerate(mesh.pN.tolist())]
        out.append("$EndNodes")
        out.append("$Elements")
        out.append(str(nE))
        for e in range(nE):
            s = int(mesh.sE[e])
            nodes = " ".join(str(int(v)) for v in mesh.iNE[e, :NODES[s]])
            g = int(mesh.gid[e])
            out.append(f"{e + 1} {SHAPE_TO_GMSH[s]} 2 {g} {g} {nodes}")
        out.append("$EndElements")
    else:
        dim = {TRI: 2, QUAD: 2, TRI6: 2, TET: 3, HEX: 3, TET10: 3}
        out.append("$Nodes")
        out.append(f"1 {nN} 1 {nN}")
        out.append(f"3 1 0 {nN}")
        out += [str(k + 1) for k in range(nN)]
        out += [f"{x!r} {y!r} {z!r}" for (x, y, z) in mesh.pN.tolist()]
        out.append("$EndNodes")
        blocks = {}
        for e in range(nE):
            blocks.setdefault((dim[int(mesh.sE[e])], int(mesh.gid[e]), int(mesh.sE[e])), []).append(e)
        out.append("$Elements")
        out.append(f"{len(blocks)} {nE} 1 {nE}")
        for (d, g, s), els in blocks.items():
            out.append(f"{d} {g} {SHAPE_TO_GMSH[s]} {len(els)}")
            for e in els:
                out.append(f"{e + 1} " + " ".join(str(int(v)) for v in mesh.iNE[e, :NODES[s]]))
        out.append("$EndElements")
    Path(path).write_text("\n".join(out) + "\n")


def write_vtk(path, mesh: Mesh, cell_data: dict | None = None, point_data: dict | None = None,
              title: str = "Generated by fosolvers_gb300") -> None:
    """Legacy ASCII VTK of the mesh with per-element (CELL_DATA, nE entries) and per-node
    (POINT_DATA) fields; arrays of shape (n,) become SCALARS, (n, 3) VECTORS."""
    nN, nE = mesh.nN, mesh.nE
    out = ["# vtk DataFile Version 3.0", title, "ASCII", "", "DATASET UNSTRUCTURED_GRID",
           f"POINTS {nN} double"]
    out += [f"{x!r} {y!r} {z!r}" for (x, y, z) in mesh.pN.tolist()]
    out.append("")
    out.append(f"CELLS {nE} {nE + int(mesh.nNE.sum())}")
    for e in range(nE):
        s, k = int(mesh.sE[e]), int(mesh.nNE[e])
        ids = mesh.iNE[e, :k] - 1
        if s == TET10:
            ids = ids[TET10_TO_VTK]
        out.append(f"{k} " + " ".join(str(int(v)) for v in ids))
    out.append("")
    out.append(f"CELL_TYPES {nE}")
    out += [str(VTK_OF.get(int(s), 0)) for s in mesh.sE]

    def fields(data, n):
        for key, a in data.items():
            a = np.asarray(a, np.float64)
            if a.shape[0] != n:
                raise ValueError(f"field {key!r} has {a.shape[0]} entries, expected {n}")
            out.append("")
            if a.ndim == 1:
                out.append(f"SCALARS {key} double")
                out.append("LOOKUP_TABLE default")
                out.extend(repr(float(x)) for x in a)
            elif a.ndim == 2 and a.shape[1] == 3:
                out.append(f"VECTORS {key} double")
                out.extend(f"{x!r} {y!r} {z!r}" for (x, y, z) in a.tolist())
            else:
                raise ValueError(f"field {key!r}: shape {a.shape} is neither (n,) nor (n, 3)")

    if cell_data:
        out.append("")
        out.append(f"CELL_DATA {nE}")
        fields(cell_data, nE)
    if point_data:
        out.append("")
        out.append(f"POINT_DATA {nN}")
        fields(point_data, nN)
    Path(path).write_text("\n".join(out) + "\n")


def read_vtk(path):
    """Points, cells and cell types of a legacy ASCII VTK unstructured grid as a Mesh
    (group ids 0), plus the CELL_DATA / POINT_DATA fields it carries."""
    toks = Path(path).read_text().split()
    i, n = 0, len(toks)
    pts = conn = types = None
    data = {"cell": {}, "point": {}}
    where = None
    while i < n:
        t = toks[i]
        if t == "POINTS":
            nn = int(toks[i + 1])
            pts = np.array(toks[i + 3:i + 3 + 3 * nn], np.float64).reshape(nn, 3)
            i += 3 + 3 * nn
        elif t == "CELLS":
            m, size = int(toks[i + 1]), int(toks[i + 2])
            flat = np.array(toks[i + 3:i + 3 + size], np.int64)
            conn, j = [], 0
            for _ in range(m):
                k = int(flat[j])
                conn.append(flat[j + 1:j + 1 + k] + 1)
                j += k + 1
            i += 3 + size
        elif t == "CELL_TYPES":
            m = int(toks[i + 1])
            types = [int(x) for x in toks[i + 2:i + 2 + m]]
            i += 2 + m
        elif t in ("CELL_DATA", "POINT_DATA"):
            where = "cell" if t == "CELL_DATA" else "point"
            cnt = int(toks[i + 1])
            i += 2
        elif t == "SCALARS":
            key = toks[i + 1]
            j = i + 3
            if toks[j] == "LOOKUP_TABLE":
                j += 2
            data[where][key] = np.array(toks[j:j + cnt], np.float64)
            i = j + cnt
        elif t == "VECTORS":
            key = toks[i + 1]
            data[where][key] = np.array(toks[i + 3:i + 3 + 3 * cnt], np.float64).reshape(cnt, 3)
            i += 3 + 3 * cnt
        else:
            i += 1
    if pts is None or conn is None or types is None:
        raise MeshFileError("POINTS, CELLS and CELL_TYPES are required")
    shapes, keep = [], []
    for k, t in enumerate(types):
        s = SHAPE_OF_VTK.get(t)
        if s is not None:
            shapes.append(s)
            keep.append(conn[k])
    mesh = _assemble(pts, shapes, keep, [0] * len(shapes))
    return mesh, data
