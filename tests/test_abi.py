"""The C ABI: libfosgpu.so loads, exports every entry point include/fosgpu.h declares,
and rejects bad set-up arguments on the host before touching the device.  CPU only."""
import ctypes as C
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

from fosolvers_gb300 import _lib

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    txt = (ROOT / "include" / "fosgpu.h").read_text()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(fos_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol(fos_lib):
    syms = declared_symbols()
    assert len(syms) >= 20
    out = subprocess.run(["nm", "-D", "--defined-only", str(_lib.LIB_PATH)], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r" T (fos_\w+)", out))
    missing = [s for s in syms if s not in exported]
    assert not missing, missing
    for s in syms:
        assert hasattr(fos_lib, s)


def test_binding_covers_header(fos_lib):
    assert set(_lib.exported_symbols()) == set(declared_symbols())


def _create(**over):
    nC, nE, nPi, nPb = 2, 4, 1, 2
    args = dict(nC=nC, nE=nE, nPi=nPi, nPb=nPb,
                iEP=np.array([1, 2, 1, 3, 2, 4], np.int32), aP=np.ones(3), normP=np.tile([1.0, 0, 0], 3),
                v=np.ones(2), iBC=np.zeros(4, np.int32), nBC=0, bcT=None, bcP=None, maxP=0,
                gamm=1.4, r=1.0, base=1, flags=0)
    args.update(over)
    h = C.c_void_p()
    L = _lib.lib()
    rc = L.fos_ctx_create(C.byref(h), args["nC"], args["nE"], args["nPi"], args["nPb"],
                          _lib.iptr(args["iEP"]), _lib.dptr(args["aP"]), _lib.dptr(args["normP"]),
                          _lib.dptr(args["v"]), _lib.iptr(args["iBC"]), args["nBC"],
                          args["bcT"], args["bcP"], args["maxP"], args["gamm"], args["r"],
                          args["base"], args["flags"])
    return rc


@pytest.mark.parametrize("over,code", [
    (dict(iEP=np.array([1, 3, 1, 3, 2, 4], np.int32)), -2),   # interior pair to a facet slot
    (dict(iEP=np.array([1, 2, 1, 2, 2, 4], np.int32)), -2),   # boundary pair to a cell
    (dict(v=np.array([1.0, 0.0])), -2),                        # zero volume
    (dict(gamm=1.0), -1),
    (dict(base=2), -1),
    (dict(iBC=np.array([0, 0, 5, 0], np.int32)), -3),          # condition row out of range
])
def test_ctx_create_rejects_bad_input(fos_lib, over, code):
    assert _create(**over) == code
    assert _lib.last_error()


def test_ctx_create_rejects_udf_condition(fos_lib):
    bcT = np.array([110], np.int32)  # BC_IN_STATIC_UDF needs libmatheval
    rc = _create(nBC=1, bcT=_lib.iptr(bcT), bcP=_lib.dptr(np.zeros(5)), maxP=5,
                 iBC=np.array([0, 0, 1, 0], np.int32))
    assert rc == -3 and "UDF" in _lib.last_error()


def test_grid_build_rejects_bad_node_ids(fos_lib):
    h = C.c_void_p()
    pN = np.zeros(12)
    iNE = np.array([1, 2, 3, 9], np.int32)
    rc = fos_lib.fos_grid_build(C.byref(h), 4, _lib.dptr(pN), 1, 4, _lib.iptr(np.array([20], np.int32)),
                                _lib.iptr(np.array([4], np.int32)), _lib.iptr(iNE), None)
    assert rc < 0 and "range" in _lib.last_error()


STRUCTS = {"fos_bdf_opts": "BdfOpts", "fos_bdf_stats": "BdfStats",
           "fos_bdf_adapt_opts": "AdaptOpts", "fos_bdf_adapt_stats": "AdaptStats"}


def test_struct_layouts_match_header(tmp_path):
    """The ctypes mirrors of the option and statistics structs have the header's size and
    field offsets (a field added on one side only would shift every later field), checked
    against gcc's own layout of include/fosgpu.h."""
    import shutil
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "fosgpu.h"', 'int main(void) {']
    for cname, pyname in STRUCTS.items():
        st = getattr(_lib, pyname)
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in st._fields_:
            lines.append(f'  printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ['  return 0;', '}']
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-I", str(ROOT / "include"), str(src), "-o", str(exe)],
                   check=True, capture_output=True)
    got = {}
    for line in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n"):
        if line:
            a, b, v = line.split()
            got[a, b] = int(v)
    for cname, pyname in STRUCTS.items():
        st = getattr(_lib, pyname)
        assert got[cname, "size"] == C.sizeof(st), cname
        for fname, _ in st._fields_:
            assert got[cname, fname] == getattr(st, fname).offset, (cname, fname)
