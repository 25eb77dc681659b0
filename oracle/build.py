"""Build the CPU oracle (test infrastructure only) into oracle/_build/liboracle.so.

The oracle is a plain-C restatement of the reference arithmetic (fos_oracle.c);
it is compiled with gcc -O3 -fopenmp (no -march flags, so x86 and Arm builds
agree) and loaded by tests/, __graft_entry__.smoke() and bench.py's CPU leg.
"""
from __future__ import annotations

import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"


def build(force: bool = False) -> Path:
    src = HERE / "fos_oracle.c"
    hdr = HERE / "fos_oracle.h"
    if LIB.exists() and not force and LIB.stat().st_mtime >= max(src.stat().st_mtime,
                                                                  hdr.stat().st_mtime,
                                                                  Path(__file__).stat().st_mtime):
        return LIB
    LIB.parent.mkdir(exist_ok=True)
    cc = shutil.which("gcc") or "cc"
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [cc, "-O3", "-std=c11", "-fopenmp", "-shared", "-fPIC", str(src), "-o", str(tmp), "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    tmp.replace(LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
