"""Build the CPU oracle (test infrastructure only).

The oracle is a plain-C restatement of the reference arithmetic (fos_oracle.c).  Two builds
of the same source:

* ``_build/liboracle.so`` -- the checker: ``gcc -O3 -std=c11 -fopenmp`` with no ISA flags,
  loaded by tests/ and __graft_entry__.smoke();
* ``_build/liboracle_tuned.so`` -- the timed CPU baseline: the same flags plus the host's
  own instruction set (``-march=native`` on x86-64, ``-mcpu=native`` on AArch64), the way
  the reference itself is built (CMakeLists.txt:7-8 uses ``-Ofast -march=native
  -fopenmp``; fast-math is left out so results stay IEEE).  Both builds use
  ``-ffp-contract=off`` (ISO C), so no multiply-add is fused differently by the two: the
  tuned library computes bit-identical results (tests/test_oracle_kat.py checks that), and
  it is used only for timing on the machine that built it.
"""
from __future__ import annotations

import platform
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"
LIB_TUNED = HERE / "_build" / "liboracle_tuned.so"
BASE_FLAGS = ["-O3", "-std=c11", "-ffp-contract=off", "-fopenmp", "-shared", "-fPIC"]


def isa_flags() -> list[str]:
    """The host-ISA flag of the tuned build (empty where the machine is neither)."""
    m = platform.machine().lower()
    if m in ("x86_64", "amd64"):
        return ["-march=native"]
    if m in ("aarch64", "arm64"):
        return ["-mcpu=native"]
    return []


def _compile(out: Path, extra: list[str], force: bool) -> Path:
    src = HERE / "fos_oracle.c"
    hdr = HERE / "fos_oracle.h"
    newest = max(src.stat().st_mtime, hdr.stat().st_mtime, Path(__file__).stat().st_mtime)
    if out.exists() and not force and out.stat().st_mtime >= newest:
        return out
    out.parent.mkdir(exist_ok=True)
    cc = shutil.which("gcc") or "cc"
    tmp = out.with_suffix(".so.tmp")
    cmd = [cc, *BASE_FLAGS, *extra, str(src), "-o", str(tmp), "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed ({' '.join(cmd)}):\n{r.stdout}\n{r.stderr}")
    tmp.replace(out)
    return out


def build(force: bool = False) -> Path:
    """The checker library (portable flags)."""
    return _compile(LIB, [], force)


def build_tuned(force: bool = False) -> Path:
    """The timing library (host ISA); falls back to the checker if the flag is refused."""
    flags = isa_flags()
    if not flags:
        return build(force)
    try:
        return _compile(LIB_TUNED, flags, force)
    except RuntimeError:
        return build(force)


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
    print(build_tuned(force="--force" in sys.argv))
