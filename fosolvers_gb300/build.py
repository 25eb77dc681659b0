"""Build libfosgpu.so (the CUDA kernels and the C ABI) in-tree for sm_103a.

Every translation unit is compiled in parallel with nvcc for one target
(-gencode arch=compute_103a,code=sm_103a) and linked into
fosolvers_gb300/libfosgpu.so next to this file.  No CMake, no torch extension
machinery: the library has a plain C ABI (include/fosgpu.h).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
BUILD = HERE / "_build"
LIB = HERE / "libfosgpu.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["fos_ctx.cu", "fos_residual.cu", "fos_jacobian.cu", "fos_bdf.cu", "fos_gnn.cu",
           "fos_ilut.cu", "fos_grid.cpp"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libfosgpu.so")


# Host code is compiled without multiply-add contraction (g++ contracts by default on AArch64
# but not on x86-64), so the host-side set-up -- face geometry, closure vectors, renumbering --
# gives the same numbers on both machines.  Device code keeps nvcc's default.
HOST_FLAGS = ["-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off"]


def _compile(src: Path, obj: Path, extra: list[str]) -> None:
    cmd = [_nvcc(), "-std=c++17", "-O3", "-lineinfo", *ARCH, *HOST_FLAGS,
           "-I", str(HERE.parent / "include"), *extra, "-c", str(src), "-o", str(obj)]
    if src.suffix == ".cpp":
        cmd = [_nvcc(), "-std=c++17", "-O3", *HOST_FLAGS,
               "-I", str(HERE.parent / "include"), "-x", "c++", "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src.name}:\n{r.stdout}\n{r.stderr}")


def build(force: bool = False, verbose: bool = False, extra: list[str] | None = None) -> Path:
    """Compile (if stale) and link libfosgpu.so; returns its path."""
    srcs = [CSRC / s for s in SOURCES if (CSRC / s).exists()]
    deps = srcs + list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + \
        [HERE.parent / "include" / "fosgpu.h", Path(__file__)]
    if LIB.exists() and not force:
        t = LIB.stat().st_mtime
        if all(p.stat().st_mtime <= t for p in deps):
            return LIB
    BUILD.mkdir(exist_ok=True)
    objs = [BUILD / (s.stem + ".o") for s in srcs]
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        futs = [ex.submit(_compile, s, o, extra or []) for s, o in zip(srcs, objs)]
        for f in futs:
            f.result()
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [_nvcc(), "-shared", *ARCH, "-o", str(tmp), *map(str, objs), "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    tmp.replace(LIB)
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
