"""Build the in-tree CUDA library ``libm3sph.so`` for sm_103a with nvcc (no cmake).

Each translation unit is compiled in parallel, then linked into one shared library next to
this file. The library exports only the C ABI declared in ``include/m3sph.h``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libm3sph.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-fvisibility=hidden"]


def _nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the m3sph library must be compiled with the CUDA toolkit")
    return cand


def sources():
    return sorted(CSRC.glob("*.cu"))


def _compile(src: Path, extra=()):
    obj = BUILD / (src.stem + ".o")
    cmd = [_nvcc(), *ARCH, *NVCC_FLAGS, *extra, "-I", str(ROOT / "include"), "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stderr}")
    return obj, r.stderr


def build(force: bool = False, verbose: bool = False, extra=()) -> Path:
    """Compile every .cu under csrc/ and link libm3sph.so; returns the library path."""
    srcs = sources()
    deps = srcs + list(CSRC.glob("*.cuh")) + [ROOT / "include" / "m3sph.h"]
    if LIB.exists() and not force:
        lib_t = LIB.stat().st_mtime
        if all(p.stat().st_mtime <= lib_t for p in deps):
            return LIB
    BUILD.mkdir(exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 4))) as ex:
        results = list(ex.map(lambda s: _compile(s, extra), srcs))
    if verbose:
        for _, err in results:
            if err:
                print(err)
    objs = [str(o) for o, _ in results]
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [_nvcc(), *ARCH, "-shared", "-o", str(tmp), *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose=True))
