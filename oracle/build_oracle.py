"""ORACLE (test infrastructure only): compile oracle/csr_omp.c into oracle/_lib/libcsr_omp.so (gcc,
OpenMP, no FMA contraction). Called by __graft_entry__.build(); the product never loads it."""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "csr_omp.c"
LIB = HERE / "_lib" / "libcsr_omp.so"


def build(force: bool = False) -> Path:
    if LIB.exists() and not force and LIB.stat().st_mtime >= SRC.stat().st_mtime:
        return LIB
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        raise RuntimeError("no C compiler for the oracle's threaded sparse product")
    LIB.parent.mkdir(exist_ok=True)
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [cc, "-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", str(SRC), "-o", str(tmp)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle C build failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
