"""Builds the CPU oracle (oracle.c) into oracle/_build/liboracle.so with gcc.

Test infrastructure only: tests/, __graft_entry__.smoke() and bench.py's CPU
baseline load it; the library never does. -ffp-contract=off keeps every float
product rounded before it is added (GCC contracts to FMA by default in GNU C
mode), which is the evaluation order the oracle's restatement fixes. OpenMP is
used when the compiler has it; results do not depend on the thread count.

The reference itself (TypeScript + WGSL run by a browser's WebGPU) has no
CPU-buildable sources, so there is no oracle/_ref build.
"""

from __future__ import annotations

import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
SOURCE = HERE / "oracle.c"
BUILD = HERE / "_build"
LIBRARY = BUILD / "liboracle.so"

BASE = ["-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-std=c11"]


def build(force: bool = False) -> Path:
    if not force and LIBRARY.exists() and LIBRARY.stat().st_mtime >= max(SOURCE.stat().st_mtime, Path(__file__).stat().st_mtime):
        return LIBRARY
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        raise RuntimeError("no C compiler found for the oracle")
    BUILD.mkdir(parents=True, exist_ok=True)
    tmp = LIBRARY.with_suffix(".so.tmp")
    for openmp in (["-fopenmp"], []):
        proc = subprocess.run([cc, *BASE, *openmp, str(SOURCE), "-o", str(tmp), "-lm"], capture_output=True, text=True)
        if proc.returncode == 0:
            break
    else:
        raise RuntimeError(f"oracle build failed:\n{proc.stderr}")
    tmp.replace(LIBRARY)
    return LIBRARY


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
