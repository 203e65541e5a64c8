"""Builds libdiorama_gb300.so for sm_103a with nvcc, in-tree, into diorama_gb300/_build/.

Each .cu file (and each host-only .cpp file) compiles to an object in parallel,
then nvcc links the shared library. The renderer and the loss are compiled with --fmad=false: their float
expressions are evaluated exactly as written (fused multiply-adds only where the
source spells out fmaf), which is what makes the forward pass bit-identical to
the CPU oracle's restatement of the reference.

    python -m diorama_gb300.build          # build if any source is newer
    python -m diorama_gb300.build --force  # rebuild everything
"""

from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PACKAGE = Path(__file__).resolve().parent
SOURCES = PACKAGE / "csrc"
BUILD = PACKAGE / "_build"
LIBRARY = BUILD / "libdiorama_gb300.so"
HEADER = PACKAGE.parent / "include" / "diorama_gb300.h"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-DNDEBUG", "--expt-relaxed-constexpr"]
# Files whose float expressions must round exactly as written.
EXACT = {"dg_render.cu", "dg_loss.cu", "dg_init.cu"}
# The backward passes and Adam agree with the oracle to rounding (1e-4 of each
# gradient group's largest), not bit for bit: their divisions and square roots
# may take the approximate forms (a reciprocal and a multiply).
APPROXIMATE = {"dg_render_bwd.cu": ["-prec-div=false", "-prec-sqrt=false"]}


def nvcc() -> str:
    found = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(found).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build diorama_gb300")
    return found


def _compile(source: Path, extra: list[str]) -> Path:
    obj = BUILD / (source.stem + ".o")
    flags = ARCH + COMMON + extra
    if source.name in EXACT:
        flags = flags + ["--fmad=false"]
    flags = flags + APPROXIMATE.get(source.name, [])
    cmd = [nvcc(), *flags, "-c", str(source), "-o", str(obj)]
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"nvcc failed on {source.name}:\n{proc.stdout}\n{proc.stderr}")
    return obj


def _stale(target: Path, inputs: list[Path]) -> bool:
    if not target.exists():
        return True
    built = target.stat().st_mtime
    return any(p.stat().st_mtime > built for p in inputs)


def build(force: bool = False, verbose: bool = False, extra: list[str] | None = None) -> Path:
    """Compiles the library if needed and returns its path."""
    extra = list(extra or [])
    sources = sorted(SOURCES.glob("*.cu")) + sorted(SOURCES.glob("*.cpp"))
    headers = sorted(SOURCES.glob("*.cuh")) + sorted(SOURCES.glob("*.h")) + [HEADER]
    if not force and not _stale(LIBRARY, sources + headers + [Path(__file__)]):
        return LIBRARY
    BUILD.mkdir(parents=True, exist_ok=True)
    with ThreadPoolExecutor(max_workers=max(1, min(len(sources), os.cpu_count() or 4))) as pool:
        objects = list(pool.map(lambda s: _compile(s, extra), sources))
    tmp = LIBRARY.with_suffix(".so.tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objects), "-lcudart"]
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"nvcc link failed:\n{proc.stdout}\n{proc.stderr}")
    os.replace(tmp, LIBRARY)
    if verbose:
        print(f"built {LIBRARY}")
    return LIBRARY


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
