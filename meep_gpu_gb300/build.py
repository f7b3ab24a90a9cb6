"""Build recipe of the CUDA library ``libmeepgb.so`` (sm_103a, in-tree).

Two translation units (the stepping library and the tensor-core DFT contraction)
compiled by nvcc straight into a shared object next to this file. ``-fmad=false`` is part of the numerics contract: no multiply-add may be
contracted, so every float32 word matches the reference's separately rounded
operations.
"""

from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

PACKAGE = Path(__file__).resolve().parent
ROOT = PACKAGE.parent
SOURCES = [PACKAGE / "csrc" / "meepgb.cu", PACKAGE / "csrc" / "dft_tc.cu"]
HEADERS = [PACKAGE / "csrc" / "dft_tc.cuh"]
LIBRARY = PACKAGE / "libmeepgb.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    found = shutil.which("nvcc")
    if found:
        return found
    candidate = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(candidate):
        return candidate
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libmeepgb.so")


def stale() -> bool:
    if not LIBRARY.exists():
        return True
    built = LIBRARY.stat().st_mtime
    inputs = SOURCES + HEADERS + [ROOT / "include" / "meepgb.h", Path(__file__)]
    return any(p.stat().st_mtime > built for p in inputs)


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile ``libmeepgb.so`` unless it is newer than every input."""
    if not force and not stale():
        return LIBRARY
    cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-fmad=false", "-std=c++17",
           "-Xcompiler", "-fPIC", "-shared", "-I", str(ROOT / "include"),
           "-o", str(LIBRARY) + ".tmp", *map(str, SOURCES)]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
        print(" ".join(cmd), file=sys.stderr)
    subprocess.run(cmd, check=True)
    os.replace(str(LIBRARY) + ".tmp", LIBRARY)
    return LIBRARY


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIBRARY)
