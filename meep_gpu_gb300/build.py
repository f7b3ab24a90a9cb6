"""Build recipe of the CUDA library ``libmeepgb.so`` (sm_103a, in-tree).

Four translation units compiled by nvcc in parallel and linked into a shared object next
to this file: the stepping library, the tensor-core DFT contraction, the wavefront step
kernel and the reduced-dimension step kernels. The wavefront unit caches every global load in L2 only (``-dlcm=cg``): its
persistent CTAs read words other SMs rewrote during the same launch, and L1 is not
coherent with them. ``-fmad=false`` is part of the numerics contract: no multiply-add may
be contracted, so every float32 word matches the reference's separately rounded
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
CSRC = PACKAGE / "csrc"
SOURCES = [CSRC / "meepgb.cu", CSRC / "dft_tc.cu", CSRC / "wave.cu", CSRC / "reduced.cu"]
HEADERS = [CSRC / "dft_tc.cuh", CSRC / "step_device.cuh", CSRC / "wave.cuh", CSRC / "reduced.cuh"]
LIBRARY = PACKAGE / "libmeepgb.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# extra flags per translation unit
UNIT_FLAGS = {"wave.cu": ["-Xptxas", "-dlcm=cg"]}


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
    common = [*ARCH, "-O3", "-lineinfo", "-fmad=false", "-std=c++17", "-Xcompiler", "-fPIC",
              "-I", str(ROOT / "include")]
    if verbose:
        common.append("-Xptxas=-v")
    objects, procs = [], []
    for source in SOURCES:
        obj = PACKAGE / (source.stem + ".o")
        cmd = [nvcc(), *common, *UNIT_FLAGS.get(source.name, []), "-c", str(source), "-o", str(obj) + ".tmp"]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        procs.append((subprocess.Popen(cmd), cmd))
        objects.append(obj)
    failed = [cmd for proc, cmd in procs if proc.wait() != 0]
    if failed:
        raise subprocess.CalledProcessError(1, failed[0])
    for obj in objects:
        os.replace(str(obj) + ".tmp", obj)
    link = [nvcc(), *ARCH, "-shared", "-Xcompiler", "-fPIC", "-o", str(LIBRARY) + ".tmp", *map(str, objects)]
    subprocess.run(link, check=True)
    os.replace(str(LIBRARY) + ".tmp", LIBRARY)
    for obj in objects:
        obj.unlink()
    return LIBRARY


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIBRARY)
