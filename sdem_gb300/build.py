"""Build recipe of the native library libsdem_gpu.so (in-tree, sm_103a only).

    python -m sdem_gb300.build

One translation unit, compiled with -fmad=false: the force law and the
integrator must round exactly as the reference's Fortran (no FMA contraction).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(HERE, "csrc", "sdem_gpu.cu")
DEPS = [SRC, os.path.join(HERE, "csrc", "dem_device.cuh"), os.path.join(HERE, "csrc", "fp64_int.cuh"),
        os.path.join(ROOT, "include", "sdem_gpu.h")]
LIB = os.path.join(HERE, "libsdem_gpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-fmad=false", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-shared",
         "-Xcompiler", "-fno-strict-aliasing", "-Xcompiler", "-ffp-contract=off"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the sm_103a library cannot be built")


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(p) <= t for p in DEPS)


def build(force: bool = False, verbose: bool = False) -> str:
    """Compiles libsdem_gpu.so next to this file; returns its path."""
    if not force and up_to_date():
        return LIB
    tmp = f"{LIB}.{os.getpid()}.tmp"
    cmd = [nvcc(), *ARCH, *FLAGS, "-o", tmp, SRC, "-lcudart"]
    if verbose:
        print(" ".join(cmd), flush=True)
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
