"""Build recipe of the native libraries (in-tree, sm_103a only).

    python -m sdem_gb300.build

libsdem_gpu.so (the particle step, include/sdem_gpu.h) and
libsdem_surrogate.so (the learned surrogate, include/sdem_surrogate.h), one
translation unit each, compiled in parallel with -fmad=false: the force law
and the integrator must round exactly as the reference's Fortran (no FMA
contraction), and the surrogate's graph features as its numpy statement.
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
SG_SRC = os.path.join(HERE, "csrc", "surrogate.cu")
SG_DEPS = [SG_SRC, os.path.join(ROOT, "include", "sdem_surrogate.h")]
SG_LIB = os.path.join(HERE, "libsdem_surrogate.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-fmad=false", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-shared",
         "-Xcompiler", "-fno-strict-aliasing", "-Xcompiler", "-ffp-contract=off"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the sm_103a library cannot be built")


def up_to_date(lib: str = LIB, deps=None) -> bool:
    deps = DEPS if deps is None else deps
    if not os.path.exists(lib):
        return False
    t = os.path.getmtime(lib)
    return all(os.path.getmtime(p) <= t for p in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    """Compiles libsdem_gpu.so and libsdem_surrogate.so next to this file
    (the stale ones, in parallel); returns the path of libsdem_gpu.so."""
    jobs = []
    for src, deps, lib in ((SRC, DEPS, LIB), (SG_SRC, SG_DEPS, SG_LIB)):
        if not force and up_to_date(lib, deps):
            continue
        tmp = f"{lib}.{os.getpid()}.tmp"
        cmd = [nvcc(), *ARCH, *FLAGS, "-o", tmp, src, "-lcudart"]
        if verbose:
            print(" ".join(cmd), flush=True)
        jobs.append((subprocess.Popen(cmd), cmd, tmp, lib))
    failed = None
    for proc, cmd, tmp, lib in jobs:
        if proc.wait() != 0:
            failed = failed or subprocess.CalledProcessError(proc.returncode, cmd)
        else:
            os.replace(tmp, lib)
    if failed:
        raise failed
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
