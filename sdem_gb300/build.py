"""Build recipe of the native libraries (in-tree, sm_103a only).

    python -m sdem_gb300.build

libsdem_gpu.so (the particle step, include/sdem_gpu.h) and
libsdem_surrogate.so (the learned surrogate, include/sdem_surrogate.h), one
translation unit each, compiled in parallel with -fmad=false: the force law
and the integrator must round exactly as the reference's Fortran (no FMA
contraction), and the surrogate's graph features as its numpy statement.
libsdem_bedgen.so (host C: the seeded random sequential placement of the
synthetic beds) is compiled with gcc beside them.
"""
from __future__ import annotations

import hashlib
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
BG_SRC = os.path.join(HERE, "csrc", "bedgen.c")
BG_LIB = os.path.join(HERE, "libsdem_bedgen.so")
BG_FLAGS = ["-O2", "-std=c11", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared"]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-fmad=false", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-shared",
         "-Xcompiler", "-fno-strict-aliasing", "-Xcompiler", "-ffp-contract=off"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the sm_103a library cannot be built")


def _nvcc_version(exe: str) -> str:
    try:
        return subprocess.run([exe, "--version"], capture_output=True, text=True, check=True).stdout
    except (OSError, subprocess.CalledProcessError):
        return "unknown"


def stamp_of(deps, cmd_flags, compiler_version: str) -> str:
    """Content key of one library: its sources and headers, the flags and the
    compiler's version string.  A library whose stamp file differs (or is
    missing) is rebuilt, whatever the files' modification times say."""
    h = hashlib.sha256()
    for p in deps:
        h.update(os.path.basename(p).encode())
        with open(p, "rb") as f:
            h.update(hashlib.sha256(f.read()).digest())
    h.update("\0".join(cmd_flags).encode())
    h.update(compiler_version.encode())
    return h.hexdigest()


def up_to_date(lib: str, stamp: str) -> bool:
    try:
        with open(lib + ".stamp") as f:
            return os.path.exists(lib) and f.read().strip() == stamp
    except OSError:
        return False


def _cc() -> str:
    return os.environ.get("CC") or shutil.which("gcc") or "cc"


def build(force: bool = False, verbose: bool = False) -> str:
    """Compiles libsdem_gpu.so, libsdem_surrogate.so and libsdem_bedgen.so
    next to this file (those whose content stamp changed, in parallel);
    returns the path of libsdem_gpu.so."""
    exe = nvcc()
    version = _nvcc_version(exe)
    cc = _cc()
    specs = [(SRC, DEPS, LIB, [exe, *ARCH, *FLAGS], ["-lcudart"], ARCH + FLAGS, version),
             (SG_SRC, SG_DEPS, SG_LIB, [exe, *ARCH, *FLAGS], ["-lcudart"], ARCH + FLAGS, version),
             (BG_SRC, [BG_SRC], BG_LIB, [cc, *BG_FLAGS], ["-lm"], BG_FLAGS, _nvcc_version(cc))]
    jobs = []
    for src, deps, lib, head, tail, flags, ver in specs:
        stamp = stamp_of(deps, flags, ver)
        if not force and up_to_date(lib, stamp):
            continue
        tmp = f"{lib}.{os.getpid()}.tmp"
        cmd = [*head, "-o", tmp, src, *tail]
        if verbose:
            print(" ".join(cmd), flush=True)
        jobs.append((subprocess.Popen(cmd), cmd, tmp, lib, stamp))
    failed = None
    for proc, cmd, tmp, lib, stamp in jobs:
        if proc.wait() != 0:
            failed = failed or subprocess.CalledProcessError(proc.returncode, cmd)
        else:
            os.replace(tmp, lib)
            with open(lib + ".stamp", "w") as f:
                f.write(stamp + "\n")
    if failed:
        raise failed
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
