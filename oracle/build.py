"""Build recipe of the CPU oracle (test infrastructure only).

    python oracle/build.py

Compiles sdem_oracle.c with -O2 -ffp-contract=off (no FMA contraction, no
fast-math) into oracle/libsdem_oracle.so.  Portable C11; builds the same on the
x86-64 development host and the aarch64 GPU host.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "sdem_oracle.c")
HDR = os.path.join(os.path.dirname(HERE), "include", "sdem_gpu.h")
LIB = os.path.join(HERE, "libsdem_oracle.so")
FLAGS = ["-O2", "-std=c11", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared"]


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and os.path.exists(LIB) and all(os.path.getmtime(p) <= os.path.getmtime(LIB) for p in (SRC, HDR)):
        return LIB
    cc = os.environ.get("CC") or shutil.which("gcc") or "cc"
    tmp = f"{LIB}.{os.getpid()}.tmp"
    cmd = [cc, *FLAGS, "-o", tmp, SRC, "-lm"]
    if verbose:
        print(" ".join(cmd), flush=True)
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
