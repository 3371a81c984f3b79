"""Build recipe of the CPU oracle (test infrastructure only).

    python oracle/build.py

Compiles sdem_oracle.c with -O2 -ffp-contract=off (no FMA contraction, no
fast-math) into oracle/libsdem_oracle.so.  Portable C11; builds the same on the
x86-64 development host and the aarch64 GPU host.
"""
from __future__ import annotations

import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "sdem_oracle.c")
HDR = os.path.join(os.path.dirname(HERE), "include", "sdem_gpu.h")
LIB = os.path.join(HERE, "libsdem_oracle.so")
FLAGS = ["-O2", "-std=c11", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared"]


def _cc_version(cc: str) -> str:
    try:
        return subprocess.run([cc, "--version"], capture_output=True, text=True, check=True).stdout
    except (OSError, subprocess.CalledProcessError):
        return "unknown"


def build(force: bool = False, verbose: bool = False) -> str:
    """Compiles the oracle when its content stamp (sources, flags, compiler
    version) differs from the one recorded beside the library."""
    cc = os.environ.get("CC") or shutil.which("gcc") or "cc"
    h = hashlib.sha256()
    for p in (SRC, HDR):
        with open(p, "rb") as f:
            h.update(hashlib.sha256(f.read()).digest())
    h.update("\0".join(FLAGS).encode())
    h.update(_cc_version(cc).encode())
    stamp = h.hexdigest()
    if not force and os.path.exists(LIB):
        try:
            with open(LIB + ".stamp") as f:
                if f.read().strip() == stamp:
                    return LIB
        except OSError:
            pass
    tmp = f"{LIB}.{os.getpid()}.tmp"
    cmd = [cc, *FLAGS, "-o", tmp, SRC, "-lm"]
    if verbose:
        print(" ".join(cmd), flush=True)
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    with open(LIB + ".stamp", "w") as f:
        f.write(stamp + "\n")
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
