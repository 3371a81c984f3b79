"""The reference's tracer output of marked particles (module Prtcl_DumpPrtcl,
src/DEM/Prtcl_DumpPrtcl.f90), for a caller that drives the GPU path.

Particles whose usrMark is 93 are traced: every WriteCacheFreq iterations
their iteration, id, type, contact flag, position, linear and angular
velocity (single precision) go to a cache of mDumpPrtclSize records, which is
written out when it is full and at the end of the run to
<DumpPrtclDir>rank<nrank I5.5>_<itime I10.10> as a stream of 52-byte records
(four int32, nine float32, the Fortran type DumpPrtclVar in stream access).

The contact flag is ContactList%IsCntct: 1 when the particle has any contact
of the live list, with another particle or a wall (Prtcl_CL_and_CF.f90:326-339).
"""
from __future__ import annotations

import os
from typing import Optional

import numpy as np

from .beds import Particles

DUMP_FLAG = 93   # Prtcl_Dump_Flag

RECORD = np.dtype([("itime", "<i4"), ("id", "<i4"), ("ptype", "<i4"), ("cntct", "<i4"),
                   ("pos", "<f4", (3,)), ("linvel", "<f4", (3,)), ("rotvel", "<f4", (3,))])


class DumpError(RuntimeError):
    pass


def reset_marks(p: Particles, y_dump: float) -> np.ndarray:
    """ResetDumpFlag: usrMark 93 for particles at y >= yDump, else 1
    (Prtcl_DumpPrtcl.f90:63-71); returns the new usrMark array."""
    return np.where(p.posR[:, 1] >= y_dump, DUMP_FLAG, 1).astype(np.int32)


class PrtclDump:
    """Initilize / WriteCache / PrtclVarDump of the reference on one rank."""

    def __init__(self, dump_dir: str, m_size: int, write_cache_freq: int = 100000, enabled: bool = True,
                 nrank: int = 0):
        if not enabled:
            self.enabled = False
            return
        if m_size < 10000:
            raise DumpError(f"InitDumpPrtclVar: So small mDumpPrtclSize:{m_size}")
        self.enabled = True
        self.dir, self.nrank = dump_dir, nrank
        self.write_cache_freq = write_cache_freq
        self.cache = np.zeros(m_size, RECORD)
        self.n = 0
        os.makedirs(dump_dir, exist_ok=True)

    def due(self, iter_number: int) -> bool:
        """mod(IterNumber, WriteCacheFreq) == 0 (Prtcl_DEMSystem.f90:257)."""
        return self.enabled and iter_number % self.write_cache_freq == 0

    def write_cache(self, itime: int, p: Particles, contacts: tuple) -> None:
        """WriteCache: the marked particles of the state after step itime, with
        `contacts` the live list (owner index, partner id, ...) as
        DEMSystem.contacts() returns it."""
        if not self.enabled:
            return
        n = p.n
        if n > len(self.cache):
            raise DumpError("WriteCache: So small mDumpPrtclSize !!!")
        owner = np.asarray(contacts[0])
        has = np.zeros(n, bool)
        if len(owner):
            has[owner] = True
        sel = np.flatnonzero(p.usrmark[:n] == DUMP_FLAG)
        lin = p.linVel.reshape(n, -1, 3)[:, 0]
        rot = p.rotVel.reshape(n, -1, 3)[:, 0]
        done = 0
        while done < len(sel):
            # the particles that fit before the cache is full, in index order
            k = min(len(sel) - done, len(self.cache) - self.n)
            ids = sel[done:done + k]
            r = self.cache[self.n:self.n + k]
            r["itime"] = itime
            r["id"] = p.id[ids]
            r["ptype"] = p.ptype[ids]
            r["cntct"] = has[ids]
            r["pos"] = p.posR[ids, :3]            # real(x, 4): rounded to nearest
            r["linvel"] = lin[ids]
            r["rotvel"] = rot[ids]
            self.n += k
            done += k
            if self.n == len(self.cache):
                self.dump(itime)

    def dump(self, itime: int) -> Optional[str]:
        """PrtclVarDump: the cached records to <dir>rank<nrank>_<itime>; None
        when the cache is empty."""
        if not self.enabled or self.n == 0:
            return None
        path = os.path.join(self.dir, f"rank{self.nrank:05d}_{itime:010d}")
        self.cache[:self.n].tofile(path)
        self.n = 0
        return path
