"""ctypes driver of the CPU oracle (oracle/sdem_oracle.c).

TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the CPU
baseline leg of bench.py, to check the GPU path.  The product never imports it.

OracleSystem mirrors sdem_gb300.capi.DEMSystem (same constructor, step, state,
forces, contacts, counters), so a test runs one Case through both.
"""
from __future__ import annotations

import ctypes as C
import os
import sys
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from sdem_gb300.beds import Case, Particles  # noqa: E402
from sdem_gb300.capi import CNT_NAMES, SdemCfg, cfg_from_case, dptr, iptr  # noqa: E402

LIB_PATH = os.path.join(HERE, "libsdem_oracle.so")
_lib = None


def load() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    import importlib.util
    spec = importlib.util.spec_from_file_location("oracle_build", os.path.join(HERE, "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.build()  # no-op when up to date
    lib = C.CDLL(LIB_PATH)
    P = C.c_void_p
    dp = C.POINTER(C.c_double)
    ip = C.POINTER(C.c_int)
    lib.orc_create.argtypes = [C.POINTER(SdemCfg)]
    lib.orc_create.restype = P
    lib.orc_set_types.argtypes = [P, C.c_int, dp, dp, dp, dp, C.c_int, dp]
    lib.orc_set_walls.argtypes = [P, C.c_int, dp, ip]
    lib.orc_set_fixed.argtypes = [P, C.c_int, ip, ip, dp]
    lib.orc_upload_particles.argtypes = [P, C.c_int, ip, ip, ip, dp, dp, dp, dp, dp, dp]
    lib.orc_upload_contacts.argtypes = [P, C.c_int, ip, ip, dp, dp]
    lib.orc_step.argtypes = [P, C.c_int]
    lib.orc_nlocal.argtypes = [P]
    lib.orc_download_particles.argtypes = [P, ip, ip, ip, dp, dp, dp, dp, dp, dp]
    lib.orc_download_forces.argtypes = [P, dp, dp]
    lib.orc_download_contacts.argtypes = [P, C.c_int, ip, ip, ip, dp, dp]
    lib.orc_counters.argtypes = [P, ip]
    lib.orc_last_error.argtypes = [P]
    lib.orc_last_error.restype = C.c_char_p
    lib.orc_destroy.argtypes = [P]
    lib.orc_destroy.restype = None
    lib.orc_binary_prop.argtypes = [C.c_int] + [C.c_double] * 13 + [C.c_int, dp]
    lib.orc_binary_prop.restype = None
    lib.orc_pure_prop.argtypes = [C.c_double, C.c_double, dp, dp, dp]
    lib.orc_pure_prop.restype = None
    lib.orc_make_wall.argtypes = [dp, dp, dp, dp, dp]
    lib.orc_make_wall.restype = None
    lib.orc_grid.argtypes = [P, dp, dp, ip]
    lib.orc_grid.restype = None
    lib.orc_set_iter.argtypes = [P, C.c_int]
    lib.orc_set_iter.restype = None
    for name in ("orc_set_types", "orc_set_walls", "orc_set_fixed", "orc_upload_particles", "orc_upload_contacts", "orc_step",
                 "orc_nlocal", "orc_download_particles", "orc_download_forces", "orc_download_contacts",
                 "orc_counters"):
        getattr(lib, name).restype = C.c_int
    _lib = lib
    return lib


class OracleError(RuntimeError):
    pass


class OracleSystem:
    def __init__(self, case: Case, n_capacity: Optional[int] = None, max_gid: Optional[int] = None):
        self.lib = load()
        self.case = case
        self.cfg = cfg_from_case(case, n_capacity, max_gid)
        self.h = self.lib.orc_create(C.byref(self.cfg))
        t = case.tables
        self._check(self.lib.orc_set_types(self.h, t.n_types, dptr(t.radius), dptr(t.mass), dptr(t.inertia),
                                           dptr(t.bpp), t.n_wall_types, dptr(t.bpw)))
        w, f = case.walls.arrays()
        self._check(self.lib.orc_set_walls(self.h, case.walls.n, dptr(w) if case.walls.n else None,
                                           iptr(f) if case.walls.n else None))
        if case.fixed is not None and case.fixed.n:
            fx = case.fixed
            self._fix = (np.ascontiguousarray(fx.id, dtype=np.int32), np.ascontiguousarray(fx.ptype, dtype=np.int32),
                         np.ascontiguousarray(fx.pos, dtype=np.float64))
            self._check(self.lib.orc_set_fixed(self.h, fx.n, iptr(self._fix[0]), iptr(self._fix[1]),
                                               dptr(self._fix[2])))
        self.upload(case.particles)
        if case.contacts is not None:
            self.upload_contacts(*case.contacts)

    def _check(self, rc: int) -> None:
        if rc:
            raise OracleError(f"oracle error {rc}: {self.lib.orc_last_error(self.h).decode()}")

    def upload(self, p: Particles) -> None:
        a = lambda x: np.ascontiguousarray(x, dtype=np.float64)
        i = lambda x: np.ascontiguousarray(x, dtype=np.int32)
        k = (i(p.id), i(p.ptype), i(p.usrmark), a(p.posR), a(p.linVel), a(p.linAcc), a(p.theta), a(p.rotVel),
             a(p.rotAcc))
        self._check(self.lib.orc_upload_particles(self.h, p.n, iptr(k[0]), iptr(k[1]), iptr(k[2]), dptr(k[3]),
                                                  dptr(k[4]), dptr(k[5]), dptr(k[6]), dptr(k[7]), dptr(k[8])))

    def upload_contacts(self, owner, partner, tandelta, velrel) -> None:
        o = np.ascontiguousarray(owner, dtype=np.int32)
        q = np.ascontiguousarray(partner, dtype=np.int32)
        t = np.ascontiguousarray(tandelta, dtype=np.float64)
        v = np.ascontiguousarray(velrel, dtype=np.float64)
        self._check(self.lib.orc_upload_contacts(self.h, len(o), iptr(o), iptr(q), dptr(t), dptr(v)))

    def step(self, n: int = 1) -> None:
        self._check(self.lib.orc_step(self.h, int(n)))

    def state(self) -> Particles:
        n = self.lib.orc_nlocal(self.h)
        ts, rs = self.cfg.tsize, self.cfg.rsize
        m = max(n, 1)
        out = Particles(np.zeros(m, np.int32), np.zeros(m, np.int32), np.zeros(m, np.int32), np.zeros((m, 4)),
                        np.zeros((m, ts, 3)), np.zeros((m, ts, 3)), np.zeros((m, 3)), np.zeros((m, rs, 3)),
                        np.zeros((m, rs, 3)))
        self._check(self.lib.orc_download_particles(self.h, iptr(out.id), iptr(out.ptype), iptr(out.usrmark),
                                                    dptr(out.posR), dptr(out.linVel), dptr(out.linAcc),
                                                    dptr(out.theta), dptr(out.rotVel), dptr(out.rotAcc)))
        return out.take(slice(0, n))

    def forces(self):
        n = self.lib.orc_nlocal(self.h)
        F = np.zeros((max(n, 1), 3))
        T = np.zeros((max(n, 1), 3))
        self._check(self.lib.orc_download_forces(self.h, dptr(F), dptr(T)))
        return F[:n], T[:n]

    def contacts(self):
        nc = C.c_int()
        self._check(self.lib.orc_download_contacts(self.h, 0, C.byref(nc), None, None, None, None))
        m = nc.value
        o = np.zeros(max(m, 1), np.int32)
        q = np.zeros(max(m, 1), np.int32)
        t = np.zeros((max(m, 1), 3))
        v = np.zeros(max(m, 1))
        self._check(self.lib.orc_download_contacts(self.h, max(m, 1), C.byref(nc), iptr(o), iptr(q), dptr(t),
                                                   dptr(v)))
        return o[:m], q[:m], t[:m], v[:m]

    def counters(self) -> dict:
        out = np.zeros(9, np.int32)
        self._check(self.lib.orc_counters(self.h, iptr(out)))
        return dict(zip(CNT_NAMES, (int(x) for x in out)))

    def grid(self):
        cl = C.c_double()
        org = np.zeros(3)
        dims = np.zeros(3, np.int32)
        self.lib.orc_grid(self.h, C.byref(cl), dptr(org), iptr(dims))
        return cl.value, org, dims

    def close(self) -> None:
        if self.h:
            self.lib.orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def binary_prop(cf_type, ri, mi, ei, pri, rj, mj, ej, prj, mus, muk, mur, en, et, iswall):
    out = np.zeros(11)
    load().orc_binary_prop(cf_type, ri, mi, ei, pri, rj, mj, ej, prj, mus, muk, mur, en, et, int(iswall), dptr(out))
    return out


def pure_prop(diameter, density):
    r, m, i = C.c_double(), C.c_double(), C.c_double()
    load().orc_pure_prop(diameter, density, C.byref(r), C.byref(m), C.byref(i))
    return r.value, m.value, i.value


def make_wall(p1, p2, p3, p4):
    arr = [np.ascontiguousarray(p, dtype=np.float64) for p in (p1, p2, p3, p4)]
    out = np.zeros(25)
    load().orc_make_wall(dptr(arr[0]), dptr(arr[1]), dptr(arr[2]), dptr(arr[3]), dptr(out))
    return out
