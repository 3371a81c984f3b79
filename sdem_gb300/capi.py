"""ctypes binding of libsdem_gpu.so (include/sdem_gpu.h) and a Python handle.

This is the binding a Python caller (and the test suite) uses; a Fortran
caller binds the same symbols through ISO_C_BINDING.  Loading fails loudly
when the library is missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import math
import os
from typing import Optional

import numpy as np

from .beds import Case, Particles

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libsdem_gpu.so")

SDEM_OK = 0
ERRORS = {1: "SDEM_E_ARG", 2: "SDEM_E_CUDA", 3: "SDEM_E_CL_FULL", 4: "SDEM_E_BAD_ID", 5: "SDEM_E_NCV20",
          6: "SDEM_E_GRID", 7: "SDEM_E_TIMEOUT", 8: "SDEM_E_CAPACITY", 9: "SDEM_E_NOMEM",
          10: "SDEM_E_UNSUPPORTED"}
CNT_NAMES = ("pp", "ppg", "ppfix", "pw", "cnsv", "nlocal", "iter", "next_wall_update", "cnsv_cross")

EXPORTED = ("sdem_default_cfg", "sdem_create", "sdem_set_types", "sdem_set_walls", "sdem_upload_particles",
            "sdem_upload_contacts", "sdem_step", "sdem_step_async", "sdem_get_stream",
            "sdem_download_particles", "sdem_download_contacts", "sdem_check_restart_limit",
            "sdem_download_forces", "sdem_counters", "sdem_counters_lagged", "sdem_counter_sums",
            "sdem_launch_count", "sdem_profile_begin", "sdem_profile_end", "sdem_profile_phase_name",
            "sdem_count_contacts_noalloc", "sdem_selftest_fp64", "sdem_probe_fp64_peak",
            "sdem_set_launch", "sdem_get_launch", "sdem_batch_create_grouped",
            "sdem_snapshot_begin", "sdem_snapshot_end", "sdem_snapshot_contacts", "sdem_set_fixed", "sdem_last_error",
            "sdem_destroy", "sdem_batch_create", "sdem_batch_step_async", "sdem_batch_sync", "sdem_batch_step",
            "sdem_batch_last_error", "sdem_batch_destroy")


def selftest_fp64(n: int, seed: int = 1) -> int:
    """Mismatching operand pairs of the library's integer-pipe binary64
    arithmetic against the GPU's own instructions (0 expected)."""
    lib = load()
    out = C.c_longlong()
    rc = lib.sdem_selftest_fp64(int(n), int(seed), C.byref(out))
    if rc:
        raise SdemError(rc, f"sdem_selftest_fp64 failed ({ERRORS.get(rc, rc)})")
    return int(out.value)


class SdemCfg(C.Structure):
    """struct sdem_cfg of include/sdem_gpu.h (field order matters)."""
    _fields_ = [
        ("n_capacity", C.c_int), ("max_gid", C.c_int), ("tsize", C.c_int), ("rsize", C.c_int),
        ("cf_type", C.c_int), ("ct_model", C.c_int), ("pi_method", C.c_int), ("pri_method", C.c_int),
        ("cs_method", C.c_int), ("cntct_list_size", C.c_int), ("base_wall_id", C.c_int),
        ("wall_max_update_iter", C.c_int), ("periodic", C.c_int * 3), ("quirk_ab2_rot", C.c_int),
        ("max_contacts_per_particle", C.c_int), ("dt", C.c_double), ("gravity", C.c_double * 3),
        ("dom_min", C.c_double * 3), ("dom_max", C.c_double * 3), ("cs_ratio", C.c_double),
        ("wall_neighbor_ratio", C.c_double), ("n_fixed_capacity", C.c_int), ("cs_num_levels", C.c_int),
    ]


class SdemError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


def row_capacity_for(radius) -> int:
    """Contacts per sphere the handle makes room for when a case leaves
    max_contacts_per_particle at 0: the library's default of 24, or more when
    the radii differ enough that a large sphere can touch more small ones.
    A sphere of radius R touched by spheres of radius r holds at most about
    4 pi (R + r)^2 / (2 sqrt(3) r^2) = 3.63 (1 + R/r)^2 of them (hexagonal
    cover of the sphere their centres lie on); capped at the library's 64."""
    r = np.asarray(radius, dtype=np.float64)
    if r.size == 0 or not (r.min() > 0.0):
        return 24
    q = float(r.max() / r.min())
    return int(min(64, max(24, math.ceil(3.63 * (1.0 + q) ** 2))))


def cfg_from_case(case: Case, n_capacity: Optional[int] = None, max_gid: Optional[int] = None) -> SdemCfg:
    o = case.opts
    c = SdemCfg()
    c.n_capacity = int(n_capacity or max(case.particles.n, 1))
    c.max_gid = int(max_gid or case.max_gid)
    c.tsize, c.rsize = o.tsize, o.rsize
    c.cf_type, c.ct_model = o.cf_type, o.ct_model
    c.pi_method, c.pri_method = o.pi_method, o.pri_method
    c.cs_method = o.cs_method
    c.cntct_list_size = o.cntct_list_size
    c.base_wall_id = o.base_wall_id
    c.wall_max_update_iter = o.wall_max_update_iter
    for k in range(3):
        c.periodic[k] = int(o.periodic[k])
        c.gravity[k] = o.gravity[k]
        c.dom_min[k] = o.minpoint[k]
        c.dom_max[k] = o.maxpoint[k]
    c.quirk_ab2_rot = int(o.quirk_ab2_rot)
    c.max_contacts_per_particle = int(o.max_contacts_per_particle) or row_capacity_for(case.tables.radius)
    c.dt = o.dt
    c.cs_ratio = o.cs_ratio
    c.wall_neighbor_ratio = o.wall_neighbor_ratio
    c.n_fixed_capacity = int(case.fixed.n) if case.fixed is not None else 0
    c.cs_num_levels = int(getattr(o, "cs_num_levels", 0))
    return c


_lib = None


def load(path: str = LIB_PATH) -> C.CDLL:
    """Loads the sm_103a library.  Raises if it was not built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with `python -m sdem_gb300.build` "
                           "(the GPU path has no fallback)")
    lib = C.CDLL(path)
    P = C.c_void_p
    dp = C.POINTER(C.c_double)
    ip = C.POINTER(C.c_int)
    lib.sdem_default_cfg.argtypes = [C.POINTER(SdemCfg)]
    lib.sdem_default_cfg.restype = None
    lib.sdem_create.argtypes = [C.POINTER(SdemCfg), C.POINTER(P)]
    lib.sdem_set_types.argtypes = [P, C.c_int, dp, dp, dp, dp, C.c_int, dp]
    lib.sdem_set_walls.argtypes = [P, C.c_int, dp, ip]
    lib.sdem_set_fixed.argtypes = [P, C.c_int, ip, ip, dp]
    lib.sdem_upload_particles.argtypes = [P, C.c_int, ip, ip, ip, dp, dp, dp, dp, dp, dp]
    lib.sdem_upload_contacts.argtypes = [P, C.c_int, ip, ip, dp, dp]
    lib.sdem_step.argtypes = [P, C.c_int]
    lib.sdem_step_async.argtypes = [P, C.c_int]
    lib.sdem_get_stream.argtypes = [P, C.POINTER(P)]
    lib.sdem_download_particles.argtypes = [P, ip, ip, ip, ip, dp, dp, dp, dp, dp, dp]
    lib.sdem_download_contacts.argtypes = [P, C.c_int, ip, ip, ip, dp, dp]
    lib.sdem_check_restart_limit.argtypes = [P]
    lib.sdem_download_forces.argtypes = [P, dp, dp]
    lib.sdem_counters.argtypes = [P, ip]
    lib.sdem_counters_lagged.argtypes = [P, ip]
    lib.sdem_launch_count.argtypes = [P, C.POINTER(C.c_longlong)]
    lib.sdem_counter_sums.argtypes = [P, C.POINTER(C.c_longlong)]
    lib.sdem_profile_begin.argtypes = [P, C.c_int]
    lib.sdem_profile_end.argtypes = [P, C.c_int, dp, ip]
    lib.sdem_profile_phase_name.argtypes = [C.c_int]
    lib.sdem_profile_phase_name.restype = C.c_char_p
    lib.sdem_count_contacts_noalloc.argtypes = [C.POINTER(SdemCfg), C.c_double, C.c_int, P, P, P]
    lib.sdem_selftest_fp64.argtypes = [C.c_longlong, C.c_ulonglong, C.POINTER(C.c_longlong)]
    lib.sdem_probe_fp64_peak.argtypes = [C.c_longlong, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    lib.sdem_set_launch.argtypes = [P, C.c_int, C.c_int, C.c_int]
    lib.sdem_get_launch.argtypes = [P, ip, ip, ip]
    lib.sdem_batch_create_grouped.argtypes = [C.c_int, C.POINTER(P), C.c_int, C.POINTER(P)]
    lib.sdem_snapshot_begin.argtypes = [P, ip, ip, ip, dp, dp, dp, dp, dp, dp, dp, dp, C.c_int]
    lib.sdem_snapshot_end.argtypes = [P, ip]
    lib.sdem_snapshot_contacts.argtypes = [P, C.c_int, ip, ip, ip, dp, dp]
    lib.sdem_last_error.argtypes = [P]
    lib.sdem_last_error.restype = C.c_char_p
    lib.sdem_destroy.argtypes = [P]
    lib.sdem_destroy.restype = None
    lib.sdem_batch_create.argtypes = [C.c_int, C.POINTER(P), C.POINTER(P)]
    lib.sdem_batch_step_async.argtypes = [P, C.c_int]
    lib.sdem_batch_sync.argtypes = [P]
    lib.sdem_batch_step.argtypes = [P, C.c_int]
    lib.sdem_batch_last_error.argtypes = [P]
    lib.sdem_batch_last_error.restype = C.c_char_p
    lib.sdem_batch_destroy.argtypes = [P]
    lib.sdem_batch_destroy.restype = None
    for name in EXPORTED:
        if name not in ("sdem_default_cfg", "sdem_last_error", "sdem_destroy", "sdem_profile_phase_name",
                        "sdem_batch_last_error", "sdem_batch_destroy"):
            getattr(lib, name).restype = C.c_int
    _lib = lib
    return lib


def dptr(a: Optional[np.ndarray]):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_double))


def iptr(a: Optional[np.ndarray]):
    if a is None:
        return None
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_int))


NOALLOC_MAX_PARTICLES = 65536
NOALLOC_MAX_CELLS = 524288


def probe_fp64_peak(iters: int = 20000) -> dict:
    """sdem_probe_fp64_peak: DFMA chains on every SM; returns the measured
    DFMA/s, FP64 TFLOP/s (2 per DFMA) and the kernel time."""
    lib = load()
    r, ms = C.c_double(), C.c_double()
    rc = lib.sdem_probe_fp64_peak(int(iters), C.byref(r), C.byref(ms))
    if rc:
        raise SdemError(rc, "sdem_probe_fp64_peak failed")
    return {"dfma_per_s": r.value, "tflops": 2.0 * r.value / 1e12, "ms": ms.value}


def count_contacts_noalloc(cfg: SdemCfg, max_radius: float, n: int, d_posR: int, d_counts: int,
                           stream: int = 0) -> None:
    """sdem_count_contacts_noalloc: device pointers in, device counts out, no
    device allocation (see include/sdem_gpu.h)."""
    lib = load()
    rc = lib.sdem_count_contacts_noalloc(C.byref(cfg), float(max_radius), int(n), C.c_void_p(d_posR),
                                         C.c_void_p(d_counts), C.c_void_p(stream))
    if rc:
        raise SdemError(rc, lib.sdem_last_error(None).decode())


class DEMSystem:
    """One bed on the current GPU, driven through the C ABI."""

    def __init__(self, case: Case, n_capacity: Optional[int] = None, max_gid: Optional[int] = None):
        self.lib = load()
        self.case = case
        self.cfg = cfg_from_case(case, n_capacity, max_gid)
        self.h = C.c_void_p()
        rc = self.lib.sdem_create(C.byref(self.cfg), C.byref(self.h))
        if rc:
            msg = self.lib.sdem_last_error(self.h).decode() if self.h else ""
            self.lib.sdem_destroy(self.h)
            self.h = None
            raise SdemError(rc, msg)
        t = case.tables
        self._check(self.lib.sdem_set_types(self.h, t.n_types, dptr(t.radius), dptr(t.mass), dptr(t.inertia),
                                            dptr(t.bpp), t.n_wall_types, dptr(t.bpw)))
        w, f = case.walls.arrays()
        self._check(self.lib.sdem_set_walls(self.h, case.walls.n, dptr(w) if case.walls.n else None,
                                            iptr(f) if case.walls.n else None))
        if case.fixed is not None and case.fixed.n:
            self.set_fixed(case.fixed)
        self.upload(case.particles)
        if case.contacts is not None:
            self.upload_contacts(*case.contacts)

    def set_fixed(self, fx) -> None:
        """Fixed spheres (beds.FixedSpheres: ids above max_gid, types, centres)."""
        self._fix = (np.ascontiguousarray(fx.id, dtype=np.int32), np.ascontiguousarray(fx.ptype, dtype=np.int32),
                     np.ascontiguousarray(fx.pos, dtype=np.float64))
        self._check(self.lib.sdem_set_fixed(self.h, len(self._fix[0]), iptr(self._fix[0]), iptr(self._fix[1]),
                                            dptr(self._fix[2])))

    def _check(self, rc: int) -> None:
        if rc:
            raise SdemError(rc, self.lib.sdem_last_error(self.h).decode())

    def upload(self, p: Particles) -> None:
        a = lambda x: np.ascontiguousarray(x, dtype=np.float64)
        i = lambda x: np.ascontiguousarray(x, dtype=np.int32)
        self._keep = (i(p.id), i(p.ptype), i(p.usrmark), a(p.posR), a(p.linVel), a(p.linAcc), a(p.theta),
                      a(p.rotVel), a(p.rotAcc))
        k = self._keep
        self._check(self.lib.sdem_upload_particles(self.h, p.n, iptr(k[0]), iptr(k[1]), iptr(k[2]), dptr(k[3]),
                                                   dptr(k[4]), dptr(k[5]), dptr(k[6]), dptr(k[7]), dptr(k[8])))

    def upload_contacts(self, owner, partner, tandelta, velrel) -> None:
        o = np.ascontiguousarray(owner, dtype=np.int32)
        q = np.ascontiguousarray(partner, dtype=np.int32)
        t = np.ascontiguousarray(tandelta, dtype=np.float64)
        v = np.ascontiguousarray(velrel, dtype=np.float64)
        self._check(self.lib.sdem_upload_contacts(self.h, len(o), iptr(o), iptr(q), dptr(t), dptr(v)))

    def step(self, n: int = 1) -> None:
        self._check(self.lib.sdem_step(self.h, int(n)))

    def step_async(self, n: int = 1) -> None:
        self._check(self.lib.sdem_step_async(self.h, int(n)))

    def stream(self) -> int:
        s = C.c_void_p()
        self._check(self.lib.sdem_get_stream(self.h, C.byref(s)))
        return s.value or 0

    def state(self, out: Optional[Particles] = None) -> Particles:
        """The particle state.  With `out` (arrays of at least n_capacity rows,
        C-contiguous, e.g. in pinned host memory) the download lands there and
        views of its first n rows are returned."""
        cap = self.cfg.n_capacity
        ts, rs = self.cfg.tsize, self.cfg.rsize
        n = C.c_int()
        fresh = out is None
        if fresh:
            out = Particles(np.zeros(cap, np.int32), np.zeros(cap, np.int32), np.zeros(cap, np.int32),
                            np.zeros((cap, 4)), np.zeros((cap, ts, 3)), np.zeros((cap, ts, 3)), np.zeros((cap, 3)),
                            np.zeros((cap, rs, 3)), np.zeros((cap, rs, 3)))
        else:
            for a, shape, dt in ((out.id, (cap,), np.int32), (out.posR, (cap, 4), np.float64),
                                 (out.linVel, (cap, ts, 3), np.float64), (out.rotVel, (cap, rs, 3), np.float64)):
                if a.shape[0] < cap or a.shape[1:] != shape[1:] or a.dtype != dt or not a.flags.c_contiguous:
                    raise ValueError("state(out=...): arrays must be C-contiguous with n_capacity rows")
        self._check(self.lib.sdem_download_particles(self.h, C.byref(n), iptr(out.id), iptr(out.ptype),
                                                     iptr(out.usrmark), dptr(out.posR), dptr(out.linVel),
                                                     dptr(out.linAcc), dptr(out.theta), dptr(out.rotVel),
                                                     dptr(out.rotAcc)))
        k = n.value
        if fresh:
            return out.take(slice(0, k))
        return Particles(out.id[:k], out.ptype[:k], out.usrmark[:k], out.posR[:k], out.linVel[:k], out.linAcc[:k],
                         out.theta[:k], out.rotVel[:k], out.rotAcc[:k])

    def forces(self):
        n = self.counters()["nlocal"]
        F = np.zeros((max(n, 1), 3))
        T = np.zeros((max(n, 1), 3))
        self._check(self.lib.sdem_download_forces(self.h, dptr(F), dptr(T)))
        return F[:n], T[:n]

    def contacts(self):
        nc = C.c_int()
        self._check(self.lib.sdem_download_contacts(self.h, 0, C.byref(nc), None, None, None, None))
        # the records are now the library's finished snapshot: read them there
        return self._snapshot_records(nc.value)

    def _snapshot_records(self, m: int):
        nc = C.c_int()
        o = np.zeros(max(m, 1), np.int32)
        q = np.zeros(max(m, 1), np.int32)
        t = np.zeros((max(m, 1), 3))
        v = np.zeros(max(m, 1))
        self._check(self.lib.sdem_snapshot_contacts(self.h, max(m, 1), C.byref(nc), iptr(o), iptr(q), dptr(t),
                                                    dptr(v)))
        m = nc.value
        return o[:m], q[:m], t[:m], v[:m]

    def snapshot_begin(self, out: Particles, F: Optional[np.ndarray] = None, T: Optional[np.ndarray] = None,
                       contacts: bool = False) -> None:
        """Freezes the state after the steps enqueued so far and starts its
        download into `out` (n_capacity rows, C-contiguous; page-locked memory
        lets the copy run at full speed) and F, T ((n_capacity, 3) each, or
        None).  Steps issued before snapshot_end overlap the copy."""
        cap = self.cfg.n_capacity
        for a in (out.id, out.posR, out.linVel, out.rotVel) + tuple(x for x in (F, T) if x is not None):
            if a.shape[0] < cap or not a.flags.c_contiguous:
                raise ValueError("snapshot_begin: arrays must be C-contiguous with n_capacity rows")
        self._snap = (out, F, T)
        self._check(self.lib.sdem_snapshot_begin(self.h, iptr(out.id), iptr(out.ptype), iptr(out.usrmark),
                                                 dptr(out.posR), dptr(out.linVel), dptr(out.linAcc),
                                                 dptr(out.theta), dptr(out.rotVel), dptr(out.rotAcc),
                                                 dptr(F) if F is not None else None,
                                                 dptr(T) if T is not None else None, 1 if contacts else 0))

    def snapshot_end(self):
        """Waits for the snapshot; returns (Particles views of its n rows, F[:n], T[:n])."""
        n = C.c_int()
        self._check(self.lib.sdem_snapshot_end(self.h, C.byref(n)))
        out, F, T = self._snap
        self._snap = None
        k = n.value
        p = Particles(out.id[:k], out.ptype[:k], out.usrmark[:k], out.posR[:k], out.linVel[:k], out.linAcc[:k],
                      out.theta[:k], out.rotVel[:k], out.rotAcc[:k])
        return p, (F[:k] if F is not None else None), (T[:k] if T is not None else None)

    def snapshot_contacts(self):
        """Contact records of the last finished snapshot taken with contacts=True."""
        nc = C.c_int()
        self._check(self.lib.sdem_snapshot_contacts(self.h, 0, C.byref(nc), None, None, None, None))
        return self._snapshot_records(nc.value)

    def counter_sums(self) -> dict:
        out = (C.c_longlong * 3)()
        self._check(self.lib.sdem_counter_sums(self.h, out))
        return {"pp": out[0], "pw": out[1], "steps": out[2]}

    def set_launch(self, pipeline_chunks: int = 0, force_blocks_per_sm: int = 0, first_chunk_percent: int = 0) -> None:
        """sdem_set_launch: the step's launch shape (results do not depend on
        it); first_chunk_percent -1 restores the default split (a first chunk
        of whole search waves), 0 keeps a value."""
        self._check(self.lib.sdem_set_launch(self.h, int(pipeline_chunks), int(force_blocks_per_sm),
                                             int(first_chunk_percent)))

    def get_launch(self) -> tuple:
        """(pipeline_chunks, force_blocks_per_sm, first_chunk_percent; 0 = the default split)."""
        a, b, c = C.c_int(), C.c_int(), C.c_int()
        self._check(self.lib.sdem_get_launch(self.h, C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, c.value

    def launch_count(self) -> int:
        n = C.c_longlong()
        self._check(self.lib.sdem_launch_count(self.h, C.byref(n)))
        return n.value

    def profile_begin(self, max_steps: int) -> None:
        self._check(self.lib.sdem_profile_begin(self.h, int(max_steps)))

    def profile_end(self) -> tuple:
        """-> ({phase: summed ms}, steps timed)"""
        ms = np.zeros(32)
        ns = C.c_int()
        k = self.lib.sdem_profile_end(self.h, 32, dptr(ms), C.byref(ns))
        if k <= 0:
            raise SdemError(k, self.lib.sdem_last_error(self.h).decode())
        names = [self.lib.sdem_profile_phase_name(i).decode() for i in range(k)]
        return dict(zip(names, ms[:k].tolist())), ns.value

    def check_restart_limit(self) -> None:
        self._check(self.lib.sdem_check_restart_limit(self.h))

    def counters(self) -> dict:
        out = np.zeros(9, np.int32)
        self._check(self.lib.sdem_counters(self.h, iptr(out)))
        return dict(zip(CNT_NAMES, (int(x) for x in out)))

    def counters_lagged(self) -> dict:
        """Counters of the step before the last one enqueued (sdem_counters_lagged)."""
        out = np.zeros(9, np.int32)
        self._check(self.lib.sdem_counters_lagged(self.h, iptr(out)))
        return dict(zip(CNT_NAMES, (int(x) for x in out)))

    def close(self) -> None:
        if self.h:
            self.lib.sdem_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class DEMBatch:
    """Many DEMSystem beds advanced together (sdem_batch_*): one CUDA graph
    per batch step holds every member's step.  The members stay usable for
    downloads and single steps; they must outlive the batch."""

    def __init__(self, members, group_size: int = 0):
        self.lib = load()
        self.members = list(members)
        arr = (C.c_void_p * len(self.members))(*[m.h.value for m in self.members])
        self.b = C.c_void_p()
        rc = self.lib.sdem_batch_create_grouped(len(self.members), arr, int(group_size), C.byref(self.b))
        if rc:
            msg = self.lib.sdem_batch_last_error(self.b).decode() if self.b else ""
            self.lib.sdem_batch_destroy(self.b)
            self.b = None
            raise SdemError(rc, msg)

    def _check(self, rc: int) -> None:
        if rc:
            raise SdemError(rc, self.lib.sdem_batch_last_error(self.b).decode())

    def step(self, n: int = 1) -> None:
        self._check(self.lib.sdem_batch_step(self.b, int(n)))

    def step_async(self, n: int = 1) -> None:
        self._check(self.lib.sdem_batch_step_async(self.b, int(n)))

    def sync(self) -> None:
        self._check(self.lib.sdem_batch_sync(self.b))

    def close(self) -> None:
        if self.b:
            self.lib.sdem_batch_destroy(self.b)
            self.b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
