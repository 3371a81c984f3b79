"""Seeded synthetic beds and the cases they belong to.

A Case is one complete input of the hot path: options (the &DEMOptions fields
the path reads), material tables, plane walls and particle arrays in the
reference's layouts.  The reference's own particle maker is clock-seeded
(Prtcl_Variables.f90:225-227), so every bed here is generated from an explicit
seed instead and stands in for a restart file of the reference.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, replace
from typing import Optional, Tuple

import numpy as np

from . import props
from .geometry import WallSet, box_walls


@dataclass
class Options:
    """&DEMOptions fields of the hot path (Prtcl_Parameters.f90:45-95)."""
    dt: float = 1.0e-5
    gravity: Tuple[float, float, float] = (0.0, -9.81, 0.0)
    minpoint: Tuple[float, float, float] = (0.0, 0.0, 0.0)
    maxpoint: Tuple[float, float, float] = (1.0, 1.0, 1.0)
    periodic: Tuple[int, int, int] = (0, 0, 0)
    cs_ratio: float = 1.0
    cs_method: int = 1
    cs_num_levels: int = 0
    cf_type: int = props.CFT_LSD
    ct_model: int = 1
    pi_method: int = 1
    pri_method: int = 1
    cntct_list_size: int = 6
    base_wall_id: int = 10000000
    wall_max_update_iter: int = 100
    wall_neighbor_ratio: float = 2.0
    quirk_ab2_rot: int = 1
    max_contacts_per_particle: int = 0

    @property
    def tsize(self) -> int:
        return self.pi_method

    @property
    def rsize(self) -> int:
        return self.pri_method


@dataclass
class Particles:
    id: np.ndarray        # int32 (n,)
    ptype: np.ndarray     # int32 (n,), 1-based
    usrmark: np.ndarray   # int32 (n,)
    posR: np.ndarray      # (n, 4): x, y, z, radius
    linVel: np.ndarray    # (n, tsize, 3)
    linAcc: np.ndarray    # (n, tsize, 3)
    theta: np.ndarray     # (n, 3)
    rotVel: np.ndarray    # (n, rsize, 3)
    rotAcc: np.ndarray    # (n, rsize, 3)

    @property
    def n(self) -> int:
        return len(self.id)

    def copy(self) -> "Particles":
        return Particles(*(a.copy() for a in (self.id, self.ptype, self.usrmark, self.posR, self.linVel,
                                               self.linAcc, self.theta, self.rotVel, self.rotAcc)))

    def take(self, idx) -> "Particles":
        return Particles(*(a[idx].copy() for a in (self.id, self.ptype, self.usrmark, self.posR, self.linVel,
                                                    self.linAcc, self.theta, self.rotVel, self.rotAcc)))


@dataclass
class FixedSpheres:
    """Fixed spheres (GPFix_id, GPFix_pType, GPFix_PosR; PIO_ReadFixedCoord,
    Prtcl_IOAndVisu.f90:164-291).  The reference numbers them file position +
    numPrtcl, above every moving id; the radius comes from the type."""
    id: np.ndarray      # int32 (n,)
    ptype: np.ndarray   # int32 (n,), 1-based
    pos: np.ndarray     # (n, 3)

    @property
    def n(self) -> int:
        return len(self.id)


@dataclass
class Case:
    name: str
    opts: Options
    tables: props.Tables
    walls: WallSet
    particles: Particles
    contacts: Optional[tuple] = None   # (owner_idx, partner_id, tandelta (nc,3), velrel) or None
    note: str = ""
    fixed: Optional[FixedSpheres] = None

    @property
    def max_gid(self) -> int:
        return int(self.particles.id.max()) if self.particles.n else 1


def new_particles(pos: np.ndarray, ptype: np.ndarray, radius_of_type: np.ndarray, vel: np.ndarray,
                  tsize: int, rsize: int, first_id: int = 1) -> Particles:
    n = len(pos)
    posR = np.zeros((n, 4))
    posR[:, :3] = pos
    posR[:, 3] = radius_of_type[ptype - 1]
    linVel = np.zeros((n, tsize, 3))
    linVel[:, :, :] = vel[:, None, :]   # every AB level starts at the initial velocity
    return Particles(id=np.arange(first_id, first_id + n, dtype=np.int32), ptype=ptype.astype(np.int32),
                     usrmark=np.zeros(n, dtype=np.int32), posR=posR, linVel=linVel,
                     linAcc=np.zeros((n, tsize, 3)), theta=np.zeros((n, 3)), rotVel=np.zeros((n, rsize, 3)),
                     rotAcc=np.zeros((n, rsize, 3)))


# --------------------------------------------------------------------------
# workloads
# --------------------------------------------------------------------------
def lsd_mono_case(n: int = 20000, seed: int = 1, box=(0.04, 0.2, 0.04), d: float = 1.0e-3,
                  steps_dt: float = 2.0e-6, pi: int = 2, pri: int = 2) -> Case:
    """20k monodisperse LSD spheres on a seeded jittered lattice (pitch 1.2 d,
    jitter U(-0.1d, 0.1d) per axis, velocity U(-0.05, 0.05) m/s) in a
    0.04 x 0.2 x 0.04 m box (gravity -y) with a floor and four side walls;
    Adams-Bashforth 2, dt = 2e-6 s.  Restitution 0.9, friction 0.3, rolling
    friction 0.1.  The reference's LSD has no direct k_n input: Young's modulus
    is chosen so that its stiffness K_n*V**0.4 equals 1e4 N/m at V = 0.05 m/s."""
    rng = np.random.default_rng(seed)
    pitch = 1.2 * d
    nxz = int(box[0] / pitch)
    nzz = int(box[2] / pitch)
    per_layer = nxz * nzz
    layers = int(math.ceil(n / per_layer))
    idx = np.arange(n)
    iy, rem = np.divmod(idx, per_layer)
    ix, iz = np.divmod(rem, nzz)
    pos = np.stack([(ix + 0.5) * pitch + box[0] * 0.0 + (box[0] - nxz * pitch) * 0.5,
                    (iy + 0.5) * pitch + 0.5 * (pitch - d) * 0.0,
                    (iz + 0.5) * pitch + (box[2] - nzz * pitch) * 0.5], axis=1)
    if layers * pitch > box[1]:
        raise ValueError("box too short for the lattice")
    pos = pos + rng.uniform(-0.1 * d, 0.1 * d, size=pos.shape)
    vel = rng.uniform(-0.05, 0.05, size=(n, 3))
    nu = 0.3
    E = props.lsd_youngs_for_stiffness(1.0e4, 0.05, d, 2500.0, nu)
    tables = props.build_tables(props.CFT_LSD, [d], [2500.0], [E], [nu], (0.3, 0.3, 0.1, 0.9, 0.9),
                                [E], [nu], (0.3, 0.3, 0.1, 0.9, 0.9))
    opts = Options(dt=steps_dt, minpoint=(0.0, 0.0, 0.0), maxpoint=tuple(box), cf_type=props.CFT_LSD,
                   pi_method=pi, pri_method=pri)
    parts = new_particles(pos, np.ones(n, dtype=np.int32), tables.radius, vel, opts.tsize, opts.rsize)
    walls = box_walls(opts.minpoint, opts.maxpoint, infinite=True, base_wall_id=opts.base_wall_id)
    return Case(f"lsd_mono_{n}", opts, tables, walls, parts,
                note=f"LSD E={E:.6g} Pa (k_n(0.05 m/s)=1e4 N/m), nu=0.3, e=0.9, mu=0.3, mu_r=0.1")


def hertz_poly_tables(ntypes: int = 41, d_lo: float = 0.8e-3, d_hi: float = 1.2e-3, E: float = 5.0e7,
                      nu: float = 0.3, e_n: float = 0.8, mu: float = 0.4, mu_r: float = 0.1,
                      density: float = 2500.0):
    diam = np.linspace(d_lo, d_hi, ntypes) if ntypes > 1 else np.array([0.5 * (d_lo + d_hi)])
    coefs = (mu, mu, mu_r, e_n, e_n)
    tables = props.build_tables(props.CFT_NLIN, list(diam), [density] * ntypes, [E] * ntypes, [nu] * ntypes,
                                coefs, [E], [nu], coefs)
    return diam, tables


def deposited_positions(rng, diam_of_particle: np.ndarray, box, floor_y: float, overlap,
                        spacing: float, jitter: float):
    """Layer-by-layer deposition onto a body-centred column grid.

    Even layers sit on the grid (spacing/2 + i*spacing), odd layers on the grid
    shifted by half a spacing in x and z.  Each sphere (lateral jitter
    U(-jitter, jitter)) is lowered until it rests on the highest of the floor,
    the spheres of the layer below and the sphere two layers below in its own
    column, then sunk by `overlap` (a number, or a function of (layer, number
    of layers) giving the sink of that layer).  With spacing >= max diameter +
    2*jitter no two spheres of one layer touch.  Returns positions in
    placement order (bottom layer first)."""
    n = len(diam_of_particle)
    r = 0.5 * diam_of_particle
    pos = np.zeros((n, 3))
    per_even = (int((box[0] - spacing) / spacing) + 1) * (int((box[2] - spacing) / spacing) + 1)
    n_layers = int(math.ceil(n / max(per_even - per_even ** 0.5, 1)))
    sink = overlap if callable(overlap) else (lambda k, nl: overlap)
    done = 0
    layers = []   # per layer: (origin, x, z, y, r) grids with NaN where empty
    k = 0
    while done < n:
        org = 0.5 * spacing + (0.5 * spacing if k % 2 else 0.0)
        nxl = int((box[0] - org - 0.5 * spacing) / spacing) + 1
        nzl = int((box[2] - org - 0.5 * spacing) / spacing) + 1
        cnt = min(nxl * nzl, n - done)
        gx, gz = np.divmod(np.arange(cnt), nzl)
        xg = org + gx * spacing
        zg = org + gz * spacing
        x = xg + rng.uniform(-jitter, jitter, cnt)
        z = zg + rng.uniform(-jitter, jitter, cnt)
        rr = r[done:done + cnt]
        y = floor_y + rr
        for back in (1, 2, 3, 4):
            if len(layers) < back:
                continue
            porg, px, pz, py, pr = layers[-back]
            pnx, pnz = px.shape
            bx = np.floor((xg - porg) / spacing + 1e-9).astype(np.int64)
            bz = np.floor((zg - porg) / spacing + 1e-9).astype(np.int64)
            for dxs in (-1, 0, 1, 2):
                for dzs in (-1, 0, 1, 2):
                    qx = bx + dxs
                    qz = bz + dzs
                    ok = (qx >= 0) & (qx < pnx) & (qz >= 0) & (qz < pnz)
                    qx2 = np.clip(qx, 0, pnx - 1)
                    qz2 = np.clip(qz, 0, pnz - 1)
                    sy = py[qx2, qz2]
                    sr = pr[qx2, qz2]
                    reach = (rr + sr) ** 2 - ((x - px[qx2, qz2]) ** 2 + (z - pz[qx2, qz2]) ** 2)
                    valid = ok & np.isfinite(sy) & (reach > 0)
                    y = np.where(valid, np.maximum(y, sy + np.sqrt(np.where(valid, reach, 0.0))), y)
        y = y - sink(k, n_layers)
        pos[done:done + cnt] = np.stack([x, y, z], axis=1)
        grids = [np.full((nxl, nzl), np.nan) for _ in range(4)]
        for g, v in zip(grids, (x, z, y, rr)):
            g[gx, gz] = v
        layers.append((org, *grids))
        done += cnt
        k += 1
    if pos[:, 1].max() + r.max() > box[1]:
        raise ValueError("deposited bed is taller than the box")
    return pos


def settled_deposition(rng, ptype: np.ndarray, ids: np.ndarray, tables, box, spacing: float, jitter: float,
                       gravity: float = 9.81, wall_type: int = 1):
    """Deposition onto a body-centred column grid in static equilibrium along
    its resting contacts.

    Geometry: layer by layer (even layers on the grid spacing/2 + i*spacing,
    odd layers shifted by half a spacing in x and z, lateral jitter
    U(-jitter, jitter)), every sphere rests on the highest of the floor and the
    spheres of the four layers below -- its support.  Loads: the weight of a
    sphere plus everything resting on it, summed from the top down.  Sinks:
    from the bottom up, each sphere is lowered with its support and then by
    delta/cos(theta) more, where delta = (N/K)^(2/3) is the Hertz overlap that
    carries the normal load N = load/cos(theta) of the inclined contact, with
    the pair's own K (the reference's table record of the lower-id sphere,
    Prtcl_Property.f90:137-142, 241-242) or the wall's.  Positions in placement
    order (bottom layer first)."""
    n = len(ptype)
    nT = len(tables.radius)
    r = tables.radius[ptype - 1]
    m = tables.mass[ptype - 1]
    pos = np.zeros((n, 3))
    sup = np.full(n, -1, dtype=np.int64)
    layer_of = np.zeros(n, dtype=np.int64)
    done = 0
    layers = []   # per layer: (origin, x, z, y, r, global index) grids
    k = 0
    while done < n:
        org = 0.5 * spacing + (0.5 * spacing if k % 2 else 0.0)
        nxl = int((box[0] - org - 0.5 * spacing) / spacing) + 1
        nzl = int((box[2] - org - 0.5 * spacing) / spacing) + 1
        cnt = min(nxl * nzl, n - done)
        gx, gz = np.divmod(np.arange(cnt), nzl)
        xg = org + gx * spacing
        zg = org + gz * spacing
        x = xg + rng.uniform(-jitter, jitter, cnt)
        z = zg + rng.uniform(-jitter, jitter, cnt)
        rr = r[done:done + cnt]
        y = rr.copy()
        s_of = np.full(cnt, -1, dtype=np.int64)
        for back in (1, 2, 3, 4):
            if len(layers) < back:
                continue
            porg, px, pz, py, pr, pid = layers[-back]
            pnx, pnz = px.shape
            bx = np.floor((xg - porg) / spacing + 1e-9).astype(np.int64)
            bz = np.floor((zg - porg) / spacing + 1e-9).astype(np.int64)
            for dxs in (-1, 0, 1, 2):
                for dzs in (-1, 0, 1, 2):
                    qx = bx + dxs
                    qz = bz + dzs
                    ok = (qx >= 0) & (qx < pnx) & (qz >= 0) & (qz < pnz)
                    qx2 = np.clip(qx, 0, pnx - 1)
                    qz2 = np.clip(qz, 0, pnz - 1)
                    sy = py[qx2, qz2]
                    reach = (rr + pr[qx2, qz2]) ** 2 - ((x - px[qx2, qz2]) ** 2 + (z - pz[qx2, qz2]) ** 2)
                    valid = ok & np.isfinite(sy) & (reach > 0)
                    cand = np.where(valid, sy + np.sqrt(np.where(valid, reach, 0.0)), -np.inf)
                    better = cand > y
                    y = np.where(better, cand, y)
                    s_of = np.where(better, pid[qx2, qz2], s_of)
        sl = slice(done, done + cnt)
        pos[sl] = np.stack([x, y, z], axis=1)
        sup[sl] = s_of
        layer_of[sl] = k
        grids = [np.full((nxl, nzl), np.nan) for _ in range(4)]
        for g_, v in zip(grids, (x, z, y, rr)):
            g_[gx, gz] = v
        gid_grid = np.full((nxl, nzl), -1, dtype=np.int64)
        gid_grid[gx, gz] = np.arange(done, done + cnt)
        layers.append((org, *grids, gid_grid))
        done += cnt
        k += 1
    # loads, top down
    load = m * gravity
    for L in range(k - 1, -1, -1):
        idx = np.nonzero(layer_of == L)[0]
        s_ = sup[idx]
        on = s_ >= 0
        np.add.at(load, s_[on], load[idx[on]])
    # sinks, bottom up
    bpp = tables.bpp.reshape(nT, nT, 11)
    bpw = tables.bpw.reshape(-1, nT, 11)
    geo_y = pos[:, 1].copy()
    for L in range(k):
        idx = np.nonzero(layer_of == L)[0]
        s_ = sup[idx]
        on = s_ >= 0
        cos_t = np.ones(len(idx))
        K = bpw[wall_type - 1, ptype[idx] - 1, 2].copy()
        base = np.zeros(len(idx))
        if on.any():
            a, b = idx[on], s_[on]
            # a support far to the side would let the sphere roll off: the sink
            # is computed with cos(theta) >= 0.3 there
            cos_t[on] = np.maximum((geo_y[a] - geo_y[b]) / (r[a] + r[b]), 0.3)
            lo = np.where(ids[a] < ids[b], a, b)
            hi = np.where(ids[a] < ids[b], b, a)
            K[on] = bpp[ptype[hi] - 1, ptype[lo] - 1, 2]
            base[on] = geo_y[b] - pos[b, 1]   # the support's own sink
        delta = (load[idx] / cos_t / K) ** (2.0 / 3.0)
        pos[idx, 1] = geo_y[idx] - base - delta / cos_t
    if pos[:, 1].max() + r.max() > box[1]:
        raise ValueError("deposited bed is taller than the box")
    return pos


def hertz_poly_case(n: int = 1_000_000, seed: int = 2, box=(0.1, 0.6, 0.1), ntypes: int = 41,
                    dt: float = 1.0e-6, pi: int = 2, pri: int = 2) -> Case:
    """Polydisperse Hertz-Mindlin bed: d uniform in [0.8, 1.2] mm realised as
    `ntypes` discrete types (10 um steps for 41), density 2500 kg/m^3,
    E = 5e7 Pa, nu = 0.3, restitution 0.8, friction 0.4 (rolling 0.1), in a
    0.1 x 0.6 x 0.1 m box with a floor and four side walls, gravity -y,
    dt = 1e-6 s.  Positions: settled_deposition (column grid spacing 1.3 mm,
    lateral jitter 0.05 mm), a packed bed in static equilibrium along its
    resting contacts, at rest.  Particle order and ids are a seeded shuffle
    (the reference's maker also shuffles its particles, Prtcl_Variables.f90:279-288)."""
    rng = np.random.default_rng(seed)
    diam, tables = hertz_poly_tables(ntypes)
    ptype = rng.integers(1, ntypes + 1, size=n).astype(np.int32)
    perm = rng.permutation(n)            # storage position of the k-th placed sphere
    ids = np.empty(n, dtype=np.int64)
    ids[perm] = np.arange(1, n + 1)      # id = storage position + 1
    ids = ids.astype(np.int64)
    placed_ids = np.empty(n, dtype=np.int64)
    placed_ids[:] = perm + 1
    pos = settled_deposition(rng, ptype, placed_ids, tables, box, spacing=1.3e-3, jitter=0.05e-3)
    opts = Options(dt=dt, minpoint=(0.0, 0.0, 0.0), maxpoint=tuple(box), cf_type=props.CFT_NLIN,
                   pi_method=pi, pri_method=pri)
    vel = np.zeros((n, 3))
    placed = new_particles(pos, ptype, tables.radius, vel, opts.tsize, opts.rsize)
    parts = placed.take(np.argsort(perm))
    parts.id = np.arange(1, n + 1, dtype=np.int32)
    walls = box_walls(opts.minpoint, opts.maxpoint, infinite=True, base_wall_id=opts.base_wall_id)
    return Case(f"hertz_poly_{n}", opts, tables, walls, parts,
                note="Hertz E=5e7 Pa, nu=0.3, e=0.8, mu=0.4, mu_r=0.1, 41 types d=0.80..1.20 mm")


_bedgen = None


def _bedgen_lib():
    """libsdem_bedgen.so (host C, built by sdem_gb300.build)."""
    global _bedgen
    if _bedgen is None:
        import ctypes as C
        import os
        path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libsdem_bedgen.so")
        if not os.path.exists(path):
            raise RuntimeError(f"{path} is missing: build it with `python -m sdem_gb300.build`")
        lib = C.CDLL(path)
        dp = C.POINTER(C.c_double)
        lib.bedgen_rsp.argtypes = [C.c_int, dp, dp, dp, C.c_ulonglong, C.c_longlong, dp,
                                   C.POINTER(C.c_longlong), C.POINTER(C.c_int)]
        lib.bedgen_rsp.restype = C.c_int
        _bedgen = lib
    return _bedgen


def rsp_positions(radius: np.ndarray, lo, hi, seed: int, max_tries: int = 10_000_000) -> np.ndarray:
    """Seeded random sequential placement: sphere i (in index order) takes the
    first uniform random centre in [lo + r_i, hi - r_i] that overlaps no sphere
    placed before it (sdem_gb300/csrc/bedgen.c).  Raises when one sphere needs
    more than max_tries proposals."""
    import ctypes as C
    lib = _bedgen_lib()
    r = np.ascontiguousarray(radius, dtype=np.float64)
    lo_ = np.ascontiguousarray(lo, dtype=np.float64)
    hi_ = np.ascontiguousarray(hi, dtype=np.float64)
    pos = np.zeros((len(r), 3))
    dp = C.POINTER(C.c_double)
    props_ = C.c_longlong()
    fail = C.c_int()
    rc = lib.bedgen_rsp(len(r), r.ctypes.data_as(dp), lo_.ctypes.data_as(dp), hi_.ctypes.data_as(dp),
                        int(seed) & 0xFFFFFFFFFFFFFFFF, int(max_tries), pos.ctypes.data_as(dp), C.byref(props_),
                        C.byref(fail))
    if rc == 2:
        raise ValueError(f"rsp_positions: sphere {fail.value} found no free place in {max_tries} proposals")
    if rc:
        raise ValueError(f"rsp_positions: bad arguments or no memory (code {rc})")
    return pos


def hertz_poly_setup(box=(0.1, 0.6, 0.1), dt: float = 1.0e-6, pi: int = 2, pri: int = 2):
    """Options and walls of the 1M polydisperse Hertz configuration: Hertz,
    AB2, dt = 1e-6 s, gravity -y, a floor and four infinite side walls."""
    opts = Options(dt=dt, minpoint=(0.0, 0.0, 0.0), maxpoint=tuple(box), cf_type=props.CFT_NLIN,
                   pi_method=pi, pri_method=pri)
    walls = box_walls(opts.minpoint, opts.maxpoint, infinite=True, base_wall_id=opts.base_wall_id)
    return opts, walls


def hertz_poly_rsp_case(n: int = 1_000_000, seed: int = 2, box=(0.1, 0.6, 0.1), ntypes: int = 41,
                        fill: float = 0.25, dt: float = 1.0e-6, pi: int = 2, pri: int = 2, **table_kw) -> Case:
    """The 1M polydisperse Hertz configuration as placed, before settling:
    d uniform in [0.8, 1.2] mm as `ntypes` discrete types, seeded random
    sequential placement (rsp_positions) in the bottom of the 0.1 x 0.6 x 0.1 m
    box, as high as a solid fraction `fill` needs (0.218 m for 1M spheres at
    0.25), at rest, no contacts.  Floor and four side walls, gravity -y.
    table_kw passes other material values to hertz_poly_tables."""
    rng = np.random.default_rng(seed)
    diam, tables = hertz_poly_tables(ntypes, **table_kw)
    ptype = rng.integers(1, ntypes + 1, size=n).astype(np.int32)
    r = tables.radius[ptype - 1]
    height = float((4.0 / 3.0 * math.pi * r ** 3).sum() / fill / (box[0] * box[2]))
    if height > box[1]:
        raise ValueError("hertz_poly_rsp_case: the box is too short for this fill")
    pos = rsp_positions(r, (0.0, 0.0, 0.0), (box[0], height, box[2]), seed=seed)
    opts, walls = hertz_poly_setup(box, dt, pi, pri)
    parts = new_particles(pos, ptype, tables.radius, np.zeros((n, 3)), opts.tsize, opts.rsize)
    return Case(f"hertz_poly_rsp_{n}", opts, tables, walls, parts,
                note=f"random sequential placement at solid fraction {fill} up to y={height:.4f} m")


def random_cloud_case(n: int, seed: int, box=(0.01, 0.01, 0.01), ntypes: int = 5, cf_type: int = props.CFT_NLIN,
                      d_lo: float = 0.8e-3, d_hi: float = 1.2e-3, vmax: float = 0.3, pi: int = 2, pri: int = 2,
                      dt: float = 1.0e-6, overlap_frac: float = 0.02, density_frac: float = 0.45,
                      finite_walls: bool = False) -> Case:
    """Small dense cloud for parity tests: random sequential placement that
    accepts small overlaps (up to overlap_frac of the smaller diameter), so the
    first step already has many contacts; random velocities U(-vmax, vmax)
    and angular velocities."""
    rng = np.random.default_rng(seed)
    if cf_type == props.CFT_NLIN:
        diam, tables = hertz_poly_tables(ntypes, d_lo, d_hi)
    else:
        diam = np.linspace(d_lo, d_hi, ntypes) if ntypes > 1 else np.array([d_lo])
        E = props.lsd_youngs_for_stiffness(1.0e4, 0.05, float(diam.mean()), 2500.0, 0.3)
        c = (0.3, 0.2, 0.1, 0.9, 0.9)
        tables = props.build_tables(props.CFT_LSD, list(diam), [2500.0] * ntypes, [E] * ntypes, [0.3] * ntypes,
                                    c, [E], [0.3], c)
    ptype = rng.integers(1, ntypes + 1, size=n).astype(np.int32)
    r = 0.5 * diam[ptype - 1]
    pos = np.zeros((n, 3))
    placed = 0
    tries = 0
    lo = np.array([0.0, 0.0, 0.0])
    hi = np.array(box)
    while placed < n:
        tries += 1
        if tries > 200 * n:
            raise ValueError("random_cloud_case: box too small")
        p = rng.uniform(lo + r[placed] * 0.9, hi - r[placed] * 0.9)
        if placed:
            dd = np.sqrt(((pos[:placed] - p) ** 2).sum(axis=1))
            lim = r[:placed] + r[placed] - overlap_frac * 2.0 * np.minimum(r[:placed], r[placed])
            if np.any(dd < lim):
                continue
        pos[placed] = p
        placed += 1
    vel = rng.uniform(-vmax, vmax, size=(n, 3))
    opts = Options(dt=dt, minpoint=(0.0, 0.0, 0.0), maxpoint=tuple(box), cf_type=cf_type, pi_method=pi,
                   pri_method=pri)
    parts = new_particles(pos, ptype, tables.radius, vel, opts.tsize, opts.rsize)
    parts.rotVel[:] = rng.uniform(-50.0, 50.0, size=(n, 1, 3))
    if finite_walls:
        walls = box_walls(opts.minpoint, opts.maxpoint, infinite=False, base_wall_id=opts.base_wall_id)
    else:
        walls = box_walls(opts.minpoint, opts.maxpoint, infinite=True, base_wall_id=opts.base_wall_id)
    return Case(f"cloud_{n}_{seed}", opts, tables, walls, parts)


def lattice_cloud_case(n: int, seed: int, nn: float = 1.05e-3, ntypes: int = 7, cf_type: int = props.CFT_NLIN,
                       d_lo: float = 0.8e-3, d_hi: float = 1.2e-3, vmax: float = 0.3, pi: int = 2, pri: int = 2,
                       dt: float = 1.0e-6, jitter: float = 0.02e-3, finite_walls: bool = False,
                       margin: float = 0.8e-3) -> Case:
    """Dense cloud for parity tests: an FCC lattice with nearest-neighbour
    distance `nn`, random types (diameters spread over [d_lo, d_hi]), jitter
    U(-jitter, jitter), velocities U(-vmax, vmax) and angular velocities
    U(-50, 50) rad/s.  Neighbours whose radii sum exceeds their distance start
    in contact, so the first step has several contacts per sphere."""
    rng = np.random.default_rng(seed)
    if cf_type == props.CFT_NLIN:
        diam, tables = hertz_poly_tables(ntypes, d_lo, d_hi)
    else:
        diam = np.linspace(d_lo, d_hi, ntypes) if ntypes > 1 else np.array([0.5 * (d_lo + d_hi)])
        E = props.lsd_youngs_for_stiffness(1.0e4, 0.05, float(diam.mean()), 2500.0, 0.3)
        c = (0.3, 0.2, 0.1, 0.9, 0.9)
        tables = props.build_tables(props.CFT_LSD, list(diam), [2500.0] * ntypes, [E] * ntypes, [0.3] * ntypes,
                                    c, [E], [0.3], c)
    cube = nn * math.sqrt(2.0)
    m = int(math.ceil((n / 4.0) ** (1.0 / 3.0)))
    basis = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    g = np.stack(np.meshgrid(np.arange(m), np.arange(m), np.arange(m), indexing="ij"), -1).reshape(-1, 3)
    pos = ((g[:, None, :] + basis[None, :, :]).reshape(-1, 3) * cube)[:n] + margin
    pos = pos + rng.uniform(-jitter, jitter, size=pos.shape)
    box = tuple(float(v) for v in (pos.max(axis=0) + margin))
    ptype = rng.integers(1, ntypes + 1, size=n).astype(np.int32)
    vel = rng.uniform(-vmax, vmax, size=(n, 3))
    opts = Options(dt=dt, minpoint=(0.0, 0.0, 0.0), maxpoint=box, cf_type=cf_type, pi_method=pi, pri_method=pri)
    parts = new_particles(pos, ptype, tables.radius, vel, opts.tsize, opts.rsize)
    parts.rotVel[:] = rng.uniform(-50.0, 50.0, size=(n, 1, 3))
    # spheres near the walls already touch them
    walls = box_walls((margin * 0.4, margin * 0.4, margin * 0.4), tuple(b - margin * 0.4 for b in box),
                      infinite=not finite_walls, base_wall_id=opts.base_wall_id)
    return Case(f"lattice_{n}_{seed}", opts, tables, walls, parts)


def periodic_lattice_case(n: int, seed: int, periodic=(1, 1, 1), nn: float = 1.05e-3, vmax: float = 0.3,
                          offset: float = 0.3e-3, **kw) -> Case:
    """lattice_cloud_case in a box whose periodic sides are whole FCC periods
    (m cubes of nn*sqrt(2)), so spheres near a periodic face touch the images
    of spheres near the opposite face exactly as they touch their lattice
    neighbours.  Non-periodic sides get plane walls that the outermost spheres
    touch by at most 10 um."""
    jitter = kw.get("jitter", 0.02e-3)
    cube = nn * math.sqrt(2.0)
    if not (offset + jitter < 0.5 * cube):
        raise ValueError("offset too large: the lattice would leave its periodic box")
    m = int(math.ceil((n / 4.0) ** (1.0 / 3.0)))
    case = lattice_cloud_case(n, seed, nn=nn, vmax=vmax, margin=offset, **kw)
    p = case.particles
    pos, r = p.posR[:, :3], p.posR[:, 3]
    hi = list(case.opts.maxpoint)
    wlo, whi = [0.0] * 3, [0.0] * 3
    for k in range(3):
        if periodic[k]:
            hi[k] = m * cube
        wlo[k] = float((pos[:, k] - r).min()) + 1.0e-5
        whi[k] = float((pos[:, k] + r).max()) - 1.0e-5
    opts = replace(case.opts, maxpoint=tuple(hi), periodic=tuple(int(v) for v in periodic))
    walls = box_walls(tuple(wlo), tuple(whi), base_wall_id=opts.base_wall_id,
                      skip_axes=[k for k in range(3) if periodic[k]])
    return Case(f"periodic_{n}_{seed}_{''.join(str(int(v)) for v in periodic)}", opts, case.tables, walls, p)


def hopper_case(n: int, seed: int, width: float = 20.0e-3, outlet: float = 6.0e-3, angle_deg: float = 60.0,
                d_small: float = 0.5e-3, d_large: float = 1.5e-3, frac_large: float = 0.3, e_n: float = 0.7,
                mu: float = 0.5, E: float = 5.0e7, dt: float = 5.0e-7, vfall: float = 0.5, pi: int = 2,
                pri: int = 2) -> Case:
    """A small hopper of the bidisperse kind: Hertz spheres of diameters
    d_small and d_large (by count (1 - frac_large) : frac_large) in a square
    funnel of four finite inclined planes (angle_deg from the horizontal) whose
    lower edges frame a square outlet, with four finite vertical planes
    holding a column above it.  Below the outlet the domain ends at y = 0, so
    spheres that fall through leave it and are deleted (one rank,
    Comm_For_Exchange).  The spheres start on a jittered cubic lattice (pitch
    0.97 d_large, so neighbouring large spheres and the walls already touch)
    filling the outlet throat and the funnel from the bottom up, moving down
    at up to vfall m/s; the ones in the throat fall fast (40-80 m/s) so that
    a few steps already delete some."""
    rng = np.random.default_rng(seed)
    diam = np.array([d_small, d_large])
    coefs = (mu, mu, 0.1, e_n, e_n)
    tables = props.build_tables(props.CFT_NLIN, list(diam), [2500.0] * 2, [E] * 2, [0.3] * 2, coefs, [E], [0.3],
                                coefs)
    W, a = width, outlet
    c = 0.5 * W
    run = 0.5 * (W - a)
    drop = run * math.tan(math.radians(angle_deg))
    y_o = 4.0e-3                       # outlet level; the throat below it is open down to y = 0
    y_t = y_o + drop                   # top of the funnel
    y_top = y_t + 0.75 * W             # top of the column
    centre = np.array([c, 0.5 * (y_o + y_t), c])
    walls = WallSet()
    kw = dict(infinite=False, base_wall_id=10000000)

    def add(quad):
        q = [np.array(p, dtype=float) for p in quad]
        nrm = np.cross(q[1] - q[0], q[2] - q[0])
        if np.dot(nrm, centre - q[0]) < 0:     # normals point into the hopper
            q = q[::-1]
        walls.add(*(tuple(p) for p in q), **kw)

    lo, hi = c - 0.5 * a, c + 0.5 * a
    # inclined sides (z = 0, z = W, x = 0, x = W edges at the top)
    add([(0, y_t, 0), (W, y_t, 0), (hi, y_o, lo), (lo, y_o, lo)])
    add([(0, y_t, W), (W, y_t, W), (hi, y_o, hi), (lo, y_o, hi)])
    add([(0, y_t, 0), (0, y_t, W), (lo, y_o, hi), (lo, y_o, lo)])
    add([(W, y_t, 0), (W, y_t, W), (hi, y_o, hi), (hi, y_o, lo)])
    # vertical column
    add([(0, y_t, 0), (W, y_t, 0), (W, y_top, 0), (0, y_top, 0)])
    add([(0, y_t, W), (W, y_t, W), (W, y_top, W), (0, y_top, W)])
    add([(0, y_t, 0), (0, y_t, W), (0, y_top, W), (0, y_top, 0)])
    add([(W, y_t, 0), (W, y_t, W), (W, y_top, W), (W, y_top, 0)])
    ptype = np.where(rng.uniform(size=4 * n) < frac_large, 2, 1).astype(np.int32)
    pitch = 0.97 * d_large
    g = np.arange(0.5 * pitch, max(W, y_top) + pitch, pitch)
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    pts = np.stack([X.ravel(), Y.ravel(), Z.ravel()], 1)
    pts = pts + rng.uniform(-0.02 * pitch, 0.02 * pitch, size=pts.shape)
    rmax = 0.5 * d_large
    inside = np.ones(len(pts), bool)
    for w in walls.walls:
        nrm, dd = w[12:15], w[15]
        inside &= (pts @ nrm + dd) >= 0.95 * rmax
    throat = ((np.abs(pts[:, 0] - c) < 0.5 * a - 1.1 * rmax) & (np.abs(pts[:, 2] - c) < 0.5 * a - 1.1 * rmax)
              & (pts[:, 1] > 0.6 * rmax) & (pts[:, 1] < y_o))
    ok = (inside & (pts[:, 1] >= y_o) & (pts[:, 1] < y_top - rmax)) | throat
    pts = pts[ok]
    pts = pts[np.argsort(pts[:, 1], kind="stable")][:n]
    if len(pts) < n:
        raise ValueError("hopper_case: the hopper holds fewer lattice sites than n")
    ptype = ptype[:n]
    vel = np.zeros((n, 3))
    vel[:, 1] = -rng.uniform(0.0, vfall, size=n)
    in_throat = pts[:, 1] < y_o
    vel[in_throat, 1] = -rng.uniform(40.0, 80.0, size=int(in_throat.sum()))
    vel[:, 0] = rng.uniform(-0.05, 0.05, size=n)
    vel[:, 2] = rng.uniform(-0.05, 0.05, size=n)
    opts = Options(dt=dt, minpoint=(-1.0e-3, 0.0, -1.0e-3), maxpoint=(W + 1.0e-3, y_top + 1.0e-3, W + 1.0e-3),
                   cf_type=props.CFT_NLIN, pi_method=pi, pri_method=pri)
    parts = new_particles(pts, ptype, tables.radius, vel, opts.tsize, opts.rsize)
    return Case(f"hopper_{n}_{seed}", opts, tables, walls, parts)


def fixed_floor_case(n: int, seed: int, **kw) -> Case:
    """lattice_cloud_case whose floor wall is replaced by a rough floor of
    fixed spheres (one under every sphere of the lowest layer, overlapping it
    by 2%), plus a few fixed spheres in place of moving ones inside the
    cloud: moving-fixed pairs are found both from fixed and from moving
    targets."""
    case = lattice_cloud_case(n, seed, **kw)
    rng = np.random.default_rng(seed + 1000)
    p = case.particles
    ft = 1                                              # the fixed spheres' type
    rf = float(case.tables.radius[ft - 1])
    lo = p.posR[:, :3].min(axis=0)
    hi = p.posR[:, :3].max(axis=0)
    low = np.nonzero(p.posR[:, 1] < p.posR[:, 1].min() + 0.5 * float(case.tables.radius.min()))[0]
    # one fixed sphere under every sphere of the lowest layer, 2% into it
    floor = p.posR[low, :3].copy()
    floor[:, 1] -= 0.98 * (p.posR[low, 3] + rf)
    floor[:, [0, 2]] += rng.uniform(-0.1 * rf, 0.1 * rf, size=(len(floor), 2))
    y_floor = float(floor[:, 1].min())
    # a few inside the cloud, in place of moving spheres
    k = max(1, n // 50)
    pick = rng.choice(np.setdiff1d(np.arange(n), low), size=k, replace=False)
    inner = p.posR[np.sort(pick), :3].copy()
    keep = np.setdiff1d(np.arange(n), pick)
    parts = p.take(keep)
    parts.id[:] = np.arange(1, len(keep) + 1, dtype=np.int32)
    pos = np.concatenate([floor, inner])
    nmax = int(parts.id.max())
    fixed = FixedSpheres(id=np.arange(nmax + 1, nmax + 1 + len(pos), dtype=np.int32),
                         ptype=np.full(len(pos), ft, np.int32), pos=pos)
    walls = WallSet()
    for w, f in zip(case.walls.walls[1:], case.walls.flags[1:]):   # no floor wall
        walls.walls.append(w)
        walls.flags.append(f)
    lo_dom = list(case.opts.minpoint)
    lo_dom[1] = min(lo_dom[1], y_floor - 2.0 * rf)
    opts = replace(case.opts, minpoint=tuple(lo_dom))
    return Case(f"fixedfloor_{n}_{seed}", opts, case.tables, walls, parts, fixed=fixed)


def sandbox_case(rng: np.random.Generator, index: int, n_lo: int = 2000, n_hi: int = 50000,
                 layout: str = "lattice", cf_type: Optional[int] = None) -> Case:
    """One sandbox of the batched workload: n ~ U{n_lo..n_hi} spheres with d
    uniform in [0.8, 1.2] mm (five types, density 2500 kg/m^3), sliding
    friction U(0.1, 0.5), restitution U(0.5, 0.95), linear spring-dashpot or
    Hertz-Mindlin by a coin flip, dt = 2e-6 s, AB2; a jittered simple-cubic
    lattice (pitch 1.3 d_max) filling a box of aspect ratios x:y:z = a:1:b with
    a, b ~ U(0.5, 2), five infinite walls, velocities U(-0.05, 0.05) m/s.  The
    parameters are drawn from `rng` in a fixed order (cf_type, when given,
    replaces the coin flip's model after the flip).  layout="deposited"
    puts the same spheres, on the same footprint, as a bed already in
    contact: deposited_positions (column grid spacing 1.1 d_max, jitter
    0.04 d_max), each sphere resting on its support without overlap, at
    rest."""
    n = int(rng.integers(n_lo, n_hi + 1))
    mu = float(rng.uniform(0.1, 0.5))
    e_n = float(rng.uniform(0.5, 0.95))
    cf = props.CFT_LSD if rng.uniform() < 0.5 else props.CFT_NLIN
    if cf_type is not None:
        cf = cf_type
    a, b = float(rng.uniform(0.5, 2.0)), float(rng.uniform(0.5, 2.0))
    seed = int(rng.integers(0, 2**31 - 1))
    ntypes = 5
    diam = np.linspace(0.8e-3, 1.2e-3, ntypes)
    coefs = (mu, mu, 0.1, e_n, e_n)
    if cf == props.CFT_NLIN:
        E = 5.0e7
    else:
        E = props.lsd_youngs_for_stiffness(1.0e4, 0.05, float(diam.mean()), 2500.0, 0.3)
    tables = props.build_tables(cf, list(diam), [2500.0] * ntypes, [E] * ntypes, [0.3] * ntypes, coefs, [E], [0.3],
                                coefs)
    pitch = 1.3 * diam[-1]
    k = (n / (a * b)) ** (1.0 / 3.0)
    nx, ny, nz = max(1, int(math.ceil(a * k))), max(1, int(math.ceil(k))), max(1, int(math.ceil(b * k)))
    while nx * ny * nz < n:
        ny += 1
    g = np.stack(np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij"), -1).reshape(-1, 3)
    # fill from the floor up
    g = g[np.lexsort((g[:, 2], g[:, 0], g[:, 1]))][:n]
    r = np.random.default_rng(seed)
    pos = (g + 0.5) * pitch + 0.2e-3 + r.uniform(-0.05, 0.05, size=(n, 3)) * pitch
    box = (nx * pitch + 0.4e-3, (ny + 2) * pitch + 0.4e-3, nz * pitch + 0.4e-3)
    ptype = r.integers(1, ntypes + 1, size=n).astype(np.int32)
    vel = r.uniform(-0.05, 0.05, size=(n, 3))
    if layout == "deposited":
        dmax = float(diam[-1])
        tall = (box[0], 1.0e3, box[2])
        pos = deposited_positions(r, diam[ptype - 1], tall, 0.0, 0.0, 1.1 * dmax, 0.04 * dmax)
        box = (box[0], float(pos[:, 1].max()) + 3.0 * dmax, box[2])
        vel = np.zeros((n, 3))
    elif layout != "lattice":
        raise ValueError(f"sandbox_case: unknown layout {layout!r}")
    opts = Options(dt=2.0e-6, minpoint=(0.0, 0.0, 0.0), maxpoint=box, cf_type=cf, pi_method=2, pri_method=2)
    parts = new_particles(pos, ptype, tables.radius, vel, opts.tsize, opts.rsize)
    walls = box_walls(opts.minpoint, opts.maxpoint, infinite=True, base_wall_id=opts.base_wall_id, skip_axes=())
    return Case(f"sandbox_{index}", opts, tables, walls, parts,
                note=f"{'Hertz' if cf == props.CFT_NLIN else 'LSD'} mu={mu:.3f} e={e_n:.3f} n={n}")


def scaled(case: Case, **opt_changes) -> Case:
    return replace(case, opts=replace(case.opts, **opt_changes))
