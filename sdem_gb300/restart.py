"""Reader and writer of the reference's restart file (RestartFor<RunName><itime>).

Byte layout (native endian, int32 and float64), as PIO_Write_Restart writes it
(src/DEM/Prtcl_IOAndVisu.f90:849-1031) and PIO_Read_Restart/PIO_RestartCL read
it (:731-844, :296-377), for the standalone build (no CFDDEM block):

    np                          int32
    nCntctTotal                 int32   (listed contact entries, see below)
    np x real3                  positions
    np x (id, pType, usrMark)   int32 x 3
    np x nreal3 x real3         linVel(1:tsize), linAcc(1:tsize), theta,
                                rotVel(1:rsize), rotAcc(1:rsize)
                                (nreal3 = 2*(1+tsize+rsize)-1)
    np x ncv                    int32, contacts per particle (walls included)
    nCntctTotal x (id, k)       int32 pairs: partner id and the 1-based index of
                                the contact's record in the TanDel block; a
                                particle-particle contact is listed under both
                                particles with the same k
    nTanDel x real4             TanDelta (x, y, z), VelRel_Init

The reference numbers TanDel records in the order of its contact container's
slots (CL_Prepare_Restart, Prtcl_CL_and_CF.f90:344-359), an artefact of its
free list; this writer numbers them in order of first listing, one record per
contact (the two listings of a pair of local spheres share it; contacts with
periodic images have their own).  Its reader
resolves the indices either way, so files interoperate; byte equality with a
file the reference wrote holds up to that numbering.
"""
from __future__ import annotations

from typing import Optional, Tuple

import numpy as np

from .beds import FixedSpheres, Particles

NCV_LIMIT = 20   # CL_Count_Cntctlink aborts above this (Prtcl_CL_and_CF.f90:641,648)


class RestartError(RuntimeError):
    pass


def write_restart(path: str, p: Particles, contacts: Optional[tuple], tsize: int, rsize: int,
                  base_wall_id: int = 10000000) -> None:
    """contacts = (owner_idx, partner_id, tandelta (nc,3), velrel), records grouped
    by owner as sdem_download_contacts returns them; None for no contacts."""
    n = p.n
    if contacts is None:
        owner = np.zeros(0, np.int32)
        partner = np.zeros(0, np.int32)
        tand = np.zeros((0, 3))
        vrel = np.zeros(0)
    else:
        owner, partner, tand, vrel = (np.asarray(a) for a in contacts)
    order = np.argsort(owner, kind="stable")
    owner, partner, tand, vrel = owner[order], partner[order], tand[order], vrel[order]
    ncv = np.bincount(owner, minlength=n).astype(np.int32) if len(owner) else np.zeros(n, np.int32)
    if len(ncv) and ncv.max(initial=0) > NCV_LIMIT:
        raise RestartError("CL_Count_Cntctlink: so big ncv (more than 20 contacts on one particle)")
    # A pair of local spheres is listed under both, with one record; a
    # contact with a periodic image is listed under its local sphere only,
    # and two spheres can each touch the other's image (two records under
    # the same two ids).  Listings share a record when their ids and their
    # history agree bit for bit; records are numbered in order of first
    # listing.
    g = np.asarray(p.id, np.int64)[owner] if len(owner) else np.zeros(0, np.int64)
    q = partner.astype(np.int64)
    wall = q > base_wall_id
    a = np.where(wall, g, np.minimum(g, q))
    b = np.where(wall, q, np.maximum(g, q))
    hist = np.ascontiguousarray(np.concatenate([tand.reshape(-1, 3), vrel.reshape(-1, 1)], axis=1),
                                dtype=np.float64).view(np.int64)
    # listings grouped by the two ids (stable: a group's first entry is its
    # earliest listing), then split where the history differs; two ids are
    # listed at most twice in a valid list, and longer runs take the general
    # grouping over ids and history together
    ab = (a << 32) | (b & 0xFFFFFFFF)
    o = np.argsort(ab, kind="stable")
    sab = ab[o]
    run_start = np.ones(len(o), bool)
    if len(o) > 1:
        run_start[1:] = sab[1:] != sab[:-1]
    starts = np.flatnonzero(run_start)
    if len(o) and np.diff(np.append(starts, len(o))).max() > 2:
        keys = np.ascontiguousarray(np.concatenate([a[:, None], b[:, None], hist], axis=1))
        kv = keys.view(np.dtype((np.void, keys.shape[1] * keys.itemsize))).ravel()
        _, first, inverse = np.unique(kv, return_index=True, return_inverse=True)
        group_of = inverse.ravel()
    else:
        new_group = run_start.copy()
        if len(o) > 1:
            new_group[1:] |= np.any(hist[o][1:] != hist[o][:-1], axis=1)
        gid = np.cumsum(new_group) - 1
        first = o[new_group]
        group_of = np.empty(len(o), np.int64)
        group_of[o] = gid
    rank = np.empty(len(first), np.int64)
    rank[np.argsort(first, kind="stable")] = np.arange(len(first))
    index = rank[group_of] + 1                    # 1-based record of each listing
    pairs = np.stack([partner.astype(np.int32), index.astype(np.int32)], axis=1) if len(owner) else \
        np.zeros((0, 2), np.int32)
    firsts = np.sort(first)
    recs = np.concatenate([tand.reshape(-1, 3)[firsts], vrel.reshape(-1)[firsts, None]], axis=1) if len(owner) \
        else np.zeros((0, 4))
    nreal3 = 2 * (1 + tsize + rsize) - 1
    with open(path, "wb") as f:
        np.array([n, len(owner)], dtype=np.int32).tofile(f)
        np.ascontiguousarray(p.posR[:, :3], dtype=np.float64).tofile(f)
        np.stack([p.id, p.ptype, p.usrmark], axis=1).astype(np.int32).tofile(f)
        blk = np.concatenate([p.linVel.reshape(n, tsize, 3), p.linAcc.reshape(n, tsize, 3),
                              p.theta.reshape(n, 1, 3), p.rotVel.reshape(n, rsize, 3),
                              p.rotAcc.reshape(n, rsize, 3)], axis=1)
        assert blk.shape[1] == nreal3
        np.ascontiguousarray(blk, dtype=np.float64).tofile(f)
        ncv.tofile(f)
        pairs.tofile(f)
        np.ascontiguousarray(recs, dtype=np.float64).reshape(-1, 4).tofile(f)


def read_restart(path: str, tsize: int, rsize: int, radius_of_type: np.ndarray,
                 dom_min=None, dom_max=None) -> Tuple[Particles, tuple]:
    """Returns (particles, contacts) as PIO_Read_Restart + PIO_RestartCL build them
    on one rank: particles outside [dom_min, dom_max) are skipped, the radius
    comes from the type (Prtcl_IOAndVisu.f90:809).  A path ending in .gz is
    read through gzip."""
    if path.endswith(".gz"):
        import gzip
        with gzip.open(path, "rb") as f:
            raw = np.frombuffer(f.read(), dtype=np.uint8)
    else:
        raw = np.fromfile(path, dtype=np.uint8)
    off = 0

    def take(dtype, count):
        nonlocal off
        a = np.frombuffer(raw, dtype=dtype, count=count, offset=off)
        off += a.nbytes
        return a

    n, nct = (int(v) for v in take(np.int32, 2))
    pos = take(np.float64, 3 * n).reshape(n, 3)
    ints = take(np.int32, 3 * n).reshape(n, 3)
    nreal3 = 2 * (1 + tsize + rsize) - 1
    blk = take(np.float64, 3 * nreal3 * n).reshape(n, nreal3, 3)
    ncv = take(np.int32, n)
    pairs = take(np.int32, 2 * nct).reshape(nct, 2)
    ntan = (raw.size - off) // 32
    tan = take(np.float64, 4 * ntan).reshape(ntan, 4)
    keep = np.ones(n, bool)
    if dom_min is not None:
        for k in range(3):
            keep &= (pos[:, k] >= dom_min[k]) & (pos[:, k] < dom_max[k])
    sel = np.nonzero(keep)[0]
    posR = np.zeros((len(sel), 4))
    posR[:, :3] = pos[sel]
    posR[:, 3] = np.asarray(radius_of_type)[ints[sel, 1] - 1]
    t0, t1, t2 = tsize, 2 * tsize, 2 * tsize + 1
    parts = Particles(id=ints[sel, 0].copy(), ptype=ints[sel, 1].copy(), usrmark=ints[sel, 2].copy(), posR=posR,
                      linVel=blk[sel, :t0].copy(), linAcc=blk[sel, t0:t1].copy(), theta=blk[sel, t1].copy(),
                      rotVel=blk[sel, t2:t2 + rsize].copy(), rotAcc=blk[sel, t2 + rsize:t2 + 2 * rsize].copy())
    # every listing with its owner's position in the file; the kept owners
    # are renumbered in order
    owner_all = np.repeat(np.arange(n, dtype=np.int64), ncv.astype(np.int64))
    new_index = np.full(n, -1, np.int64)
    new_index[sel] = np.arange(len(sel))
    keep_l = new_index[owner_all] >= 0
    rec = pairs[keep_l, 1].astype(np.int64) - 1
    contacts = (new_index[owner_all[keep_l]].astype(np.int32), pairs[keep_l, 0].astype(np.int32),
                np.ascontiguousarray(tan[rec, :3]), np.ascontiguousarray(tan[rec, 3]))
    return parts, contacts


# FixedSpheresCoord.dat: per fixed sphere x, y, z, diameter (float64) and its
# type (int32), 36 bytes, packed (the MPI struct of PIO_ReadFixedCoord)
FIXED_RECORD = np.dtype([("pos", "<f8", (3,)), ("diam", "<f8"), ("ptype", "<i4")])


def write_fixed_coords(path: str, pos: np.ndarray, ptype: np.ndarray, radius_of_type: np.ndarray) -> None:
    """FixedSpheresCoord.dat for the fixed spheres at `pos` of types `ptype`
    (1-based; the diameter written is twice the type's radius)."""
    rec = np.zeros(len(pos), FIXED_RECORD)
    rec["pos"] = pos
    rec["ptype"] = ptype
    rec["diam"] = 2.0 * np.asarray(radius_of_type)[np.asarray(ptype) - 1]
    rec.tofile(path)


def read_fixed_coords(path: str, num_prtcl_fix: int, num_prtcl: int, radius_of_type: np.ndarray,
                      dom_min, dom_max) -> FixedSpheres:
    """PIO_ReadFixedCoord (Prtcl_IOAndVisu.f90:163-291) on one rank: the
    fixed spheres of the file, numbered file position + numPrtcl (above
    every moving id), the radius from the type.  The checks of the reference
    raise RestartError: a file whose size is not numPrtclFix records ("file
    byte wrong"), a diameter that differs from its type's by more than 1e-6
    relative ("Diameter not coordinate"), a sphere outside [dom_min, dom_max)
    (nfix_sum /= numPrtclFix)."""
    import os
    if os.path.getsize(path) != FIXED_RECORD.itemsize * num_prtcl_fix:
        raise RestartError("PIO_ReadFixedCoord: file byte wrong")
    rec = np.fromfile(path, dtype=FIXED_RECORD)
    ptype = rec["ptype"].astype(np.int32)
    radius = np.asarray(radius_of_type, np.float64)[ptype - 1]
    if np.any(np.abs(2.0 * radius / rec["diam"] - 1.0) > 1.0e-6):
        raise RestartError("PIO_ReadFixedCoord: Diameter not coordinate")
    pos = rec["pos"].astype(np.float64)
    inside = np.ones(len(rec), bool)
    for k in range(3):
        inside &= (pos[:, k] >= dom_min[k]) & (pos[:, k] < dom_max[k])
    if not inside.all():
        raise RestartError("PIO_ReadFixedCoord: nfix_sum /= numPrtclFix")
    ids = (np.arange(1, len(rec) + 1) + num_prtcl).astype(np.int32)
    return FixedSpheres(id=ids, ptype=ptype, pos=pos)
