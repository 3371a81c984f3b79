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

from .beds import Particles

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
    ids = p.id
    index = {}
    pairs = np.zeros((len(owner), 2), np.int32)
    recs = []
    for k in range(len(owner)):
        g = int(ids[owner[k]])
        q = int(partner[k])
        # A pair of local spheres is listed under both, with one record; a
        # contact with a periodic image is listed under its local sphere only,
        # and two spheres can each touch the other's image (two records under
        # the same two ids).  Listings share a record when their ids and their
        # history agree bit for bit.
        h = np.array([tand[k, 0], tand[k, 1], tand[k, 2], vrel[k]], np.float64).tobytes()
        key = (g, q) if q > base_wall_id else (min(g, q), max(g, q), h)
        if key not in index:
            index[key] = len(recs) + 1
            recs.append((tand[k, 0], tand[k, 1], tand[k, 2], vrel[k]))
        pairs[k] = (q, index[key])
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
        np.array(recs, dtype=np.float64).reshape(-1, 4).tofile(f)


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
    start = np.concatenate([[0], np.cumsum(ncv)[:-1]]).astype(np.int64)
    own, par, td, vr = [], [], [], []
    for new_i, i in enumerate(sel):
        for k in range(start[i], start[i] + ncv[i]):
            q, j = int(pairs[k, 0]), int(pairs[k, 1])
            own.append(new_i)
            par.append(q)
            td.append(tan[j - 1, :3])
            vr.append(tan[j - 1, 3])
    contacts = (np.array(own, np.int32), np.array(par, np.int32), np.array(td, np.float64).reshape(-1, 3),
                np.array(vr, np.float64))
    return parts, contacts
