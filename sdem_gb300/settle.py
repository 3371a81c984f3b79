"""Gravity settling of a placed bed with the GPU path itself.

The 1M polydisperse Hertz configuration is a seeded random sequential
placement (beds.hertz_poly_rsp_case) that settles under gravity.  Settling it
at the configuration's own time step would take ~0.2 s of simulated time,
200,000 steps.  The preparation therefore runs in stages, all in the
configuration's stiffness (E = 5e7 Pa, so the overlaps never have to shrink
later):

  1. collapse: restitution 0.3 at dt = 4e-6 s (12 steps per contact at the
     ~1.5 m/s impact speed), 42,000 steps: the packing falls into contact;
  2. damp: restitution 0.1 at dt = 4e-6 s, 6,000 steps, every velocity and
     acceleration set to zero every 1,500 steps (a quench): the slow
     breathing of the bed on its contacts dies out;
  3. the configuration itself (restitution 0.8, friction 0.4, dt = 1e-6 s),
     started from rest (one quench), 3,000 steps.

Each stage is a new handle that receives the previous one's particles and
contact list (spring history included), as a restart would.  The result is a
Case in the configuration's material with the settled state and contact list.
The settled state is cached on disk (keyed by the inputs and the library's
content stamp), because the preparation takes about a minute on one GB300.
"""
from __future__ import annotations

import hashlib
import json
import os
import time
from dataclasses import asdict, dataclass, replace
from typing import Callable, List, Optional, Sequence

import numpy as np

from . import beds

HERE = os.path.dirname(os.path.abspath(__file__))
CACHE_DIR = os.path.join(os.path.dirname(HERE), ".bedcache")


@dataclass(frozen=True)
class Stage:
    steps: int
    dt: float
    youngs: float
    restitution: float
    quench_every: int = 0   # >0: velocities and accelerations set to zero every that many steps


STAGES = (Stage(42000, 4.0e-6, 5.0e7, 0.3),
          Stage(6000, 4.0e-6, 5.0e7, 0.1, quench_every=1500),
          Stage(3000, 1.0e-6, 5.0e7, 0.8, quench_every=3000))


def quench(p: beds.Particles) -> beds.Particles:
    """The state at rest: linear and angular velocities and accelerations
    (every Adams-Bashforth level) set to zero; positions and rotations kept."""
    q = p.copy()
    for a in (q.linVel, q.linAcc, q.rotVel, q.rotAcc):
        a[...] = 0.0
    return q


def bed_stats(state: beds.Particles, counters: dict) -> dict:
    v = np.linalg.norm(state.linVel[:, 0, :], axis=1)
    top = state.posR[:, 1] + state.posR[:, 3]
    return {"n": int(state.n), "pp": int(counters["pp"]), "pw": int(counters["pw"]),
            "pp_per_particle": counters["pp"] / max(state.n, 1),
            "v_max": float(v.max(initial=0.0)), "v_mean": float(v.mean()) if state.n else 0.0,
            "v_median": float(np.median(v)) if state.n else 0.0,
            "height": float(np.quantile(top, 0.999)) if state.n else 0.0}


def settle(placed: beds.Case, stages: Sequence[Stage], final_tables, final_dt: float, chunk: int = 1000,
           progress: Optional[Callable[[int, int, dict], None]] = None):
    """Runs `stages` on the GPU from `placed`; returns (case, log): the case
    carries final_tables, final_dt and the settled particles and contacts."""
    from .capi import DEMSystem
    ntypes = placed.tables.n_types
    parts, contacts = placed.particles, placed.contacts
    log: List[dict] = []
    for k, st in enumerate(stages):
        _, tables = beds.hertz_poly_tables(ntypes, E=st.youngs, e_n=st.restitution)
        case = replace(placed, opts=replace(placed.opts, dt=st.dt), tables=tables, particles=parts,
                       contacts=contacts)
        t0 = time.perf_counter()
        with DEMSystem(case) as h:
            if st.quench_every:
                h.upload(quench(parts))
                if contacts is not None:
                    h.upload_contacts(*contacts)
            step = st.quench_every if st.quench_every else chunk
            done = 0
            while done < st.steps:
                m = min(step, st.steps - done)
                h.step(m)
                done += m
                if progress is not None:
                    progress(k, done, bed_stats(h.state(), h.counters()))
                if st.quench_every and done % st.quench_every == 0 and done < st.steps:
                    cur, cc = h.state(), h.contacts()
                    h.upload(quench(cur))
                    h.upload_contacts(*cc)
            parts = h.state()
            contacts = h.contacts()
            entry = {"stage": k, **asdict(st), "wall_s": time.perf_counter() - t0, **bed_stats(parts, h.counters())}
        log.append(entry)
    out = replace(placed, opts=replace(placed.opts, dt=final_dt), tables=final_tables, particles=parts,
                  contacts=contacts)
    return out, log


def _lib_stamp() -> str:
    parts = []
    for name in ("libsdem_gpu.so.stamp", "libsdem_bedgen.so.stamp"):
        try:
            with open(os.path.join(HERE, name)) as f:
                parts.append(f.read().strip())
        except OSError:
            parts.append("none")
    return ":".join(parts)


def settled_hertz_poly_case(n: int = 1_000_000, seed: int = 2, fill: float = 0.25, box=(0.1, 0.6, 0.1),
                            stages: Sequence[Stage] = STAGES, cache: bool = True,
                            progress: Optional[Callable[[int, int, dict], None]] = None) -> beds.Case:
    """The 1M polydisperse Hertz configuration settled under gravity: placed by
    beds.hertz_poly_rsp_case(n, seed, box, fill), settled by `stages` on the
    GPU, in the configuration's material (E = 5e7 Pa, restitution 0.8,
    friction 0.4) at dt = 1e-6 s.  The case's note holds the settling log
    (JSON)."""
    box = tuple(float(v) for v in box)
    key_src = json.dumps({"n": n, "seed": seed, "fill": fill, "box": box, "stages": [asdict(s) for s in stages],
                          "lib": _lib_stamp()}, sort_keys=True)
    key = hashlib.sha256(key_src.encode()).hexdigest()[:20]
    path = os.path.join(CACHE_DIR, f"hertz_poly_settled_{n}_{seed}_{key}.npz")
    if cache and os.path.exists(path):
        with np.load(path) as z:
            parts = beds.Particles(z["id"], z["ptype"], z["usrmark"], z["posR"], z["linVel"], z["linAcc"],
                                   z["theta"], z["rotVel"], z["rotAcc"])
            contacts = (z["c_owner"], z["c_partner"], z["c_tandelta"], z["c_velrel"])
            log = json.loads(str(z["log"]))
        _, tables = beds.hertz_poly_tables(41)
        opts, walls = beds.hertz_poly_setup(box)
        case = beds.Case(f"hertz_poly_settled_{n}", opts, tables, walls, parts, contacts=contacts)
    else:
        placed = beds.hertz_poly_rsp_case(n, seed, box=box, fill=fill)
        _, tables = beds.hertz_poly_tables(placed.tables.n_types)
        case, log = settle(placed, stages, tables, 1.0e-6, progress=progress)
        case = replace(case, name=f"hertz_poly_settled_{n}")
        if cache:
            os.makedirs(CACHE_DIR, exist_ok=True)
            p, c = case.particles, case.contacts
            tmp = f"{path}.{os.getpid()}.tmp.npz"
            np.savez(tmp, id=p.id, ptype=p.ptype, usrmark=p.usrmark, posR=p.posR, linVel=p.linVel,
                     linAcc=p.linAcc, theta=p.theta, rotVel=p.rotVel, rotAcc=p.rotAcc, c_owner=c[0],
                     c_partner=c[1], c_tandelta=c[2], c_velrel=c[3], log=json.dumps(log))
            os.replace(tmp, path)
    return replace(case, note=json.dumps({"settling": log, "fill": fill, "seed": seed}))
