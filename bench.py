#!/usr/bin/env python
"""Throughput of the GB300 sDEM hot path: particle-steps/s.

  python bench.py [--gpus N --steps K --warmup W] [--impl reference]
                  [--workload hertz_poly_1m | hertz_poly_1m_deposited | lsd_mono_20k | hopper_4m
                              | sandboxes | surrogate]

The headline workload (hertz_poly_1m) is the 1M-sphere polydisperse Hertz
bed settled under gravity (seeded random sequential placement, settled by
the GPU path itself and cached on disk; make_case below).

Our arm: one DEMSystem per GPU (replicas: each rank advances its own
independent bed, no collective on the data path), W untimed steps, then K
timed steps (CUDA events on the library's stream, barrier + synchronize on both
sides, max over ranks).  The 1M bed (~300 MB of state) is larger than L2, so
no flush is needed between steps.  e2e: the same metric through the C ABI
with host buffers: upload of the state, K sdem_step_async(h,1) calls each
followed by a read-back of the step's counters, download of the state; once
with page-locked host arrays (e2e) and once with ordinary ones
(e2e_pageable).

--impl reference: the CPU restatement of the reference's algorithm (the
reference's Fortran+MPI build cannot be compiled here or on the GPU host: no
Fortran compiler, no MPI) on all host cores, one process per x-slab of the same
bed (domain decomposition without halo), rank 0 only.
"""
from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s, 1M Hertz spheres"
UNIT = "particle-steps/s"
# From the ncu captures in profiles/ (each file gives its command):
# profiles/kernels_hertz_poly_settled_1m.txt, one step of the settled 1M bed.
FORCE_DRAM_BYTES_PER_CONTACT = 401.4     # k_force: dram__bytes_read.sum + dram__bytes_write.sum per contact
FP64_INST_PER_SM_CLK = 2.0               # DADD/DMUL/DFMA thread operations per SM per clock (FP64 pipe)
NUM_SMS = 152
# Executed DADD + DMUL + DFMA thread instructions of the step's kernels,
# modelled per particle-particle contact, per sphere and per wall contact.
FP64_PER_CONTACT = {"k_force": 120.1, "k_gather": 24.2}
FP64_PER_SPHERE = {"k_integrate": 51.0, "k_bin": 3.0, "k_wall_detect": 0.74}
FP64_PER_WALL_CONTACT = {"k_wall_force": 123.3, "k_gather": 12.0}

# name -> (metric, default particles, base seed)
WORKLOADS = {
    "hertz_poly_1m": (METRIC, 1_000_000, 2),
    "hertz_poly_1m_deposited": ("particle-steps/s, 1M Hertz spheres (deposited bed)", 1_000_000, 2),
    "lsd_mono_20k": ("particle-steps/s, 20k LSD spheres", 20_000, 1),
    "hopper_4m": ("particle-steps/s, 4M bidisperse Hertz hopper", 4_000_000, 3),
}


def make_case(workload: str, n: int, seed: int):
    """The bed of a workload and a description of it for the JSON line.

    hertz_poly_1m: the 1M polydisperse Hertz configuration (d uniform in
      [0.8, 1.2] mm as 41 types, E 5e7 Pa, restitution 0.8, friction 0.4,
      dt 1e-6 s, AB2, 0.1 x 0.6 x 0.1 m box, five walls): seeded random
      sequential placement settled under gravity on the GPU
      (sdem_gb300.settle; cached on disk after the first run).
    hertz_poly_1m_deposited: the same material on a geometric deposition
      (sdem_gb300.beds.hertz_poly_case), about one resting contact per sphere.
    lsd_mono_20k: 20,000 monodisperse LSD spheres (restitution 0.9, friction
      0.3, dt 2e-6 s, AB2) from the seeded jittered lattice, after 10,000 GPU
      steps of settling (half the configuration's 20,000).
    hopper_4m: 4,000,000 bidisperse Hertz spheres (0.5 / 1.5 mm, 70:30,
      friction 0.5, restitution 0.7, dt 5e-7 s) in a hopper of four 60-degree
      finite planes over a 10 mm square outlet (0.26 m wide, a column above);
      after 1,000 GPU steps of discharge."""
    from sdem_gb300 import beds
    if workload == "hertz_poly_1m":
        from sdem_gb300 import settle
        case = settle.settled_hertz_poly_case(n=n, seed=seed)
        log = json.loads(case.note)["settling"]
        last = log[-1]
        desc = {"bed": f"seeded random sequential placement (seed {seed}, solid fraction 0.25) settled under "
                       f"gravity by the GPU path (sdem_gb300.settle: {sum(e['steps'] for e in log)} steps in "
                       f"{len(log)} stages)",
                "bed_height_m": last["height"], "bed_v_mean_mps": last["v_mean"], "bed_v_max_mps": last["v_max"]}
        return case, desc
    if workload == "hertz_poly_1m_deposited":
        return beds.hertz_poly_case(n=n, seed=seed), {
            "bed": f"seeded geometric deposition (seed {seed}, sdem_gb300.beds.hertz_poly_case)"}
    from sdem_gb300.capi import DEMSystem
    if workload == "lsd_mono_20k":
        case0 = beds.lsd_mono_case(n=n, seed=seed)
        prep = 10000
        desc = {"bed": f"seeded jittered lattice (seed {seed}) after {prep} GPU steps of settling"}
    elif workload == "hopper_4m":
        case0 = beds.hopper_case(n, seed, width=0.26, outlet=10.0e-3)
        prep = 1000
        desc = {"bed": f"hopper filled on a jittered lattice (seed {seed}) after {prep} GPU steps of discharge"}
    else:
        raise ValueError(workload)
    with DEMSystem(case0) as h:
        h.step(prep)
        case = beds.Case(case0.name, case0.opts, case0.tables, case0.walls, h.state(), contacts=h.contacts())
    return case, desc


# ---------------------------------------------------------------------------
# CPU leg: the oracle on x-slabs of the bed, one process per core
# ---------------------------------------------------------------------------
def _slab_worker(args):
    path, k, nslab, steps, warm, budget_s = args
    sys.path.insert(0, ROOT)
    from oracle.oracle import OracleSystem
    from sdem_gb300 import beds
    meta = json.load(open(os.path.join(path, "meta.json")))
    P = {name: np.load(os.path.join(path, name + ".npy"), mmap_mode="r")
         for name in ("id", "ptype", "usrmark", "posR", "linVel", "linAcc", "theta", "rotVel", "rotAcc")}
    x = P["posR"][:, 0]
    lo, hi = meta["xmin"] + (meta["xmax"] - meta["xmin"]) * k / nslab, \
        meta["xmin"] + (meta["xmax"] - meta["xmin"]) * (k + 1) / nslab
    sel = np.nonzero((x >= lo) & (x < hi))[0]
    parts = beds.Particles(*(np.ascontiguousarray(P[name][sel]) for name in
                             ("id", "ptype", "usrmark", "posR", "linVel", "linAcc", "theta", "rotVel", "rotAcc")))
    import pickle
    case = pickle.load(open(os.path.join(path, "case.pkl"), "rb"))
    case = beds.Case(case.name, case.opts, case.tables, case.walls, parts)
    o = OracleSystem(case, max_gid=meta["max_gid"])
    if warm:
        o.step(warm)
    if steps is None:   # calibrate a bounded sample
        t0 = time.perf_counter()
        o.step(1)
        t1 = time.perf_counter() - t0
        steps = int(max(2, min(400, budget_s / max(t1, 1e-6))))
    t0 = time.perf_counter()
    o.step(steps)
    el = time.perf_counter() - t0
    return len(sel), steps, el, o.counters()["pp"]


def cpu_leg(case, steps, warm, budget_s=1.5, procs=None):
    """Oracle over all host cores: returns (particle-steps/s, cores, sample text)."""
    procs = procs or os.cpu_count() or 1
    from oracle.oracle import load as load_oracle
    load_oracle()   # build once before the workers start
    tmp = tempfile.mkdtemp(prefix="sdem_bench_")
    p = case.particles
    for name in ("id", "ptype", "usrmark", "posR", "linVel", "linAcc", "theta", "rotVel", "rotAcc"):
        np.save(os.path.join(tmp, name + ".npy"), getattr(p, name))
    import pickle
    from sdem_gb300 import beds
    empty = beds.Particles(*(getattr(p, name)[:0] for name in
                             ("id", "ptype", "usrmark", "posR", "linVel", "linAcc", "theta", "rotVel", "rotAcc")))
    pickle.dump(beds.Case(case.name, case.opts, case.tables, case.walls, empty), open(os.path.join(tmp, "case.pkl"), "wb"))
    json.dump({"xmin": float(case.opts.minpoint[0]), "xmax": float(case.opts.maxpoint[0]),
               "max_gid": int(case.max_gid)}, open(os.path.join(tmp, "meta.json"), "w"))
    ctx = mp.get_context("spawn")
    with ctx.Pool(procs) as pool:
        res = pool.map(_slab_worker, [(tmp, k, procs, steps, warm, budget_s) for k in range(procs)])
    n_tot = sum(r[0] for r in res)
    work = sum(r[0] * r[1] for r in res)
    tmax = max(r[2] for r in res)
    ksteps = sorted(set(r[1] for r in res))
    sample = (f"{n_tot} particles of the bed in {procs} x-slabs (one oracle process per slab, no halo), "
              f"{ksteps[0] if len(ksteps) == 1 else ksteps} steps each, wall time of the slowest slab {tmax:.2f} s")
    return work / tmax, procs, sample


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.path = tempfile.mktemp(prefix="clocks_", suffix=".csv")
        self.gpu = gpu_index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        try:
            rows = [r.split(",") for r in open(self.path).read().strip().splitlines() if r.strip()]
        except Exception:
            rows = []
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
                for k, nm in enumerate(names):
                    if r[5 + k].strip().lower().startswith("active"):
                        reasons.add(nm)
            except Exception:
                pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def pinned_particles(p, rows=None):
    """A copy of Particles p in page-locked host memory (rows >= p.n rows)."""
    import torch

    rows = p.n if rows is None else rows

    def pin(a):
        t = torch.zeros((rows,) + a.shape[1:], dtype=torch.int32 if a.dtype == np.int32 else torch.float64,
                        pin_memory=True)
        v = t.numpy()
        v[:p.n] = a
        return v

    return type(p)(*(pin(getattr(p, f)) for f in ("id", "ptype", "usrmark", "posR", "linVel", "linAcc", "theta",
                                                    "rotVel", "rotAcc")))


# ---------------------------------------------------------------------------
def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def reference_arm(args):
    ws, rank, _ = dist_setup()
    if rank != 0:
        return
    metric, n_def, seed = WORKLOADS[args.workload]
    # the bed is the one our arm times (the settled bed is prepared on the GPU
    # once and cached; the timed region below is CPU only)
    case, desc = make_case(args.workload, args.n or n_def, seed)
    procs = os.cpu_count() or 1
    rate, cores, sample = cpu_leg(case, steps=args.steps, warm=args.warmup, procs=procs)
    line = {"impl": "reference", "metric": metric, "value": rate, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * case.particles.n / rate,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": args.workload, "n_particles": case.particles.n, **desc,
                       "parallelism": f"{cores} processes"},
            "cpu_baseline": {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": "CPU restatement of the reference (oracle/sdem_oracle.c), not the reference "
                                       "itself: " + sample},
            "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


STATE_FIELDS = ("id", "ptype", "usrmark", "posR", "linVel", "linAcc", "theta", "rotVel", "rotAcc")


def e2e_run(case, K, pinned: bool, barrier, shape=None, reps: int = 3):
    """The metric through the C ABI with host buffers: upload of the state,
    K x (sdem_step_async(h,1) + the step's counters read back), download of
    the state.  pinned: page-locked host arrays; else ordinary (pageable)
    numpy arrays, what a Fortran caller's arrays are unless it registers
    them.  The arrays have been through one untimed upload and download
    first.  The run is timed `reps` times (each from its own upload of the
    same state); returns (median elapsed s, h2d bytes, d2h bytes, all
    elapsed s)."""
    import torch
    from sdem_gb300 import beds
    from sdem_gb300.capi import DEMSystem
    sys2 = DEMSystem(case)
    if shape:
        from sdem_gb300 import tune
        tune.apply(sys2, shape)
    sys2.step(1)
    st0 = sys2.state()
    if pinned:
        st = pinned_particles(st0)
        out_buf = pinned_particles(st0, rows=sys2.cfg.n_capacity)
    else:
        st = st0
        cap = sys2.cfg.n_capacity
        out_buf = beds.Particles(*(np.zeros((cap,) + getattr(st0, f).shape[1:], dtype=getattr(st0, f).dtype)
                                   for f in STATE_FIELDS))
    # the host arrays carry one upload and one download before the timed run,
    # as an application's reused state arrays do: the first transfer from
    # freshly allocated host pages pays their one-time mapping, not the path
    sys2.upload(st)
    sys2.state(out=out_buf)
    els = []
    for _ in range(reps):
        barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sys2.upload(st)
        sys2.step_async(1)
        for k in range(1, K + 1):
            if k < K:
                sys2.step_async(1)          # step k+1 is queued ...
                sys2.counters_lagged()      # ... while step k's counters are read
            else:
                sys2.counters()
        out = sys2.state(out=out_buf)
        torch.cuda.synchronize()
        els.append(time.perf_counter() - t0)
    h2d = sum(getattr(st, f).nbytes for f in STATE_FIELDS)
    d2h = sum(getattr(out, f).nbytes for f in STATE_FIELDS) + K * 4 * 9
    sys2.close()
    return statistics.median(els), h2d, d2h, els


def fp64_step_model(C: float, n: int, pw: float) -> float:
    """Executed FP64 thread instructions of one step from the per-kernel
    counts measured by ncu (the constants above)."""
    return (C * sum(FP64_PER_CONTACT.values()) + n * sum(FP64_PER_SPHERE.values())
            + pw * sum(FP64_PER_WALL_CONTACT.values()))


def our_arm(args):
    import torch
    ws, rank, local = dist_setup()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    else:
        dist = None

    def barrier():
        if dist:
            dist.barrier()

    from sdem_gb300 import replicas

    from sdem_gb300 import build
    build.build()
    from sdem_gb300.capi import DEMSystem, probe_fp64_peak
    metric, n_def, base_seed = WORKLOADS[args.workload]
    seed = replicas.rank_seed(base_seed, rank)
    case, desc = make_case(args.workload, args.n or n_def, seed)
    n = case.particles.n
    fp64_peak = probe_fp64_peak()          # the FP64 pipe of this GPU, measured now (DFMA chains)
    # launch shape by the autotuner (results do not depend on it; cached per size class)
    from sdem_gb300 import tune
    shape = tune.tune_handle(case) if not args.no_tune else None
    sysm = DEMSystem(case)
    if shape:
        tune.apply(sysm, shape)
    sysm.step(args.warmup)
    stream = torch.cuda.ExternalStream(sysm.stream())
    K = args.steps
    barrier()
    torch.cuda.synchronize()
    l0 = sysm.launch_count()
    sums0 = sysm.counter_sums()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        e0.record(stream)
        sysm.step_async(K)
        e1.record(stream)
        e1.synchronize()
    torch.cuda.synchronize()
    barrier()
    ms = e0.elapsed_time(e1)
    launches = sysm.launch_count() - l0
    cnt = sysm.counters()
    sums1 = sysm.counter_sums()
    # per-phase breakdown: a separate window with CUDA events between the
    # phases (the library then runs the search/force chunks in one stream)
    nph = min(K, 50)
    sysm.profile_begin(nph)
    sysm.step(nph)
    phases, nprof = sysm.profile_end()
    C_avg = (sums1["pp"] - sums0["pp"]) / max(sums1["steps"] - sums0["steps"], 1)
    PW_avg = (sums1["pw"] - sums0["pw"]) / max(sums1["steps"] - sums0["steps"], 1)
    value, t_max, n_all = replicas.aggregate(ms * 1e-3, n, K, device="cuda")
    ms_max = t_max * 1e3

    # dominant kernel: the contact-force kernel (one thread per contact)
    C = C_avg
    dom = max(phases, key=phases.get)
    t_force = phases["force"] / nprof * 1e-3
    force_bytes = 80.0 * C          # per persistent contact: key, spring and VelRel_Init read + written
    achieved = force_bytes / t_force / 1e9
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    # DRAM bytes of k_force per contact from one ncu capture of the same kernel
    # (profiles/), scaled to this launch by its contacts
    traffic = FORCE_DRAM_BYTES_PER_CONTACT * C
    # algorithmic FP64 operations of k_force per Hertz contact (force law + normal
    # vector; the two r*Moment scalings are the gather's): 121 add/sub/mul,
    # 8 sqrt, 7 divisions, each sqrt/div counted as one operation
    fp64_per_contact = 136
    t_step = ms / K * 1e-3
    step_bytes = n * 352.0 + C * 80.0   # per-step algorithmic bytes of the whole path

    e2e = e2e_pageable = None
    if args.e2e_steps < 0:
        args.e2e_steps = K      # the same number of steps as the device-timed run
    if args.e2e_steps > 0:
        Ke = args.e2e_steps
        runs = {}
        for pinned in (True, False):
            el, h2d, d2h, els = e2e_run(case, Ke, pinned, barrier, shape)
            _, el, _ = replicas.aggregate(el, n, Ke, device="cuda")
            runs[pinned] = {"value": n_all * Ke / el, "unit": UNIT, "h2d_bytes_per_step": int(h2d / Ke),
                            "d2h_bytes_per_step": int(d2h / Ke), "steps": Ke,
                            "runs_ms": [round(x * 1e3, 3) for x in els]}
        e2e = dict(runs[True], note="upload of the state from page-locked host memory, K x (sdem_step_async(h,1) "
                   "+ the counters of each step read back: sdem_counters_lagged while the next step runs, "
                   "sdem_counters after the last), download of the state into page-locked host memory; the "
                   "host arrays went through one untimed upload and download first; median of three timed "
                   "runs (runs_ms, rank 0's)")
        e2e_pageable = dict(runs[False], note="the same with ordinary (pageable) host arrays, as an unmodified "
                            "Fortran caller passes them")

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        rate, cores, sample = cpu_leg(case, steps=None, warm=0)
        cpu = {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": "CPU restatement of the reference (oracle/sdem_oracle.c): " + sample}

    if rank == 0:
        clocks = clk.summary()
        clk_mhz = float(clocks.get("sm_mhz") or 2070.0)
        pipe_peak = FP64_INST_PER_SM_CLK * NUM_SMS * clk_mhz * 1e6     # FP64 thread ops per second
        step_ops = fp64_step_model(C, n, PW_avg)
        line = {
            "metric": metric, "value": value, "unit": UNIT, "n_gpus": ws, "steps": K, "warmup": args.warmup,
            "ms_per_step": ms_max / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic",
            "config": {"workload": args.workload, "n_particles": n,
                       "contact_model": "Hertz-Mindlin" if case.opts.cf_type == 2 else "linear spring-dashpot",
                       "types": int(case.tables.n_types), "dt": case.opts.dt,
                       "integrator": {1: "FE", 2: "AB2", 3: "AB3"}[case.opts.pi_method],
                       "pp_contacts_avg": C, "pw_contacts_avg": PW_avg, "contacts_per_particle": C / n,
                       "pp_contacts_last": cnt["pp"], **desc,
                       "l2": "state > L2 (no flush)" if n >= 500_000 else "state < L2 (no flush)",
                       "parallelism": f"replicas x{ws}"},
            "e2e": e2e,
            "e2e_pageable": e2e_pageable,
            "gpu_launches": launches,
            "tuning": ({"pipeline_chunks": shape["pipeline_chunks"],
                        "force_blocks_per_sm": shape["force_blocks_per_sm"],
                        "first_chunk_percent": shape["first_chunk_percent"],
                        "ms_per_step_tried": shape["tried"], "note": "sdem_gb300.tune.tune_handle, cached by size "
                        "class; results are bit-identical for every launch shape"} if shape else None),
            "roofline": {"bound": "hbm", "kernel": "k_force", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                         "frac": achieved / hbm, "traffic": traffic,
                         "algorithmic_bytes": "80 B per contact x contacts per launch",
                         "peak_note": "hbm_gbs of measured (MEASURED_PEAKS.json)",
                         "note": "k_force is FP64-ALU bound on GB300, see fp64 and step_fp64"},
            "fp64": {"kernel": "k_force", "achieved_tflops": fp64_per_contact * C / t_force / 1e12,
                     "peak_tflops": fp64_peak["tflops"],
                     "frac": fp64_per_contact * C / t_force / 1e12 / fp64_peak["tflops"],
                     "algorithmic_ops_per_contact": fp64_per_contact,
                     "executed_inst_per_contact": FP64_PER_CONTACT["k_force"],
                     "pipe_frac": FP64_PER_CONTACT["k_force"] * C / t_force / pipe_peak,
                     "note": "peak: DFMA chains measured in this run (sdem_probe_fp64_peak, 2 flops per DFMA); "
                             "pipe_frac: executed DADD/DMUL/DFMA per second over the pipe's 2 per SM per clock "
                             "at the sampled SM clock"},
            "step_fp64": {"executed_per_step": step_ops, "achieved_per_s": step_ops / t_step,
                          "pipe_peak_per_s": pipe_peak, "frac": step_ops / t_step / pipe_peak,
                          "probe_dfma_per_s": fp64_peak["dfma_per_s"],
                          "note": "executed DADD+DMUL+DFMA of every step kernel (ncu counts per contact, per "
                                  "sphere and per wall contact, profiles/) over ms_per_step, against the FP64 "
                                  "pipe's 2 per SM per clock x 152 SMs at the sampled SM clock"},
            "step_roofline": {"achieved": step_bytes / t_step / 1e9, "peak": hbm, "unit": "GB/s",
                              "frac": step_bytes / t_step / 1e9 / hbm,
                              "algorithmic_bytes": "352 B per particle + 80 B per contact per step"},
            "phases_ms_per_step": {k: v / nprof for k, v in phases.items()},
            "phases_note": "separate window of %d steps with events between phases, search/force chunks in one "
                           "stream; the timed steps overlap each chunk's search with the previous chunk's forces "
                           "on two streams" % nprof,
            "dominant_phase": dom,
            "cpu_baseline": cpu,
            "clocks": clocks,
        }
        print(json.dumps(line), flush=True)
    sysm.close()
    if dist:
        dist.destroy_process_group()


def sandboxes_arm(args):
    """The batched workload (its own line): `--instances` sandboxes of
    2,000-50,000 spheres with their own materials, contact models and boxes
    (sdem_gb300.beds.sandbox_case, parameters from seed 4), deposited as
    beds in contact (`--sandbox-layout lattice`: the configuration's falling
    lattice), stepped `--contact-steps` batch steps, then the autotuner (sdem_gb300.tune) picks each size
    class's launch shape and the batch's group size.  Timed, from that state:
    (a) the tuned batch, (b) the batch with the default shapes, (c) one
    instance after another (each instance's steps, then the next: one launch
    sequence per instance), (d) every instance on its own stream from one host
    thread.  Host wall-clock around synchronised runs; particle-steps/s of the
    whole set."""
    import torch
    from sdem_gb300 import beds, tune
    from sdem_gb300.capi import DEMBatch, DEMSystem
    torch.cuda.set_device(0)
    rng = np.random.default_rng(4)
    cases = [beds.sandbox_case(rng, i, layout=args.sandbox_layout) for i in range(args.instances)]
    total = sum(c.particles.n for c in cases)
    members = [DEMSystem(c) for c in cases]
    t0 = time.perf_counter()
    pre = DEMBatch(members)
    pre.step(args.contact_steps + args.contact_steps % 2)
    pre.close()
    t_contact = time.perf_counter() - t0
    contacts = sum(m.counters()["pp"] + m.counters()["pw"] for m in members)
    # tuning: one representative (its state and contacts now) per size class
    t0 = time.perf_counter()
    classes = {}
    for m in members:
        classes.setdefault(tune.size_class(m.case), []).append(m)
    shapes = {}
    for key, ms_ in classes.items():
        rep = ms_[len(ms_) // 2]
        rc = beds.Case(rep.case.name, rep.case.opts, rep.case.tables, rep.case.walls, rep.state(),
                       contacts=rep.contacts())
        shapes[key] = tune.tune_handle(rc, steps=6)
    default_shape = [m.get_launch() for m in members]
    for m in members:
        tune.apply(m, shapes[tune.size_class(m.case)])
    group = tune.tune_batch(members, steps=4)
    t_tune = time.perf_counter() - t0
    K = args.steps + args.steps % 2          # whole graph replays

    def run_batch(gs):
        b = DEMBatch(members, group_size=gs)
        b.step(2 * ((args.warmup + 1) // 2))   # even: the captured parities hold
        t = time.perf_counter()
        b.step(K)
        el = time.perf_counter() - t
        b.close()
        return el

    t_tuned = run_batch(group["group_size"])
    for m, (c, f, p) in zip(members, default_shape):
        m.set_launch(c, f, p or -1)
    t_default = run_batch(0)
    for m in members:                        # each instance's own graphs, captured before timing
        m.step(4)
    t0 = time.perf_counter()
    for m in members:
        m.step(K)
    t_seq = time.perf_counter() - t0
    t0 = time.perf_counter()
    for m in members:
        m.step_async(K)
    for m in members:
        m.counters()
    t_streams = time.perf_counter() - t0
    line = {"metric": "particle-steps/s, %d sandboxes" % args.instances, "value": total * K / t_tuned,
            "unit": UNIT, "n_gpus": 1, "steps": K, "warmup": args.warmup, "ms_per_step": t_tuned / K * 1e3,
            "higher_is_better": True, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "sandboxes", "instances": args.instances, "particles": total,
                       "layout": args.sandbox_layout, "contact_steps": args.contact_steps,
                       "contacts_at_start": contacts,
                       "contacts_per_particle": contacts / total, "models": {
                           "hertz": sum(1 for c in cases if c.opts.cf_type == props_cft_nlin()),
                           "lsd": sum(1 for c in cases if c.opts.cf_type != props_cft_nlin())}},
            "batch_default_shapes": total * K / t_default,
            "one_instance_after_another": total * K / t_seq,
            "instances_on_own_streams": total * K / t_streams,
            "tuning": {"group_size": group["group_size"], "group_sizes_ms": group["tried"],
                       "shapes": {k: {"pipeline_chunks": v["pipeline_chunks"],
                                      "force_blocks_per_sm": v["force_blocks_per_sm"],
                                      "first_chunk_percent": v["first_chunk_percent"]} for k, v in shapes.items()},
                       "seconds": t_tune, "contact_seconds": t_contact},
            "note": "host wall clock around synchronised runs of the same sandboxes in contact, in this order: "
                    "tuned batch, batch with default shapes, one instance after another, every instance on its "
                    "own stream"}
    print(json.dumps(line), flush=True)
    for m in members:
        m.close()


def surrogate_arm(args):
    """The learned surrogate (its own line; not the headline): a network
    trained on plain-DEM trajectories of `--train-beds` Hertz sandboxes
    (`--train-n`/2 to `--train-n` spheres, parameters from seed 5, advanced
    together by the batched form: 15,000 settling steps, then
    `--train-frames` frames a stride of 100 steps apart) for
    `--train-iters` Adam steps, then on the 1M
    Hertz bed: K surrogate strides (graph build, features, forward, stride
    update) against K x 100 plain DEM steps, and a run of the runner with the
    plain-DEM judge every `--judge-every` strides (bounds: 2% relative bed
    height, 5% mean relative wall pressure).  Simulated seconds per wall
    second, host clock around synchronised runs."""
    import torch
    from sdem_gb300 import beds, props, surrogate as sg
    from sdem_gb300.capi import DEMSystem
    torch.cuda.set_device(0)
    S, vscale = 100, 0.05
    t0 = time.perf_counter()
    rng = np.random.default_rng(5)
    # Hertz sandboxes (the configuration's material ranges), all advanced
    # together by the plain path's batched form; the last one is held out
    cases = [beds.sandbox_case(rng, k, n_lo=args.train_n // 2, n_hi=args.train_n, cf_type=props.CFT_NLIN)
             for k in range(args.train_beds + 1)]
    systems = [DEMSystem(c) for c in cases]
    recorded = sg.record_samples_batch(systems, cases, S, args.train_frames, settle=15000)
    for s in systems:
        s.close()
    sets = [[sg.to_device(x, c, 1.2e-3, vscale) for x in xs] for xs, c in zip(recorded, cases)]
    del recorded
    train, held = [x for ss in sets[:-1] for x in ss], sets[-1]
    t_data = time.perf_counter() - t0
    net = sg.Network(seed=0)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    losses = [float(net.train_step(train[i % len(train)].graph, train[i % len(train)].xn,
                                   train[i % len(train)].target, lr=2e-3)) for i in range(args.train_iters)]
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    mse, mse_free = sg.evaluate(net, held)

    case, _ = make_case("hertz_poly_1m_deposited", args.n or 1_000_000, 2)
    dem = DEMSystem(case)
    dem.step(args.warmup)
    dmax = 2.0 * float(case.tables.radius.max())
    runner = sg.SurrogateRunner(net, dem, case, S, dmax, vscale, judge_every=args.judge_every, bound=0.02,
                                fallback_strides=args.judge_every, pressure_bound=0.05)
    K = max(1, args.strides)
    start = (runner.posR.clone(), runner.vel.clone(), runner.omega.clone())

    def reset():
        # every timed stride starts from the plain DEM's state: the cost of a
        # stride on the bed itself, not on whatever an untrained rollout makes
        runner.posR.copy_(start[0])
        runner.vel.copy_(start[1])
        runner.omega.copy_(start[2])

    runner._surrogate_stride(runner.posR, runner.vel, runner.omega)     # warm-up
    phases, E = surrogate_phases(runner, net, sg, torch, reset)
    # the same forward on the warp-level mma.sync kernel, for comparison
    assert net.lib.sdem_sg_set_tensor_path(0) == 0
    phases_mma, _ = surrogate_phases(runner, net, sg, torch, reset)
    assert net.lib.sdem_sg_set_tensor_path(1) == 0
    t_sur = 0.0
    for _ in range(K):
        reset()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        runner._surrogate_stride(runner.posR, runner.vel, runner.omega)
        torch.cuda.synchronize()
        t_sur += time.perf_counter() - t0
    t0 = time.perf_counter()
    dem.step(K * S)
    dem.counters()
    t_plain = time.perf_counter() - t0
    # the judged run starts again from the plain state the timing started from
    reset()
    runner.edge_ref = None
    h = S * case.opts.dt
    t_sim0 = runner.t
    t0 = time.perf_counter()
    stats = runner.run(2 * args.judge_every)
    torch.cuda.synchronize()
    t_run = time.perf_counter() - t0
    run_strides = runner.t - t_sim0
    line = {"metric": "simulated s per wall s, surrogate vs plain DEM, 1M Hertz spheres",
            "value": K * h / t_sur, "unit": "sim-s/s", "n_gpus": 1, "steps": K, "warmup": args.warmup,
            "higher_is_better": True, "dtype": "bf16 (network), f64 (plain DEM and stride update)",
            "data": "synthetic",
            "plain_dem": K * h / t_plain, "ratio_vs_plain": t_plain / t_sur,
            "ms_per_stride": {"surrogate": t_sur / K * 1e3, "plain_dem": t_plain / K * 1e3},
            "surrogate_phases_ms": phases,
            "forward_tensor": {"flop": surrogate_forward_flop(case.particles.n, E),
                               "achieved_tflops": surrogate_forward_flop(case.particles.n, E) / phases["forward"] / 1e9,
                               "peak_tflops": measured_bf16_tflops(), "peak_note": "bf16 dense, burst, of measured",
                               "gemm": "tcgen05 (k_gemm_tc) for the forward layers",
                               "mma_sync_forward_ms": phases_mma["forward"],
                               "mma_sync_achieved_tflops": surrogate_forward_flop(case.particles.n, E)
                               / phases_mma["forward"] / 1e9},
            "with_judge": {"strides": 2 * args.judge_every, "sim_s_per_s": run_strides * h / t_run,
                           "rewound_strides": stats["rewound_strides"],
                           "judged": stats["judged"], "fallbacks": stats["fallbacks"],
                           "diverged": stats["diverged"],
                           "bed_height_rel_err": stats["errors"],
                           "wall_pressure_rel_err": stats["pressure_errors"],
                           "bounds": {"bed_height": runner.bound, "wall_pressure": runner.pressure_bound}},
            "training": {"beds": args.train_beds, "spheres_per_bed": [c.particles.n for c in cases[:-1]],
                         "frames_per_bed": args.train_frames, "generator": "sdem_batch (one graph per group)",
                         "samples": len(train), "iters": args.train_iters,
                         "loss_first10": float(np.mean(losses[:10])), "loss_last10": float(np.mean(losses[-10:])),
                         "heldout_mse": mse, "heldout_mse_free_flight": mse_free, "data_s": t_data,
                         "train_s": t_train},
            "config": {"workload": "surrogate_hertz_poly_1m", "particles": case.particles.n, "edges": E,
                       "stride_steps": S,
                       "dt": case.opts.dt,
                       "latent": sg.LATENT, "layers": sg.LAYERS, "cutoff_dmax": sg.CUTOFF_FACTOR},
            "note": "host wall clock around synchronised runs; the stride update integrates the predicted "
                    "stride-mean accelerations (semi-implicit Euler over the stride)"}
    print(json.dumps(line), flush=True)
    dem.close()


def transfers_arm(args):
    """The host side of the end-to-end figure (its own line): the host link's
    copy bandwidth (260 MiB from page-locked memory, one stream against four)
    and the library's upload and download of the 1M bed's state
    (sdem_upload_particles / sdem_download_particles, page-locked and pageable
    host arrays, median of 5 after one untimed transfer).  Host clock around
    synchronised calls."""
    import torch
    from sdem_gb300 import beds
    from sdem_gb300.capi import DEMSystem
    torch.cuda.set_device(0)
    N = 260 * 2**20
    hbuf = torch.empty(N, dtype=torch.uint8, pin_memory=True)
    hbuf.fill_(1)
    dbuf = torch.empty(N, dtype=torch.uint8, device="cuda")
    streams = [torch.cuda.Stream() for _ in range(4)]

    def copy_rate(ns, h2d):
        parts = [(i * N // ns, (i + 1) * N // ns) for i in range(ns)]
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for (a, b), st in zip(parts, streams):
            with torch.cuda.stream(st):
                if h2d:
                    dbuf[a:b].copy_(hbuf[a:b], non_blocking=True)
                else:
                    hbuf[a:b].copy_(dbuf[a:b], non_blocking=True)
        torch.cuda.synchronize()
        return N / (time.perf_counter() - t0) / 1e9

    link = {}
    for h2d in (True, False):
        for ns in (1, 4):
            copy_rate(ns, h2d)
            link[f"{'h2d' if h2d else 'd2h'}_{ns}_streams_gbs"] = max(copy_rate(ns, h2d) for _ in range(5))
    case, _ = make_case("hertz_poly_1m_deposited", args.n or 1_000_000, 2)
    s = DEMSystem(case)
    s.step(2)
    st0 = s.state()
    out = {}
    for pinned in (True, False):
        st = pinned_particles(st0) if pinned else st0
        cap = s.cfg.n_capacity
        buf = (pinned_particles(st0, rows=cap) if pinned else
               beds.Particles(*(np.zeros((cap,) + getattr(st0, f).shape[1:], dtype=getattr(st0, f).dtype)
                                for f in STATE_FIELDS)))
        s.upload(st)
        s.state(out=buf)
        up, down = [], []
        for _ in range(5):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            s.upload(st)
            t1 = time.perf_counter()
            s.state(out=buf)
            t2 = time.perf_counter()
            up.append((t1 - t0) * 1e3)
            down.append((t2 - t1) * 1e3)
        key = "page_locked" if pinned else "pageable"
        out[key] = {"upload_ms": statistics.median(up), "download_ms": statistics.median(down),
                    "bytes_each_way": int(sum(getattr(st, f).nbytes for f in STATE_FIELDS))}
    s.close()
    line = {"metric": "host transfers of the 1M bed's state", "unit": "ms", "n_gpus": 1, "data": "synthetic",
            "config": {"workload": "transfers", "particles": case.particles.n}, "host_link": link,
            "state_transfers": out,
            "note": "host clock around synchronised calls; the state arrays went through one untimed upload "
                    "and download first"}
    print(json.dumps(line), flush=True)


def surrogate_gemm_arm(args):
    """The surrogate's GEMM alone (its own line): the first edge layer of the
    network's forward -- E rows gathered from node latents twice plus the
    edge latents (three 128-wide segments, R = 384) times a 128 x 384 weight,
    bias, ReLU, bf16 output -- and the second edge layer (R = 128), on the
    tcgen05 kernel and on the mma.sync kernel.  E = --n rows (default 2^22),
    node rows E / 24.  CUDA events on the current stream, median of 5 after 3
    warm-ups; FLOP = 2 E R J."""
    import ctypes
    import torch
    from sdem_gb300 import build, surrogate as sg
    build.build()
    torch.cuda.set_device(0)
    lib = sg.load()
    E = args.n or (1 << 22)
    nodes = max(E // 24, 1)
    L = 128
    g = torch.Generator(device="cuda").manual_seed(11)
    h = (torch.randn((nodes, L), device="cuda", generator=g) * 0.5).to(torch.bfloat16)
    e = (torch.randn((E, L), device="cuda", generator=g) * 0.5).to(torch.bfloat16)
    dst = torch.randint(0, nodes, (E,), device="cuda", generator=g, dtype=torch.int32)
    src = torch.randint(0, nodes, (E,), device="cuda", generator=g, dtype=torch.int32)
    W1 = (torch.randn((L, 3 * L), device="cuda", generator=g) * 0.05).to(torch.bfloat16)
    W2 = (torch.randn((L, L), device="cuda", generator=g) * 0.05).to(torch.bfloat16)
    bias = torch.zeros(L, device="cuda")
    z = torch.empty((E, L), dtype=torch.bfloat16, device="cuda")
    out = torch.empty((E, L), dtype=torch.float32, device="cuda")
    A1 = sg._Op(0, (h, 0, L, L, dst), (h, 0, L, L, src), (e, 0, L, L, None))
    B1 = sg._Op(0, (W1, 0, 3 * L, 3 * L, None))
    A2 = sg._Op(0, (z, 0, L, L, None))
    B2 = sg._Op(0, (W2, 0, L, L, None))
    ep1 = sg._ep(bias=bias, relu=1, out_bf=z, ld_out_bf=L)
    ep2 = sg._ep(out=out, ld_out=L)

    def timed(A, B, R, ep):
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        ts = []
        for k in range(8):
            ev[0].record()
            assert lib.sdem_sg_gemm(E, L, R, ctypes.byref(A.o), ctypes.byref(B.o), ctypes.byref(ep), 1, None,
                                    sg._stream()) == 0
            ev[1].record()
            torch.cuda.synchronize()
            if k >= 3:
                ts.append(ev[0].elapsed_time(ev[1]))
        return statistics.median(ts)

    res = {}
    for path, name in ((1, "tcgen05"), (0, "mma_sync")):
        assert lib.sdem_sg_set_tensor_path(path) == 0
        t1 = timed(A1, B1, 3 * L, ep1)
        t2 = timed(A2, B2, L, ep2)
        res[name] = {"edge_w1_ms": t1, "edge_w1_tflops": 2.0 * E * 3 * L * L / t1 / 1e9,
                     "edge_w2_ms": t2, "edge_w2_tflops": 2.0 * E * L * L / t2 / 1e9}
    assert lib.sdem_sg_set_tensor_path(1) == 0
    cnt = ctypes.c_uint(0)
    lib.sdem_sg_tensor_timeouts(ctypes.byref(cnt))
    peak = measured_bf16_tflops()
    tc = res["tcgen05"]
    line = {"metric": "TFLOP/s, surrogate edge-layer GEMM (bf16 in, fp32 accumulate)",
            "value": tc["edge_w1_tflops"], "unit": "TFLOP/s", "n_gpus": 1, "higher_is_better": True,
            "dtype": "bf16", "data": "synthetic",
            "config": {"workload": "surrogate_gemm", "rows": E, "node_rows": nodes, "J": L,
                       "R": [3 * L, L], "gather": "rows of two 128-wide segments gathered by edge index"},
            "roofline": {"bound": "tensor", "kernel": "k_gemm_tc", "achieved": tc["edge_w1_tflops"], "peak": peak,
                         "unit": "TFLOP/s", "frac": tc["edge_w1_tflops"] / peak,
                         "peak_note": "bf16 dense, burst, of measured (MEASURED_PEAKS.json)"},
            "paths": res, "tcgen05_wait_timeouts": cnt.value}
    print(json.dumps(line), flush=True)


def surrogate_forward_flop(n: int, E: int, latent: int = 128, layers: int = 6) -> float:
    """Tensor-core flops of one surrogate forward pass (2 per multiply-add):
    encoders, `layers` edge MLPs over [h_dst, h_src, e] and node MLPs over
    [h, agg], decoder."""
    L = latent
    edge = 2 * (16 * L + L * L) + layers * 2 * (3 * L * L + L * L)
    node = 2 * (32 * L + L * L) + layers * 2 * (2 * L * L + L * L) + 2 * (L * L + L * 16)
    return float(E * edge + n * node)


def measured_bf16_tflops():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["bf16_tflops"])
    except Exception:
        return 1900.0


def surrogate_phases(runner, net, sg, torch, reset, reps: int = 3):
    """Median CUDA-event times (ms) of the parts of one surrogate stride
    (graph build, node features, forward, stride update) from the state
    reset() restores, and the edge count."""
    import ctypes
    out = {"graph": [], "features": [], "forward": [], "update": []}
    E = 0
    for _ in range(reps):
        reset()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(5)]
        ev[0].record()
        g = sg.build_graph(runner.posR, runner.grid, sender_order=False)
        ev[1].record()
        xn = sg.node_features(runner.posR, runner.vel, runner.omega, runner.planes, runner.d_max, runner.vscale)
        ev[2].record()
        y = net.forward(g, xn, keep=False)
        ev[3].record()
        gx, gy, gz = runner.case.opts.gravity
        rc = net.lib.sdem_sg_advance(runner.posR.shape[0], sg._ptr(y), sg.OUT, 9.81, gx, gy, gz, runner.h,
                                     ctypes.byref(runner.box), sg._ptr(runner.posR), sg._ptr(runner.vel),
                                     sg._ptr(runner.omega), sg._stream())
        assert rc == 0
        ev[4].record()
        torch.cuda.synchronize()
        for k, name in enumerate(("graph", "features", "forward", "update")):
            out[name].append(ev[k].elapsed_time(ev[k + 1]))
        E = g.E
    return {k: statistics.median(v) for k, v in out.items()}, E


def props_cft_nlin():
    from sdem_gb300 import props
    return props.CFT_NLIN


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=0, help="particles (default: the workload's)")
    ap.add_argument("--e2e-steps", type=int, default=-1,
                    help="steps of the end-to-end run (default: --steps; 0 skips it)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-tune", action="store_true", help="keep the library's default launch shape")
    ap.add_argument("--workload", default="hertz_poly_1m",
                    choices=[*WORKLOADS, "sandboxes", "surrogate", "surrogate_gemm", "transfers"],
                    help="hertz_poly_1m (the headline), hertz_poly_1m_deposited, lsd_mono_20k, hopper_4m; "
                         "sandboxes: the batched workload; surrogate: the learned surrogate against the plain "
                         "DEM; transfers: the host link and the state's upload and download (each its own line)")
    ap.add_argument("--instances", type=int, default=512)
    ap.add_argument("--contact-steps", type=int, default=1000,
                    help="sandboxes: batch steps before timing")
    ap.add_argument("--sandbox-layout", default="deposited", choices=["deposited", "lattice"],
                    help="sandboxes: deposited beds in contact (default) or the falling lattice")
    ap.add_argument("--train-beds", type=int, default=16)
    ap.add_argument("--train-n", type=int, default=50000, help="spheres per training bed (half to all)")
    ap.add_argument("--train-frames", type=int, default=12)
    ap.add_argument("--train-iters", type=int, default=300)
    ap.add_argument("--strides", type=int, default=5)
    ap.add_argument("--judge-every", type=int, default=5)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.workload == "sandboxes":
        sandboxes_arm(args)
    elif args.workload == "transfers":
        transfers_arm(args)
    elif args.workload == "surrogate_gemm":
        surrogate_gemm_arm(args)
    elif args.workload == "surrogate":
        surrogate_arm(args)
    elif args.impl == "reference":
        reference_arm(args)
    else:
        our_arm(args)


if __name__ == "__main__":
    main()
