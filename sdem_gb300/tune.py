"""Autotuner of the launch shapes (the batched form's block shape, cell factor
and group size).

What it may change, and why results stay exact:

- pipeline chunks (1..4), the first chunk's share of the targets and force
  blocks per SM (1..8) of one handle's step (sdem_set_launch): every order
  that matters is fixed by sort positions, so the results are bit-identical
  for every value;
- the batch's group size (members per captured graph and stream,
  sdem_batch_create_grouped): members are independent, so results are
  bit-identical;
- the cell factor (the reference's Prtcl_cs_ratio >= 1), only when the
  caller allows it: the contact set is the same for every factor (the exact
  overlap test is unchanged), but the search visits cells in another order,
  so forces are summed in another order -- equal to what the reference
  computes with that Prtcl_cs_ratio, not to its run with the original one.

There is no list-rebuild skin to tune: the reference keeps contact history
only while a pair overlaps (Prtcl_CL_and_CF.f90:500-572) and searches every
step; a Verlet skin would change neither the set nor the history, only skip
searches, and is not built.

Each candidate is timed on a fresh handle of the same case (the bed does not
advance between candidates): a few warm-up steps, then K steps timed with
CUDA events on the handle's stream.  The choice is cached on disk by size
class (particles rounded to a power of two, contact model, search method,
periodic directions), so a class is tuned once per library build.
"""
from __future__ import annotations

import itertools
import json
import math
import os
from dataclasses import replace
from typing import Callable, Dict, Iterable, Optional, Sequence

HERE = os.path.dirname(os.path.abspath(__file__))
CACHE_DIR = os.path.join(os.path.dirname(HERE), ".tunecache")

CHUNKS = (1, 2, 3, 4)
FORCE_BLOCKS = (2, 3, 4)
FIRST_CHUNK = (-1, 25, 35)        # percent of the targets in the first chunk (-1: whole search waves)
CELL_FACTORS = (1.0, 1.25, 1.5)
GROUP_SIZES = (16, 32, 64, 128)


def size_class(case) -> str:
    o = case.opts
    n = max(case.particles.n, 1)
    return (f"n2^{int(round(math.log2(n)))}_cf{o.cf_type}_cs{o.cs_method}_"
            f"per{''.join(str(int(v)) for v in o.periodic)}")


def _stamp() -> str:
    try:
        with open(os.path.join(HERE, "libsdem_gpu.so.stamp")) as f:
            return f.read().strip()[:16]
    except OSError:
        return "none"


def _cache_path(kind: str) -> str:
    return os.path.join(CACHE_DIR, f"{kind}_{_stamp()}.json")


def _load(kind: str) -> dict:
    try:
        with open(_cache_path(kind)) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(kind: str, table: dict) -> None:
    os.makedirs(CACHE_DIR, exist_ok=True)
    tmp = f"{_cache_path(kind)}.{os.getpid()}.tmp"
    with open(tmp, "w") as f:
        json.dump(table, f, indent=1, sort_keys=True)
    os.replace(tmp, _cache_path(kind))


def time_steps(system, steps: int = 10, warmup: int = 4) -> float:
    """ms per step of `system` (CUDA events on its stream)."""
    import torch
    system.step(warmup)
    st = torch.cuda.ExternalStream(system.stream())
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(st)
    system.step_async(steps)
    e1.record(st)
    e1.synchronize()
    return e0.elapsed_time(e1) / steps


def best_of(candidates: Iterable, measure: Callable[[object], float]):
    """(best candidate, {candidate: ms}) by the smallest measured time; ties
    keep the first candidate."""
    times = {}
    best, best_t = None, math.inf
    for c in candidates:
        t = measure(c)
        times[c] = t
        if t < best_t:
            best, best_t = c, t
    return best, times


def tune_handle(case, allow_cell_factor: bool = False, steps: int = 10, cache: bool = True,
                timer: Optional[Callable] = None) -> Dict:
    """The fastest (pipeline_chunks, force_blocks_per_sm, first_chunk_percent
    [, cs_ratio]) for a case's size class.  Returns {"pipeline_chunks",
    "force_blocks_per_sm", "first_chunk_percent", "cs_ratio", "ms_per_step",
    "tried"}."""
    from .capi import DEMSystem
    key = size_class(case) + ("_cell" if allow_cell_factor else "")
    table = _load("handle") if cache else {}
    if key in table:
        return table[key]
    factors = CELL_FACTORS if allow_cell_factor else (case.opts.cs_ratio,)

    def measure(c):
        chunks, fb, fp, cf = c
        trial = case if cf == case.opts.cs_ratio else replace(case, opts=replace(case.opts, cs_ratio=cf))
        with DEMSystem(trial) as h:
            h.set_launch(chunks, fb, fp)
            return (timer or time_steps)(h, steps)

    # the first chunk's share only matters with more than one chunk
    cands = [(c, f, p, x) for c, f, p, x in itertools.product(CHUNKS, FORCE_BLOCKS, FIRST_CHUNK, factors)
             if c > 1 or p == -1]
    best, times = best_of(cands, measure)
    out = {"pipeline_chunks": best[0], "force_blocks_per_sm": best[1], "first_chunk_percent": best[2],
           "cs_ratio": best[3], "ms_per_step": times[best],
           "tried": {f"{c[0]}x{c[1]}/{c[2]}@{c[3]}": t for c, t in times.items()}}
    if cache:
        table[key] = out
        _store("handle", table)
    return out


def tune_batch(systems: Sequence, steps: int = 4, cache: bool = True, key_extra: str = "",
               timer: Optional[Callable] = None) -> Dict:
    """The fastest batch group size for a set of handles (already created and
    uploaded).  Each group size builds its own batch over the same handles and
    times `steps` batch steps after two warm-up steps; the handles advance
    while they are timed.  Returns {"group_size", "ms_per_step", "tried"}."""
    import time

    from .capi import DEMBatch
    n = sum(s.case.particles.n for s in systems)
    key = f"m{len(systems)}_n2^{int(round(math.log2(max(n, 1))))}{key_extra}"
    table = _load("batch") if cache else {}
    if key in table:
        return table[key]

    def measure(gs):
        b = DEMBatch(systems, group_size=gs)
        try:
            b.step(2)
            if timer:
                return timer(b, steps)
            t0 = time.perf_counter()
            b.step(steps)
            return (time.perf_counter() - t0) * 1e3 / steps
        finally:
            b.close()

    sizes = [g for g in GROUP_SIZES if g <= max(len(systems), GROUP_SIZES[0])]
    best, times = best_of(sizes, measure)
    out = {"group_size": best, "ms_per_step": times[best], "tried": {str(g): t for g, t in times.items()}}
    if cache:
        table[key] = out
        _store("batch", table)
    return out


def apply(system, choice: Dict) -> None:
    """Sets a handle's launch shape to a tune_handle choice (the cell factor
    is a creation option: build the handle's case with choice["cs_ratio"])."""
    system.set_launch(choice["pipeline_chunks"], choice["force_blocks_per_sm"], choice.get("first_chunk_percent", -1))
