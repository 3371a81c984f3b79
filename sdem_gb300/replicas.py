"""Replica runs across GPUs: one independent bed per rank, no collective on the
data path (one bed is not split across GPUs).  Only the timing
is reduced: barrier before and after the timed region, max of the elapsed time
and sum of the particles over ranks."""
from __future__ import annotations

import os


def world():
    """(world_size, rank, local_rank) from the torchrun environment."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def rank_seed(base_seed: int, rank: int) -> int:
    return base_seed + rank


def aggregate(elapsed_s: float, n_particles: int, steps: int, device=None):
    """-> (particle-steps/s of the whole job, max elapsed, total particles)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return n_particles * steps / elapsed_s, elapsed_s, n_particles
    t_max = torch.tensor([elapsed_s], dtype=torch.float64, device=device)
    n_sum = torch.tensor([float(n_particles)], dtype=torch.float64, device=device)
    dist.all_reduce(t_max, op=dist.ReduceOp.MAX)
    dist.all_reduce(n_sum, op=dist.ReduceOp.SUM)
    return float(n_sum.item()) * steps / float(t_max.item()), float(t_max.item()), int(n_sum.item())
