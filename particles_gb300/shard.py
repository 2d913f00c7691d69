"""Particle sharding across GPUs (one process per GPU).

Particles are independent and the fields are read-only, so a multi-GPU run
splits the particles and needs no data-path collective: rank r of w
integrates the seeded particles with global indices [r n, (r + 1) n) (each
particle's initial state is a function of its global index, so the union
over ranks is the single-GPU ensemble bit for bit).  Only the timing and the
step counts are combined: the slowest rank's time and the sum of steps.
"""
from __future__ import annotations

import numpy as np


def particle_indices(rank: int, per_rank: int) -> np.ndarray:
    """Global indices of the particles rank `rank` owns (weak scaling)."""
    return np.arange(rank * per_rank, (rank + 1) * per_rank, dtype=np.uint64)


def combine(torch, elapsed_s: float, steps: float, device=None):
    """(max elapsed over ranks, sum of steps over ranks) with torch.distributed;
    the identity without an initialised process group."""
    dist = torch.distributed
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(elapsed_s), float(steps)
    t = torch.tensor([elapsed_s], dtype=torch.float64, device=device)
    a = torch.tensor([steps], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(a, op=dist.ReduceOp.SUM)
    return float(t.item()), float(a.item())
