"""Particle sharding across GPUs (one process per GPU).

Particles are independent and the fields are read-only, so a multi-GPU run
splits the particles and needs no data-path collective.  Weak scaling: rank
r of w integrates the seeded particles with global indices [r n, (r + 1) n)
(each particle's initial state is a function of its global index, so the
union over ranks is the single-GPU ensemble bit for bit).  Strong scaling of
one fixed particle set: contiguous ranges with equal expected work
(`weighted_ranges`), weighted by 1 / gamma (`expected_work`) or by the
attempts of a previous window.  Only the timing and the step counts are
combined: the slowest rank's time and the sum of steps.
"""
from __future__ import annotations

import numpy as np


def particle_indices(rank: int, per_rank: int) -> np.ndarray:
    """Global indices of the particles rank `rank` owns (weak scaling)."""
    return np.arange(rank * per_rank, (rank + 1) * per_rank, dtype=np.uint64)


def expected_work(state0: np.ndarray, b_rms: float = 1.0) -> np.ndarray:
    """Expected attempts of each particle per unit time, up to a common
    factor, from its initial state (the rows state(1:6, 1) of the reference
    layout, shape (n, 6)): steps resolve the gyration, whose frequency is
    qom |B| / gamma, so a particle's work goes as 1 / gamma (|B| ~ b_rms for
    all).  With gamma log-uniform over three decades the spread is ~1000x,
    which is why equal particle counts per GPU do not balance a run."""
    u = np.asarray(state0, np.float64)[:, 3:6]
    gamma = np.sqrt(1.0 + (u * u).sum(axis=1))
    return b_rms / gamma


def weighted_ranges(weights: np.ndarray, world: int) -> list[tuple[int, int]]:
    """Contiguous particle ranges [lo, hi) for `world` GPUs with equal sums of
    `weights` (expected work per particle, e.g. `expected_work` or the
    attempts of a previous window): range r ends at the cut whose prefix sum
    is closest to (r + 1) / world of the total, so each cut misses its
    target by at most half a particle's weight.  Every particle is in
    exactly one range; ranges may be empty only when there are fewer
    particles than GPUs."""
    w = np.asarray(weights, np.float64)
    if w.ndim != 1 or (w < 0).any() or not np.isfinite(w).all():
        raise ValueError("weights must be finite, non-negative and one-dimensional")
    if world < 1:
        raise ValueError("world must be >= 1")
    n = w.size
    c = np.cumsum(w)
    total = c[-1] if n else 0.0
    cuts = [0]
    for r in range(1, world):
        if total > 0:
            t = total * r / world
            k = int(np.searchsorted(c, t, side="left"))        # c[k] >= t: k + 1 particles
            below = c[k - 1] if k > 0 else 0.0                  # k particles
            k = k + 1 if (k < n and c[k] - t < t - below) else k
        else:
            k = (n * r) // world
        cuts.append(min(max(k, cuts[-1]), n))
    cuts.append(n)
    return [(cuts[r], cuts[r + 1]) for r in range(world)]


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
