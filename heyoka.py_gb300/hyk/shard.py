"""Sharding of an ensemble over GPUs (one process per GPU).

Trajectories are independent, so the multi-GPU path needs no collective on
the data path: every rank integrates a contiguous range of lanes on its own
device, and the host gathers the per-rank results.  The ranges are balanced
by an estimate of each lane's work (for instance the number of steps
predicted from one step size and the horizon), because the ensembles this
integrator serves have very uneven trajectories (the reference fans
iterations out over host threads or processes instead:
heyoka/_ensemble_impl.py:23-138).
"""

from __future__ import annotations

import numpy as np
import torch


def partition(n: int, world: int, weights=None):
    """Contiguous ``[lo, hi)`` lane ranges, one per rank, whose summed weights
    are as even as a prefix split allows (equal counts without weights)."""
    if world < 1:
        raise ValueError("the number of ranks must be positive")
    if n < 0:
        raise ValueError("the number of lanes must be non-negative")
    if weights is None:
        cuts = [(n * r) // world for r in range(world + 1)]
    else:
        w = np.asarray(weights, dtype=np.float64)
        if w.shape != (n,):
            raise ValueError("weights must have one entry per lane")
        if np.any(w < 0) or not np.all(np.isfinite(w)):
            raise ValueError("weights must be finite and non-negative")
        c = np.concatenate([[0.0], np.cumsum(w)])
        total = c[-1]
        cuts = [0]
        for r in range(1, world):
            k = int(np.searchsorted(c, total * r / world, side="left"))
            cuts.append(min(max(k, cuts[-1]), n))
        cuts.append(n)
    return [(cuts[r], cuts[r + 1]) for r in range(world)]


def local_range(n: int, weights=None, group=None):
    """This rank's lane range under ``torch.distributed`` (the whole range
    when the process group is not initialised)."""
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()):
        return (0, n)
    return partition(n, dist.get_world_size(group), weights)[dist.get_rank(group)]


def gather_lanes(local, n: int, weights=None, group=None, dst: int = 0):
    """Gather per-rank lane blocks (``(..., hi - lo)``, host or device) into
    the full ``(..., n)`` array on rank ``dst`` (None elsewhere).  Uses the
    host process group (gloo works): results travel once, after the
    propagation, so this is not on the data path."""
    import torch.distributed as dist

    t = torch.as_tensor(local).detach().to("cpu")
    if not (dist.is_available() and dist.is_initialized()):
        return t.numpy()
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    ranges = partition(n, world, weights)
    width = max(hi - lo for lo, hi in ranges)
    lo, hi = ranges[rank]
    if t.shape[-1] != hi - lo:
        raise ValueError("the local block has {} lanes, the partition gives {}".format(t.shape[-1], hi - lo))
    pad = torch.zeros(t.shape[:-1] + (width,), dtype=t.dtype)
    pad[..., : hi - lo] = t
    bufs = [torch.zeros_like(pad) for _ in range(world)] if rank == dst else None
    dist.gather(pad, bufs, dst=dst, group=group)
    if rank != dst:
        return None
    return torch.cat([b[..., : h - l] for b, (l, h) in zip(bufs, ranges)], dim=-1).numpy()
