"""Sharding a batched smoothing problem across processes, one GPU each.

The tracks of a packed problem are independent, so the batched smoothers
shard by track: each rank smooths a contiguous range of tracks on its own GPU
and nothing crosses between GPUs while they smooth.  The only exchange is the
host-side merge of the results on rank 0 afterwards.  A track is never split:
a single long track runs on one GPU.

``split_tracks`` balances the ranks by steps (the smoothing time of a batch
grows with its step count); ``shard`` cuts a rank's part out of a packed
problem; ``merge`` gathers per-rank arrays (states, or covariances) on rank 0
in track order through ``torch.distributed`` (any backend: gloo between CPU
processes, NCCL between GPUs), after the smoothing, off the data path.
"""
from __future__ import annotations

import numpy as np


def split_tracks(track_lengths, world: int) -> np.ndarray:
    """Track bounds [world + 1] of `world` contiguous ranges whose step counts
    are as even as whole tracks allow: rank r gets tracks bounds[r] ..
    bounds[r+1] - 1, each inner bound the track boundary whose step prefix is
    nearest to r/world of the total.  Ranges may be empty (fewer tracks than
    ranks, or one track longer than a rank's share)."""
    if world < 1:
        raise ValueError("world must be >= 1")
    lengths = np.asarray(track_lengths, dtype=np.int64)
    if (lengths < 0).any():
        raise ValueError("track lengths must be >= 0")
    prefix = np.concatenate([[0], np.cumsum(lengths)])
    total = prefix[-1]
    T = len(lengths)
    bounds = np.zeros(world + 1, dtype=np.int64)
    bounds[world] = T
    for r in range(1, world):
        target = (total * r) // world
        # the track boundary nearest the target, never before the previous bound
        b = int(np.searchsorted(prefix, target, side="left"))
        if b > 0 and (b > T or target - prefix[b - 1] <= prefix[b] - target):
            b -= 1
        bounds[r] = min(max(b, bounds[r - 1]), T)
    return bounds


def shard(P, rank: int, world: int):
    """(rank's packed problem, (first track, end track)) of a PackedProblem;
    the problem is None for a rank left without tracks."""
    if not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside [0, {world})")
    b = split_tracks(P.track_lengths(), world)
    t0, t1 = int(b[rank]), int(b[rank + 1])
    return (P.select_tracks(range(t0, t1)) if t1 > t0 else None), (t0, t1)


def merge(local, rank: int, world: int, group=None):
    """Gathers every rank's array (rows in the rank's track order) on rank 0
    and returns their concatenation there, in rank order, which is track
    order; other ranks get None.  `local` is a NumPy array whose trailing
    dimensions agree across ranks (its first dimension may differ, or be 0)."""
    local = np.ascontiguousarray(local)
    if world == 1:
        return local
    import torch.distributed as dist
    parts = [None] * world if rank == 0 else None
    dist.gather_object(local, parts, dst=0, group=group)
    if rank != 0:
        return None
    return np.concatenate(parts, axis=0)
