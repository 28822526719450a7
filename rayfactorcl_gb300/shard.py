"""Ray-range sharding across processes (one process per GPU).

A ray's Philox stream depends only on (emitter, ray index), so emitter e's rays
[0, rays[e]) can be cut into contiguous ranges on draw boundaries (four rays per
draw, RayFactorGPU.cl:497-506), traced by different processes with
``Tracer.trace_range`` and summed: the tallies equal one single-process run.
The only exchange is one sum of the n x n int64 tally matrix (the reference's
per-device tally buffers summed on the host, RayFactorCL/main.cpp:224-234).
"""
from __future__ import annotations

import numpy as np


def shard_ranges(rays, rank: int, world: int):
    """(first_ray, count) per emitter for `rank` of `world`, split on draws."""
    if world <= 0 or not (0 <= rank < world):
        raise ValueError("need 0 <= rank < world")
    rays = np.asarray(rays, np.int64)
    if np.any(rays < 0):
        raise ValueError("negative budget")
    draws = (rays + 3) // 4
    lo = np.minimum(draws * rank // world * 4, rays)
    hi = np.minimum(draws * (rank + 1) // world * 4, rays)
    return lo, hi - lo


def trace_sharded(trace_range, rays, group=None, device=None):
    """Run this process's share and sum the tallies over the process group.

    ``trace_range(first, count)`` traces the given ranges and returns the local
    int64 n x n tallies (for the CUDA library: ``Tracer.trace_range`` followed by
    ``Tracer.results()[0]``).  Returns (tallies of the whole run, F in FP64).
    """
    import torch
    import torch.distributed as dist

    rank = dist.get_rank(group) if dist.is_initialized() else 0
    world = dist.get_world_size(group) if dist.is_initialized() else 1
    rays = np.asarray(rays, np.int64)
    first, count = shard_ranges(rays, rank, world)
    local = np.ascontiguousarray(trace_range(first, count), np.int64)
    t = torch.from_numpy(local)
    if device is not None:
        t = t.to(device)
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    hits = t.cpu().numpy()
    with np.errstate(invalid="ignore", divide="ignore"):
        F = hits / rays[:, None].astype(np.float64)
    return hits, F
