"""Work sharding across ranks, one process per GPU, for the batched trackers.

Alignment pairs (SE3 batches) and Sim3 candidate trackings are independent, so each rank tracks its
own share in its own persistent launch and nothing crosses ranks on the data path.  The only
collectives are host-side and outside the timed work: the max of the ranks' times, and the gather
of poses and statistics to rank 0 afterwards.  A single keyframe's depth update is too small to
split; ranks run replicas on different keyframes.

The partition is longest-processing-time first on a per-pair cost (level-0 pixel count, which
the number of keyframe points and pyramid pixels follow): deterministic, every pair exactly once,
and no rank above the ideal share by more than one pair's cost.
"""
from __future__ import annotations

import os

import numpy as np


def rank_env():
    """(rank, world_size, local_rank) from the launcher's environment (torchrun sets them)."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def pair_cost(width: int, height: int) -> int:
    return int(width) * int(height)


def partition(costs, world: int):
    """Indices of the work items of every rank: largest first, each to the least-loaded rank
    (ties: the lower rank); every rank's list in ascending index order."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    load = [0] * world
    parts = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda q: (load[q], q))
        parts[r].append(i)
        load[r] += costs[i]
    return [sorted(p) for p in parts]


def my_share(costs, rank: int, world: int):
    return partition(costs, world)[rank]


def max_over_ranks(x: float, dist=None, device=None) -> float:
    """The largest of the ranks' values (every rank gets it); `dist` is torch.distributed or None."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(x: float, dist=None, device=None) -> float:
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def gather_rows(indices, rows, n: int, dist=None):
    """Reassemble per-item results computed on different ranks: rank r holds rows for its
    `indices`; every rank returns the (n, ...) array in item order."""
    rows = np.asarray(rows)
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        out = np.empty((n,) + rows.shape[1:], rows.dtype)
        out[list(indices)] = rows
        return out
    parts = [None] * dist.get_world_size()
    dist.all_gather_object(parts, (list(indices), rows))
    shape, dtype = None, None
    for idx, r in parts:
        if len(idx):
            shape, dtype = r.shape[1:], r.dtype
            break
    out = np.empty((n,) + (shape or rows.shape[1:]), dtype or rows.dtype)
    seen = np.zeros(n, bool)
    for idx, r in parts:
        if len(idx):
            out[idx] = r
            seen[idx] = True
    if not seen.all():
        raise RuntimeError("items missing after the gather: %s" % np.nonzero(~seen)[0][:8])
    return out
