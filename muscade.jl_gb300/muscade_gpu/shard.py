"""Sharding of independent models across GPUs (one process per GPU).

Independent models (risers, reliability samples, the perturbed solves of a
finite-difference check) share nothing, so N GPUs split them and need no
collective on the data path: each rank builds and solves its own share, and
the host gathers the per-model results at the end (a gather of Python objects
over the process group's backend, gloo on CPU or NCCL on GPUs).
"""
from __future__ import annotations

import numpy as np


def shard_bounds(costs, world: int):
    """Contiguous [start, end) ranges of the items for each rank, balanced by
    cumulative cost (e.g. element counts): rank r takes the items whose cost
    prefix falls in the r-th equal share of the total.  Every item goes to
    exactly one rank; a rank may get none when there are fewer items than ranks."""
    c = np.asarray(costs, dtype=np.float64)
    if world < 1:
        raise ValueError("world must be >= 1")
    if c.size == 0:
        return [(0, 0)] * world
    if np.any(c < 0):
        raise ValueError("costs must be non-negative")
    pre = np.concatenate([[0.0], np.cumsum(c)])
    total = pre[-1]
    # item i goes to the rank of the share that holds its midpoint
    mid = (pre[:-1] + pre[1:]) / 2
    owner = np.minimum((mid / total * world).astype(np.int64), world - 1) if total > 0 else \
        np.minimum(np.arange(c.size) * world // c.size, world - 1)
    owner = np.maximum.accumulate(owner)  # keep ranges contiguous and ordered
    bounds = []
    for r in range(world):
        idx = np.flatnonzero(owner == r)
        bounds.append((int(idx[0]), int(idx[-1]) + 1) if idx.size else (None, None))
    # fill empty ranks with empty ranges at their neighbour's boundary
    out, last = [], 0
    for b in bounds:
        if b[0] is None:
            out.append((last, last))
        else:
            out.append(b)
            last = b[1]
    return out


def my_share(items, costs, rank: int, world: int):
    """The items of `rank` (a slice of the list) and their global indices."""
    lo, hi = shard_bounds(costs, world)[rank]
    return items[lo:hi], np.arange(lo, hi)


def gather_to_root(obj, dist=None):
    """All ranks' `obj` on rank 0 (list by rank), None elsewhere; without a
    process group, [obj]."""
    if dist is None or not dist.is_initialized():
        return [obj]
    world = dist.get_world_size()
    out = [None] * world if dist.get_rank() == 0 else None
    dist.gather_object(obj, out, dst=0)
    return out
