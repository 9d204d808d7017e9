"""Multi-GPU partition of an xbatched batch by Y-block ownership.

Entries are independent, and every contribution to one Y block can be kept
on the GPU that owns that block: sort the entries by Y block, cut the sorted
order into one contiguous range of Y blocks per rank with about equal work,
and each rank runs its entries against its own Y blocks.  No reduction
collective is needed on the data path: after the call every Y block is
complete on exactly one rank.  X blocks and factor pools are read-only and
may be replicated (or each rank gathers the X blocks its entries use).

The planner is pure host code (numpy); ``tests/test_shard.py`` checks it
with ``gloo`` ranks on the CPU against a single-process sum.
"""
from __future__ import annotations

import numpy as np


def plan_by_y_owner(y_idx, world: int, weights=None):
    """Split entries into ``world`` shards so that each Y block belongs to one
    shard and the shards' work (entry count, or the sum of ``weights``) is as
    even as contiguous ranges of Y blocks allow.

    Returns (entry_ids per rank, (y_lo, y_hi) Y-block range per rank)."""
    y_idx = np.asarray(y_idx)
    if world < 1:
        raise ValueError("world must be >= 1")
    w = np.ones(len(y_idx)) if weights is None else np.asarray(weights, dtype=np.float64)
    order = np.argsort(y_idx, kind="stable")
    ys = y_idx[order]
    if len(ys) == 0:
        return [np.zeros(0, dtype=np.int64) for _ in range(world)], [(0, 0)] * world
    # cumulative work at each distinct Y block boundary
    cw = np.cumsum(w[order])
    total = cw[-1]
    bounds = [0]
    for r in range(1, world):
        target = total * r / world
        cut = int(np.searchsorted(cw, target, side="left"))
        # move the cut to the next Y-block boundary so one block never straddles ranks
        while 0 < cut < len(ys) and ys[cut] == ys[cut - 1]:
            cut += 1
        bounds.append(max(cut, bounds[-1]))
    bounds.append(len(ys))
    shards, ranges = [], []
    for r in range(world):
        a, b = bounds[r], bounds[r + 1]
        shards.append(order[a:b])
        ranges.append((int(ys[a]) if b > a else 0, int(ys[b - 1]) + 1 if b > a else 0))
    return shards, ranges


def owner_of(y_block: int, ranges) -> int:
    """Rank owning a Y block (-1 if none of the ranges holds it)."""
    for r, (lo, hi) in enumerate(ranges):
        if lo <= y_block < hi:
            return r
    return -1
