"""Sharding of independent pressure systems across ranks (one GPU each).

Batched solves need no exchange between systems, so N ranks split the
systems and each solves its share as one batch; no collective is on the
data path (the bench reduces only its timings).  The split is the greedy
longest-processing-time rule on the systems' nonzero counts: systems in
decreasing size go to the currently lightest rank (ties to the lowest
rank), which keeps the heaviest rank within max(size) of the mean load.
"""
from __future__ import annotations

import heapq


def partition_by_nnz(sizes, world: int):
    """List of system indices per rank (each list in increasing order)."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(sizes)), key=lambda i: (-sizes[i], i))
    heap = [(0, r) for r in range(world)]
    out = [[] for _ in range(world)]
    for i in order:
        load, r = heapq.heappop(heap)
        out[r].append(i)
        heapq.heappush(heap, (load + sizes[i], r))
    return [sorted(x) for x in out]


def my_share(sizes, rank: int, world: int):
    return partition_by_nnz(sizes, world)[rank]
