"""Spreading independent transforms over several GPUs ("replicas only").

The raster scan does not shard a single image or volume (every row depends
on the whole previous row), so with several GPUs each rank takes a share of
the independent items -- images, volumes, requests -- and no collective is
needed on the data path.  `partition` assigns items to ranks by their cost
(largest first onto the least-loaded rank), so every rank can compute the same
assignment locally from the item sizes.
"""
from __future__ import annotations

import heapq
from typing import List, Sequence


def transform_cost(shape: Sequence[int], iterations: int = 1) -> float:
    """Cost of one item in voxel-passes (cells x passes x iterations):
    `shape` is (H, W) or (D, H, W)."""
    cells = 1.0
    for s in shape:
        cells *= float(s)
    return cells * 2 * len(shape) * max(1, iterations)


def partition(costs: Sequence[float], world: int) -> List[List[int]]:
    """Indices of the items each of `world` ranks processes (longest
    processing time first).  Deterministic: ties break on the item index."""
    if world < 1:
        raise ValueError("world size must be at least 1")
    order = sorted(range(len(costs)), key=lambda i: (-float(costs[i]), i))
    heap = [(0.0, r) for r in range(world)]
    out: List[List[int]] = [[] for _ in range(world)]
    for i in order:
        load, r = heapq.heappop(heap)
        out[r].append(i)
        heapq.heappush(heap, (load + float(costs[i]), r))
    for r in range(world):
        out[r].sort()
    return out
