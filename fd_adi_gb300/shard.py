"""Sharding a batch of independent options across GPUs (one process per GPU).

Options are independent units, so a multi-GPU run partitions the option list
with no device collective: each rank prices its shard and only the prices
travel (gathered on the host). Shards are balanced by work (grid points), the
longest-processing-time-first rule.
"""
import heapq

import numpy as np


def partition(costs, world):
    """Split indices 0..n-1 into `world` lists of near-equal total cost.

    Each list keeps ascending index order so a shard's arena stays grouped by
    grid size when the input was."""
    costs = np.asarray(costs, dtype=np.float64)
    if world < 1:
        raise ValueError("world must be >= 1")
    heap = [(0.0, r) for r in range(world)]
    heapq.heapify(heap)
    owner = np.empty(costs.size, dtype=np.int64)
    for k in np.argsort(-costs, kind="stable"):
        load, r = heapq.heappop(heap)
        owner[k] = r
        heapq.heappush(heap, (load + costs[k], r))
    return [np.flatnonzero(owner == r).tolist() for r in range(world)]


def shard_of(costs, rank, world):
    return partition(costs, world)[rank]
