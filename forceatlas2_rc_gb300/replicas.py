"""Replica sharding across GPUs.

Layouts of different graphs are independent, so several GPUs only ever run
replicas: each rank takes its share of the graphs (or one whole copy of a
benchmark layout) and nothing is exchanged on the data path. The one
collective is the timing reduction (the slowest rank defines the job's
time).
"""
from __future__ import annotations

import heapq
from typing import Sequence


def shard_graphs(nodes: Sequence[int], edges: Sequence[int], world_size: int,
                 rank: int) -> list:
    """Indices of the graphs rank `rank` lays out.

    Graphs go, largest cost first, to the rank with the least cost so far
    (greedy longest-processing-time); cost = nodes + edges, the work of one
    iteration. Deterministic: every rank computes the same assignment without
    communicating.
    """
    if world_size < 1 or not 0 <= rank < world_size:
        raise ValueError("invalid rank / world size")
    cost = [int(n) + int(e) for n, e in zip(nodes, edges)]
    order = sorted(range(len(cost)), key=lambda i: (-cost[i], i))
    heap = [(0, r) for r in range(world_size)]
    mine = []
    for i in order:
        load, r = heapq.heappop(heap)
        if r == rank:
            mine.append(i)
        heapq.heappush(heap, (load + cost[i], r))
    return sorted(mine)


def max_over_ranks(value: float, device=None) -> float:
    """The maximum of `value` over the ranks of the default process group
    (the value itself without one)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64,
                     device=device if device is not None else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
