"""Spreading independent components over GPUs (one process per GPU).

Components of a batch (or of a forest) are independent, so more than one GPU needs no
exchange on the data path: each rank closes its own share and only the timing (or a final
host gather) is combined.  ``shard_components`` balances a batch by the dense closure cost
n^3 with the longest-processing-time-first rule; ``max_over_ranks`` is the one collective the
bench uses (the slowest rank's time).
"""
from __future__ import annotations

import heapq

import numpy as np


def shard_components(sizes, world: int, cost_exponent: int = 3) -> list[np.ndarray]:
    """Indices of the components each of ``world`` ranks closes.  Greedy: components in
    decreasing cost (n ** cost_exponent) go to the rank with the least total so far; ties go
    to the lowest rank, so every rank computes the same split.  Each rank's indices ascend."""
    if world < 1:
        raise ValueError("world must be at least 1")
    sizes = np.asarray(sizes, dtype=np.int64)
    cost = sizes.astype(np.float64) ** cost_exponent
    order = np.lexsort((np.arange(sizes.size), -cost))   # decreasing cost, then index
    heap = [(0.0, r) for r in range(world)]
    parts: list[list[int]] = [[] for _ in range(world)]
    for i in order:
        load, r = heapq.heappop(heap)
        parts[r].append(int(i))
        heapq.heappush(heap, (load + float(cost[i]), r))
    return [np.array(sorted(p), dtype=np.int64) for p in parts]


def shard_cost(sizes, parts, cost_exponent: int = 3) -> np.ndarray:
    """Total cost per rank of a split."""
    sizes = np.asarray(sizes, dtype=np.float64)
    return np.array([float((sizes[p] ** cost_exponent).sum()) for p in parts])


def max_over_ranks(value: float, device=None) -> float:
    """The largest ``value`` over all ranks of the default process group (``value`` itself
    when torch.distributed is not initialised).  Works with gloo (CPU) and nccl (``device``)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
