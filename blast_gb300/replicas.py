"""Multi-GPU use is replicas only: every matrix is independent, so ranks split a batch by
instance and exchange nothing on the data path.

* ``shard_by_cost`` splits a ragged batch over ranks so that each rank's sum of per-instance
  costs (e.g. n^3 flops) is balanced (longest-processing-time-first greedy assignment).
* ``max_over_ranks`` is the one collective the benchmark uses: the step time of the slowest rank.
* ``gather_info`` concatenates per-instance status arrays on rank 0 (host side, optional).
"""
from __future__ import annotations

import heapq

import numpy as np
import torch


def shard_by_cost(costs, world: int) -> list[np.ndarray]:
    """Instance indices for each rank; the largest costs are placed first on the least-loaded rank."""
    costs = np.asarray(costs, dtype=np.float64)
    if world <= 0:
        raise ValueError("world must be positive")
    heap = [(0.0, r) for r in range(world)]
    parts: list[list[int]] = [[] for _ in range(world)]
    for i in np.argsort(-costs, kind="stable"):
        load, r = heapq.heappop(heap)
        parts[r].append(int(i))
        heapq.heappush(heap, (load + float(costs[i]), r))
    return [np.sort(np.asarray(p, dtype=np.int64)) for p in parts]


def max_over_ranks(value: float, device=None) -> float:
    """Maximum of a scalar over all ranks of the default process group (identity without one)."""
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def gather_info(local: np.ndarray, indices: np.ndarray, total: int):
    """Rank 0 receives every rank's per-instance status in global instance order; other ranks get
    None. Uses the default process group (gloo for host tensors)."""
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        out = np.zeros(total, dtype=np.int32)
        out[indices] = local
        return out
    pairs = [None] * dist.get_world_size()
    dist.all_gather_object(pairs, (np.asarray(indices), np.asarray(local)))
    if dist.get_rank() != 0:
        return None
    out = np.zeros(total, dtype=np.int32)
    for idx, val in pairs:
        out[idx] = val
    return out
