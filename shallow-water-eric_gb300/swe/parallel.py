"""Multi-process helpers (one process per GPU).

The explicit step of one mesh has no data-parallel exchange here: ranks run
independent replicas, or independent shards of a batch of meshes.  The only
inter-rank operations are a barrier around the timed region and the max (or
sum) of per-rank numbers.  torch.distributed is plumbing: NCCL on GPUs, gloo
on the CPU in tests.
"""
from __future__ import annotations

import numpy as np


def shard_instances(sizes, world: int, rank: int):
    """Indices of the instances rank `rank` advances: greedy longest-first
    assignment to the least loaded rank, by node count (every instance exactly
    once, loads within one instance of each other)."""
    sizes = np.asarray(sizes, dtype=np.int64)
    order = np.argsort(-sizes, kind="stable")
    load = np.zeros(world, dtype=np.int64)
    owner = np.empty(len(sizes), dtype=np.int64)
    for i in order:
        r = int(np.argmin(load))
        owner[i] = r
        load[r] += sizes[i]
    return [int(i) for i in np.nonzero(owner == rank)[0]]


def allreduce_max(value: float, dist=None, device=None) -> float:
    """Max of a per-rank scalar over all ranks (identity without dist)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def allreduce_sum(value: float, dist=None, device=None) -> float:
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def aggregate_throughput(units_this_rank: float, seconds_this_rank: float, dist=None, device=None) -> float:
    """Whole-job throughput: units processed by all ranks / slowest rank's time."""
    total = allreduce_sum(units_this_rank, dist, device)
    slowest = allreduce_max(seconds_this_rank, dist, device)
    return total / slowest
