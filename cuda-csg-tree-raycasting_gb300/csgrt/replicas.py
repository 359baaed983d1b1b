"""Multi-GPU replicas: one process per GPU, no collective on the data path.

Every ray is independent and scenes are small and read-only, so several GPUs render
independent work: the same frame on every rank (weak scaling of the single-view
benchmark), or disjoint shards of a batch's views.  The only communication is the
benchmark's bookkeeping: a barrier around the timed region and the maximum of the ranks'
times.  torch.distributed carries it (NCCL between GPUs, gloo on CPU for the tests).
"""
from __future__ import annotations

import os


def dist_info():
    """(world size, rank, local rank) from the torchrun environment (1, 0, 0 without)."""
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def init(backend: str = "nccl", device=None):
    """Joins the process group when there is more than one rank; returns the
    torch.distributed module, or None for a single process."""
    ws, _, _ = dist_info()
    if ws <= 1:
        return None
    import torch.distributed as dist
    if not dist.is_initialized():
        if device is not None:
            dist.init_process_group(backend, device_id=device)
        else:
            dist.init_process_group(backend)
    return dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, value: float, device="cpu") -> float:
    """The largest of the ranks' values (the job's time is its slowest rank's)."""
    if dist is None:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def shard(costs, rank: int, world: int):
    """Indices of the views rank `rank` renders: views sorted by cost (most expensive
    first) and dealt out greedily to the least-loaded rank, so every view is rendered by
    exactly one rank and the ranks' loads are balanced."""
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    load = [0.0] * world
    mine = []
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        load[r] += costs[i]
        if r == rank:
            mine.append(i)
    return sorted(mine)


def throughput(units_per_rank, world: int, max_ms: float) -> float:
    """Whole-job rate: the units all ranks processed over the slowest rank's time (units
    per second)."""
    total = units_per_rank * world if not isinstance(units_per_rank, (list, tuple)) else sum(units_per_rank)
    return total / (max_ms * 1e-3)
