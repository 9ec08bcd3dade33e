"""Environment sharding across processes (one process per GPU).

Environments are independent, so N GPUs simply own disjoint shards of environments and
never exchange data during a step. The only cross-process operations are for measurement
and bookkeeping: a barrier around timed regions and a max-reduction of step times, both
done with torch.distributed (NCCL between GPUs, gloo on CPU).
"""
from __future__ import annotations

import os


def dist_env():
    """(rank, world_size, local_rank) from the torchrun environment (1 process if absent)."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def shard_bounds(n_total, rank, world):
    """Contiguous [start, stop) of environments owned by `rank` when n_total environments
    are split over `world` processes (sizes differ by at most one)."""
    if world <= 0 or not 0 <= rank < world:
        raise ValueError("bad rank / world size")
    base, extra = divmod(int(n_total), int(world))
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def max_across_ranks(value, dist=None, device=None):
    """Maximum of a float over all ranks (identity without a process group)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_across_ranks(value, dist=None, device=None):
    """Sum of a float over all ranks (identity without a process group): the host-side
    reduction of a loss that is a sum of per-environment terms, each rank holding the
    partial sum over its own shard."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def aggregate_throughput(envs_per_rank, world, max_seconds):
    """Whole-job environment-steps per second: every rank's environments over the slowest
    rank's time."""
    return envs_per_rank * world / max_seconds
