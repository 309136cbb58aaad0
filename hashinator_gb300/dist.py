"""Replica bookkeeping for multi-GPU runs.

The hot path does not shard a single map across GPUs: every rank serves its
own maps (replicas), so there is no exchange step on the data path. The only
collective is the timing aggregation of a benchmark: a barrier before the
timed region and the maximum elapsed time over ranks after it.
"""
from __future__ import annotations

import os


def env_ranks() -> tuple[int, int, int]:
    """(world size, rank, local rank) from the torchrun environment."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def replica_seed(base: int, rank: int) -> int:
    """Each replica works on its own seeded input."""
    return base + 7919 * rank


def max_over_ranks(value: float, device=None) -> float:
    """Maximum of a per-rank float over the default process group (identity
    without one)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_throughput(units_per_rank: int, elapsed_s: float, device=None) -> tuple[float, float]:
    """Whole-job throughput (all ranks' units over the slowest rank's time)
    and that time."""
    import torch.distributed as dist
    world = dist.get_world_size() if (dist.is_available() and dist.is_initialized()) else 1
    t = max_over_ranks(elapsed_s, device)
    return world * units_per_rank / t, t
