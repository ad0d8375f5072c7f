"""Multi-process layout of the ray-cast workload: one process per GPU.

The path shards without exchange: every rank traces its own rays against its
own copy of the BVH (weak scaling), so the only communication is the timing
reduction at the end -- the slowest rank's time, over which the aggregate
rate of all ranks is taken.  Used by bench.py under torchrun (NCCL) and
tested with gloo ranks on the CPU.
"""
from __future__ import annotations

import os


def dist_env() -> tuple[int, int, int]:
    """(world size, rank, local rank) from the torchrun environment."""
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def ray_stream(rank: int) -> int:
    """Seed stream of a rank's rays: ranks draw disjoint, reproducible sets."""
    return 3 + rank


def max_over_ranks(values: list[float], device=None) -> list[float]:
    """Element-wise maximum of per-rank values over all ranks (identity for a
    single process); device: where the reduction tensor lives (cuda for
    NCCL, cpu for gloo)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return list(values)
    t = torch.tensor(values, dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t.tolist()]


def aggregate_rate(units_per_rank: int, world_size: int, seconds: float) -> float:
    """Whole-job rate: all ranks' units over the slowest rank's time."""
    return world_size * units_per_rank / seconds
