"""Multi-process layout of the ray-cast and render workloads: one process per GPU.

The path shards without exchange: every rank traces its own rays against its
own copy of the BVH, or renders its own sample set of the view (weak
scaling), so the only communication is
  * the timing reduction at the end -- the slowest rank's time, over which
    the aggregate rate of all ranks is taken, and
  * for renders, one sum of the films: the reference's scheduler adds its
    workers' films and rescales by the total sample count
    (scheduler.cpp:281-288); reduce_film does the same across ranks.
Used by bench.py under torchrun (NCCL) and tested with gloo ranks on the CPU.
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


def rank_seed(seed: int, rank: int) -> int:
    """Seed of a rank's share of a render: the renderers' random numbers are
    a counter-based function of (seed, sample), so distinct seeds give
    independent sample sets; rank 0 keeps the caller's seed."""
    return (seed + 0x9E3779B1 * rank) & 0xFFFFFFFF


def reduce_film(image, variance, spp: int, device=None):
    """Combines the films of ranks that rendered independent sample sets of
    the same view: the spp-weighted mean of the images, sum_r spp_r img_r /
    N, and the variance of that estimate, sum_r spp_r^2 var_r / N^2 (each
    rank's variance is that of its own mean), with N = sum_r spp_r.  Returns
    (image, variance, N) on every rank (the inputs for a single process).
    image, variance: (H, W, 3) arrays; device: where the reduction tensors
    live (cuda for NCCL, cpu for gloo)."""
    import numpy as np
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return image, variance, spp
    w = float(spp)
    t = torch.from_numpy(np.stack([np.asarray(image, np.float64) * w, np.asarray(variance, np.float64) * (w * w)]))
    t = t.to(device) if device is not None else t
    n = torch.tensor([w], dtype=torch.float64, device=t.device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    dist.all_reduce(n, op=dist.ReduceOp.SUM)
    total = float(n.item())
    out = t.cpu().numpy()
    return out[0] / total, out[1] / (total * total), int(round(total))
