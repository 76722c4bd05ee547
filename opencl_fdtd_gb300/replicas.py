"""
Multi-GPU runs of this path are replicas: the benchmark's units (whole simulations) are
independent, so each rank steps its own grid on its own GPU with no data-path collective.
The only communication is the timing: a barrier before and after the timed region and the
maximum of the ranks' elapsed times, from which the whole-job throughput follows.
"""
from __future__ import annotations

import os

import torch


def rank_info():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


def max_over_ranks(value: float, device=None) -> float:
    """The maximum of ``value`` over all ranks (the value itself without a process group)."""
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device or "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier():
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.barrier()


def job_throughput(cells_per_rank: int, steps: int, elapsed_ms_per_rank: float, world: int) -> float:
    """Whole-job Mcell-updates/s of ``world`` replicas, each advancing cells_per_rank cells
    for ``steps`` steps, timed by the slowest rank."""
    slowest = max_over_ranks(elapsed_ms_per_rank)
    return world * cells_per_rank * steps / (slowest * 1e-3) / 1e6
