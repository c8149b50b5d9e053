"""Multi-process helpers for running independent transforms on several GPUs.

The transform of one matrix does not exchange data between devices: each
rank transforms its own matrices (weak scaling, no collective on the data
path).  Only timing is combined -- the slowest rank decides the job time.
"""
from __future__ import annotations

import os


def world() -> tuple[int, int, int]:
    """(world_size, rank, local_rank) from the torchrun environment."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def max_over_ranks(value: float, device=None) -> float:
    """All-reduce MAX of one float (no-op without an initialised process group)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device or "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_ms_per_fft(rank_total_ms: float, steps: int, world_size: int, device=None) -> float:
    """Whole-job time per transform: the slowest rank's total over every
    rank's transforms."""
    return max_over_ranks(rank_total_ms, device) / float(steps * world_size)
