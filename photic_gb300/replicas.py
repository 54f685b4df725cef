"""Multi-GPU as replicas: every pixel is independent, so N ranks (one
process per GPU, launched by torchrun) each fit their own shard of the
scene with no collective on the data path.  The only collectives are the
barrier around the timed region, the max over ranks of the step time and
the sum of the per-rank pixel counts.  The functions here are that logic,
testable on CPU with the gloo backend."""
from __future__ import annotations

import os
from typing import Optional, Tuple


def world() -> Tuple[int, int, int]:
    """(world size, rank, local rank) from the launcher's environment."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def shard_start(rank: int, pixels_per_rank: int) -> int:
    """First pixel id of a rank's shard (weak scaling: a fixed shard size per
    rank; the generator is keyed by pixel id, so shards never overlap)."""
    if rank < 0 or pixels_per_rank < 0:
        raise ValueError("rank and shard size must be non-negative")
    return rank * pixels_per_rank


def max_over_ranks(value: float, dist=None, device=None) -> float:
    """The largest value over all ranks (the step time the job is charged)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value: float, dist=None, device=None) -> float:
    """The sum over all ranks (pixels fitted by the whole job)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t)
    return float(t.item())


def job_rate(total_units: float, slowest_seconds: float) -> float:
    """Whole-job throughput: all ranks' units over the slowest rank's time."""
    if slowest_seconds <= 0:
        raise ValueError("time must be positive")
    return total_units / slowest_seconds


def init(backend: str = "nccl", device: Optional[object] = None):
    """Initialise torch.distributed from the environment when WORLD_SIZE > 1;
    returns the module (or None for one rank)."""
    ws, _, _ = world()
    if ws <= 1:
        return None
    import torch.distributed as dist
    if not dist.is_initialized():
        if device is not None and backend == "nccl":
            dist.init_process_group(backend, device_id=device)
        else:
            dist.init_process_group(backend)
    return dist
