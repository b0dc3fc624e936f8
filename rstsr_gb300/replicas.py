"""Replica timing for runs on several GPUs of one node.

The hot path has no exchange step (an element-wise op, a reduction or a
matmul on one device never needs another device's data), so N GPUs run N
independent replicas, one process per GPU. A run's figure is the work of all
replicas over the slowest replica's time; the only collective is the max of
the per-rank times (and a barrier around the timed region), on whatever
process group the caller set up (NCCL on GPUs, gloo on CPU in the tests).
"""

from __future__ import annotations


def world_size() -> int:
    import torch.distributed as dist

    return dist.get_world_size() if dist.is_available() and dist.is_initialized() else 1


def barrier() -> None:
    import torch.distributed as dist

    if world_size() > 1:
        dist.barrier()


def max_over_ranks(seconds: float, device: str = "cpu") -> float:
    """The slowest rank's time (every rank gets it)."""
    import torch
    import torch.distributed as dist

    if world_size() == 1:
        return float(seconds)
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank: float, seconds: float, device: str = "cpu") -> tuple[float, float]:
    """(units of all ranks per second over the slowest rank's time, that time);
    every rank processes `units_per_rank` (weak scaling)."""
    t = max_over_ranks(seconds, device)
    return units_per_rank * world_size() / t, t
