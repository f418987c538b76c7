"""Replica-parallel runs: one process per GPU, each advancing its own
independent copy of the workload (the hot path has no data exchange between
GPUs when each process owns whole problems).  The job's throughput is the work
all ranks did divided by the slowest rank's time.

Used by bench.py under torchrun (NCCL, CUDA tensors) and tested with gloo on
the CPU.
"""
from __future__ import annotations


def world():
    """(world_size, rank) of the default process group, (1, 0) without one."""
    import torch.distributed as tdist
    if tdist.is_available() and tdist.is_initialized():
        return tdist.get_world_size(), tdist.get_rank()
    return 1, 0


def max_over_ranks(value: float, device: str = "cpu") -> float:
    """The largest `value` over all ranks (identity without a process group).
    device: where the reduction tensor lives ("cuda" for NCCL, "cpu" for gloo)."""
    import torch
    import torch.distributed as tdist
    ws, _ = world()
    if ws == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(units_per_rank: float, seconds_slowest: float, world_size: int) -> float:
    """Units per second of the whole job: every rank processed units_per_rank
    in at most seconds_slowest (weak scaling: per-rank work fixed)."""
    if seconds_slowest <= 0.0:
        raise ValueError("seconds_slowest must be positive")
    return world_size * units_per_rank / seconds_slowest
