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


def _parse_cpulist(text: str) -> set:
    """'0-3,8,10-11' -> {0, 1, 2, 3, 8, 10, 11}."""
    cpus = set()
    for part in text.strip().split(","):
        if not part:
            continue
        if "-" in part:
            a, b = part.split("-")
            cpus.update(range(int(a), int(b) + 1))
        else:
            cpus.add(int(part))
    return cpus


def gpu_local_cpus(pci_bus_id: str, sysfs: str = "/sys") -> set:
    """CPUs of the NUMA node the GPU at `pci_bus_id` (e.g. "00000009:01:00.0")
    is attached to, from sysfs; an empty set when the node is unknown."""
    import os
    dom, rest = pci_bus_id.strip().lower().split(":", 1)
    dev = f"{int(dom, 16):04x}:{rest}"
    try:
        with open(os.path.join(sysfs, "bus", "pci", "devices", dev, "numa_node")) as f:
            node = int(f.read().strip())
        if node < 0:
            return set()
        with open(os.path.join(sysfs, "devices", "system", "node", f"node{node}", "cpulist")) as f:
            return _parse_cpulist(f.read())
    except (OSError, ValueError):
        return set()


def bind_local_cpus(device: int = 0) -> list:
    """Restrict this process to the CPUs next to GPU `device` (before any pinned
    host memory is allocated: first touch then places it on that node, so
    host-device copies take the GPU's own CPU link).  Returns the CPUs bound,
    [] when the placement could not be determined (then nothing changes)."""
    import os
    import subprocess
    try:
        out = subprocess.run(["nvidia-smi", "--query-gpu=pci.bus_id", "--format=csv,noheader", "-i", str(device)],
                             capture_output=True, text=True, timeout=30)
        cpus = gpu_local_cpus(out.stdout.strip()) if out.returncode == 0 else set()
        cpus &= os.sched_getaffinity(0)
        if not cpus:
            return []
        os.sched_setaffinity(0, cpus)
        return sorted(cpus)
    except (OSError, ValueError, subprocess.SubprocessError):
        return []
