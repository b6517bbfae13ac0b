"""Whole-job accounting for N independent replicas (one process per GPU).

The operator does not shard across GPUs: with N GPUs every rank runs the
same workload on its own device with no data-path collective.  The job's
time is the slowest rank's time and its throughput the units of all ranks
over that time.  Works on any torch.distributed backend (gloo on CPU, NCCL
on GPUs) or without one (N = 1).
"""
from __future__ import annotations


def job_throughput(local_units: float, local_seconds: float, device=None) -> tuple[float, float, int]:
    """Returns (total units / max seconds, max seconds, world size)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return local_units / local_seconds, local_seconds, 1
    t = torch.tensor([local_seconds], dtype=torch.float64, device=device)
    u = torch.tensor([local_units], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    secs = float(t.item())
    return float(u.item()) / secs, secs, dist.get_world_size()
