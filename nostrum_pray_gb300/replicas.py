"""Replica runs on the GPUs of one node.

The traced frame is not sharded across GPUs: every rank renders its own copy
of the workload (weak scaling; no collective on the data path). The ranks
meet only to time the run: a barrier on each side of the timed region, the
slowest rank's time, and the whole job's throughput as every rank's work over
that time.
"""
from __future__ import annotations


def _dist():
    import torch.distributed as dist
    return dist if dist.is_available() and dist.is_initialized() else None


def world_size() -> int:
    d = _dist()
    return d.get_world_size() if d else 1


def barrier() -> None:
    d = _dist()
    if d and d.get_world_size() > 1:
        d.barrier()


def slowest(seconds: float, device="cpu") -> float:
    """The largest of the ranks' local times (the local time on one rank).
    `device` holds the reduction buffer: a CUDA device for NCCL, "cpu" for
    gloo."""
    d = _dist()
    if not d or d.get_world_size() == 1:
        return float(seconds)
    import torch
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=device)
    d.all_reduce(t, op=d.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank: float, seconds: float, device="cpu") -> float:
    """Units of work of all ranks per second of the slowest rank."""
    return float(units_per_rank) * world_size() / slowest(seconds, device)
