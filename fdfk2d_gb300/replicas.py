"""Independent replicas on N GPUs of one node (one process per GPU, launched by torchrun).

The solver does not shard: each rank runs its own solves, which exchange no data.  The only
cross-rank steps are a barrier on each side of a timed region and the maximum of the ranks'
times, from which the whole job's rate is formed (units of all ranks over the slowest rank's
time).  Works with any torch.distributed backend (NCCL on GPUs, gloo on the host).
"""
from __future__ import annotations

import torch
import torch.distributed as dist


def world_size() -> int:
    """Ranks of the initialised process group (1 without one)."""
    return dist.get_world_size() if dist.is_available() and dist.is_initialized() else 1


def barrier() -> None:
    """Wait for every rank (nothing without a process group)."""
    if world_size() > 1:
        dist.barrier()


def max_over_ranks(x: float, device: torch.device | None = None) -> float:
    """The largest x of all ranks (x itself without a process group).  device: where the
    reduction buffer lives (the rank's GPU for NCCL, the host for gloo)."""
    if world_size() == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank: float, seconds: float) -> float:
    """Units per second of the whole job: every rank's units over the slowest rank's time
    (seconds = max_over_ranks of the ranks' times)."""
    if seconds <= 0:
        raise ValueError("time must be positive")
    return units_per_rank * world_size() / seconds
