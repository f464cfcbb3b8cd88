"""Independent replicas across ranks (the multi-GPU mode of this path: replicas only).

Every rank advances its own copy of the workload; nothing of the data path crosses ranks.  The timed region is
bracketed by a barrier on both sides, the slowest rank's time is the job's time, and the whole-job throughput
is the units all ranks processed divided by that time (weak scaling: the per-rank work is fixed).  The process
group is torch.distributed (NCCL on GPUs, gloo on CPU); these helpers only reduce host scalars.
"""
from __future__ import annotations

import os


def env():
    """(world size, rank, local rank) from the torchrun environment (1, 0, 0 without it)."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def barrier(pg) -> None:
    if pg is not None:
        pg.barrier()


def max_over_ranks(pg, value: float, device=None) -> float:
    """The largest `value` over the ranks (the job's time is its slowest rank's)."""
    if pg is None:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(pg, value: float, device=None) -> float:
    if pg is None:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    pg.all_reduce(t, op=pg.ReduceOp.SUM)
    return float(t.item())


def job_throughput(pg, units: float, seconds: float, device=None) -> float:
    """Units all ranks processed divided by the slowest rank's time."""
    return sum_over_ranks(pg, units, device) / max_over_ranks(pg, seconds, device)
