"""Replica parallelism across GPUs (one process per GPU).

Samples are independent, so N GPUs run N replicas of the compiled DAG on
disjoint seed ranges with no exchange on the data path; the job's time is the
slowest rank's and its throughput is all ranks' units over that time.  These
helpers hold that host logic (used by ``bench.py`` under torchrun; tested with
two ``gloo`` processes on the CPU).
"""
from __future__ import annotations

import numpy as np


def seed_range(rank: int, world: int, per_rank: int, base: int = 0) -> np.ndarray:
    """The seeds of ``rank``: ``per_rank`` consecutive seeds, disjoint across ranks."""
    if not (0 <= rank < world) or per_rank < 0:
        raise ValueError("need 0 <= rank < world and per_rank >= 0")
    start = base + rank * per_rank
    return np.arange(start, start + per_rank, dtype=np.int64)


def job_seconds(local_seconds: float, group=None) -> float:
    """The job's elapsed time: the maximum over ranks (all-reduce MAX when a process
    group is initialised, else the local time)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()):
        return float(local_seconds)
    backend = dist.get_backend(group)
    dev = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else torch.device("cpu")
    t = torch.tensor([float(local_seconds)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())


def job_throughput(units_per_rank: float, world: int, seconds: float) -> float:
    """Whole-job throughput: the units all ranks processed over the job's time."""
    return float(units_per_rank) * world / seconds
