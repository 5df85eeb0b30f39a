"""Replica parallelism host logic with two gloo processes on the CPU: disjoint
seed ranges, the job time as the maximum over ranks, whole-job throughput."""
from __future__ import annotations

import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from mc_dagprop_gb300 import replicas


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        seeds = replicas.seed_range(rank, world, 1000, base=10)
        t = replicas.job_seconds(1.0 + rank)  # rank 1 is the slow one
        out.put((rank, int(seeds[0]), int(seeds[-1]), t, replicas.job_throughput(1000 * 5, world, t)))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, a0, b0, t0, v0), (r1, a1, b1, t1, v1) = res
    assert (a0, b0, a1, b1) == (10, 1009, 1010, 2009)  # disjoint, contiguous
    assert t0 == t1 == 2.0  # the slowest rank's time on every rank
    assert v0 == v1 == pytest.approx(2 * 5000 / 2.0)


def test_local_helpers():
    assert np.array_equal(replicas.seed_range(0, 1, 3), [0, 1, 2])
    assert replicas.job_seconds(1.5) == 1.5  # no process group: the local time
    with pytest.raises(ValueError):
        replicas.seed_range(2, 2, 10)
