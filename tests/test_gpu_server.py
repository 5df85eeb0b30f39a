"""Continuous-batching server: every request's statistics equal those of the
same request run alone (exact: per-request accumulators, integer accumulation),
whatever mix it was batched with; failures are per request; the memory budget
admits work in pieces."""
from __future__ import annotations

import time

import numpy as np
import pytest

import mc_dagprop_gb300 as m
from mc_dagprop_gb300 import batching
from mc_dagprop_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _submit(server, flat, gen, seed0, n):
    return server.submit(flat["earliest"], flat["act_idx"], flat["act_duration"], flat["act_type"], flat["target"],
                         flat["pred_offsets"], flat["pred_src"], flat["pred_act"], flat["max_delay"],
                         W.to_generator(m, gen), seed0, n)


@pytest.mark.parametrize("n_streams,budget,n_warps", [(2, 8 << 30, 8), (3, 64 << 20, 0), (4, 8 << 30, 0)])
def test_served_results_equal_alone(cuda, n_streams, budget, n_warps):
    """n_warps 0: each request with its own warps per CTA, batched by class."""
    reqs = W.mixed_dags(seed=9, n_dags=24, ev_lo=50, ev_hi=3000, s_lo=64, s_hi=4000, five_types=True)
    server = m.Server(memory_budget=budget, n_streams=n_streams, n_warps=n_warps, compile_threads=4)
    tickets = []
    for i, (flat, gen, n, s0) in enumerate(reqs):
        tickets.append(_submit(server, flat, gen, s0, n))
        if i % 5 == 0:
            time.sleep(0.002)  # let some batches start while others arrive
    results = [server.wait(t, timeout_ms=60_000) for t in tickets]
    c = server.counters()
    assert c["completed"] == len(reqs) and c["queued"] == 0
    assert c["batches"] >= 2
    for (flat, gen, n, s0), got in zip(reqs, results):
        assert got is not None
        alone = batching.compile_dag(flat, gen, 8).run_stats(n=n, seed0=s0)
        for k in ("mean", "p50", "p90", "p99", "p_on_time"):
            assert np.array_equal(got[k], alone[k]), k
        assert got["latency_ms"] > 0


def test_server_rejects_bad_request_and_keeps_serving(cuda):
    server = m.Server(memory_budget=1 << 30, n_streams=2, n_warps=8, compile_threads=2)
    flat, gen = W.config0()
    bad = dict(flat, max_delay=-1.0)
    t_bad = _submit(server, bad, gen, 0, 64)
    t_ok = _submit(server, flat, gen, 0, 64)
    with pytest.raises(RuntimeError, match="max_delay"):
        server.wait(t_bad, timeout_ms=30_000)
    assert server.wait(t_ok, timeout_ms=30_000) is not None


def test_resident_dags_reused_and_evicted(cuda):
    """A DAG served before stays compiled on the device: its next requests (other
    seeds, other sample counts) skip the compile and the record upload, and
    their statistics equal a fresh run alone.  When the budget needs room, idle
    resident DAGs are evicted and later requests still succeed."""
    reqs = W.mixed_dags(seed=19, n_dags=6, ev_lo=200, ev_hi=2000, s_lo=256, s_hi=2048, five_types=True)
    server = m.Server(memory_budget=8 << 30, n_streams=2, n_warps=0, compile_threads=2)
    first = [_submit(server, f, g, s0, n) for f, g, n, s0 in reqs]
    for t in first:
        assert server.wait(t, timeout_ms=60_000) is not None
    c0 = server.counters()
    assert c0["resident_dags"] == len(reqs) and c0["resident_hits"] == 0 and c0["resident_bytes"] > 0
    again = [(f, g, n + 37, s0 + 10_000) for f, g, n, s0 in reqs]
    tickets = [_submit(server, f, g, s0, n) for f, g, n, s0 in again]
    got = [server.wait(t, timeout_ms=60_000) for t in tickets]
    c1 = server.counters()
    assert c1["resident_hits"] == len(reqs) and c1["resident_dags"] == len(reqs)
    assert c1["compile_seconds"] == c0["compile_seconds"]  # nothing compiled the second time
    for (f, g, n, s0), r in zip(again, got):
        alone = batching.compile_dag(f, g, 8).run_stats(n=n, seed0=s0)
        for k in ("mean", "p50", "p90", "p99", "p_on_time"):
            assert np.array_equal(r[k], alone[k]), k
    # DAGs of about equal size under a budget that holds about two of them:
    # residents are evicted to make room
    same = W.mixed_dags(seed=23, n_dags=6, ev_lo=800, ev_hi=800, s_lo=256, s_hi=512, five_types=True)
    probe = m.Server(memory_budget=8 << 30, n_streams=1, n_warps=0, compile_threads=1)
    for f, g, n, s0 in same:
        assert probe.wait(_submit(probe, f, g, s0, n), timeout_ms=60_000) is not None
    per_dag = probe.counters()["resident_bytes"] / len(same)
    del probe
    # a request's own block: per event 8 B of ticks, 8 of sum, 1,040 of histogram, 40 of statistics
    rq_block = 1100 * max(len(f["earliest"]) for f, _, _, _ in same) + 4096
    small = m.Server(memory_budget=int(2.5 * per_dag) + rq_block, n_streams=1, n_warps=0, compile_threads=1)
    for f, g, n, s0 in same + same:
        assert small.wait(_submit(small, f, g, s0, n), timeout_ms=60_000) is not None
    cs = small.counters()
    assert cs["evicted"] > 0 and cs["completed"] == 2 * len(same) and cs["resident_dags"] <= 3


def test_tight_budget_with_many_compile_threads_makes_progress(cuda):
    """A budget that holds one DAG and one request block, but not two DAGs and a
    block, with four compile threads and six distinct DAGs in flight at once:
    every request completes.  (A request waiting for memory holds neither budget
    nor a resident DAG; had each thread kept its compiled DAG on the device while
    waiting for its own block, the DAGs alone would fill the budget and no block
    would ever fit.)"""
    same = W.mixed_dags(seed=29, n_dags=6, ev_lo=800, ev_hi=800, s_lo=256, s_hi=512, five_types=True)
    probe = m.Server(memory_budget=8 << 30, n_streams=1, n_warps=0, compile_threads=1)
    for f, g, n, s0 in same:
        assert probe.wait(_submit(probe, f, g, s0, n), timeout_ms=60_000) is not None
    per_dag = probe.counters()["resident_bytes"] / len(same)
    del probe
    rq_block = 1100 * max(len(f["earliest"]) for f, _, _, _ in same) + 4096
    budget = int(per_dag + rq_block + 0.5 * min(per_dag, rq_block))
    tight = m.Server(memory_budget=budget, n_streams=2, n_warps=0, compile_threads=4)
    tickets = [_submit(tight, f, g, s0, n) for f, g, n, s0 in same + same]
    got = [tight.wait(t, timeout_ms=120_000) for t in tickets]
    assert all(r is not None for r in got)
    c = tight.counters()
    assert c["completed"] == 2 * len(same) and c["evicted"] > 0
    for (f, g, n, s0), r in zip(same, got[:len(same)]):
        alone = batching.compile_dag(f, g, 8).run_stats(n=n, seed0=s0)
        assert np.array_equal(r["mean"], alone["mean"])


def test_server_serves_dags_whose_window_is_off_chip(cuda):
    """A DAG whose live events exceed the shared-memory window is served from
    per-CTA realized rows in global memory, in batches of its own class, beside
    DAGs whose window is on chip: every request equals its single run."""
    wide = W.layered_dag(3, 6, 1500, 1, [1, 2], 10.0)
    small, gsmall = W.config0()
    two = list(W.GEN_TWO_TYPES)
    assert not batching.compile_dag(wide, two, 8).info()["window_in_smem"]
    server = m.Server(memory_budget=8 << 30, n_streams=2, n_warps=0, compile_threads=2)
    reqs = [(wide, two, 300, 5), (small, gsmall, 500, 7), (wide, two, 100, 11), (small, gsmall, 64, 13)]
    tickets = [_submit(server, f, g, s0, n) for f, g, n, s0 in reqs]
    for (f, g, n, s0), t in zip(reqs, tickets):
        got = server.wait(t, timeout_ms=60_000)
        assert got is not None
        alone = batching.compile_dag(f, g, 8).run_stats(n=n, seed0=s0)
        for k in ("mean", "p50", "p90", "p99", "p_on_time"):
            assert np.array_equal(got[k], alone[k]), k
    assert server.counters()["completed"] == len(reqs)
