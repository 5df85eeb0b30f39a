"""Batched persistent launch: every DAG of a batch gets exactly the statistics
the single-DAG path computes for it (the accumulation is exact integer ticks, so
the tolerance is zero), on the first run and on graph replays."""
from __future__ import annotations

import numpy as np
import pytest

import mc_dagprop_gb300 as m
from mc_dagprop_gb300 import workloads as W
from mcd_testlib import propagator_from_flat

pytestmark = pytest.mark.gpu


def _prop(flat, gen, nw):
    g = W.to_generator(m, gen)
    return m.MonteCarloPropagator.from_arrays(flat["earliest"], flat["act_idx"], flat["act_duration"],
                                              flat["act_type"], flat["target"], flat["pred_offsets"],
                                              flat["pred_src"], flat["pred_act"], flat["max_delay"], g, n_warps=nw)


@pytest.mark.parametrize("nw", [4, 16, 24])
def test_batch_equals_single_dag_statistics(cuda, nw):
    dags = W.mixed_dags(seed=5, n_dags=10, ev_lo=60, ev_hi=4000, s_lo=40, s_hi=3000, five_types=True)
    props, seed0, ns = [], [], []
    for flat, gen, n, sb in dags:
        props.append(_prop(flat, gen, nw))
        seed0.append(sb)
        ns.append(n)
    # one DAG whose window does not fit in shared memory (global scratch rows)
    wide = W.layered_dag(3, 6, 1500, 1, [1, 2], 10.0)
    props.append(_prop(wide, list(W.GEN_TWO_TYPES), nw))
    seed0.append(10**6)
    ns.append(100)
    assert props[-1].info()["window_in_smem"] is False
    # one DAG with negative times (the general-key kernel variant: a launch of its own)
    neg = dict(dags[0][0], earliest=dags[0][0]["earliest"] - 500.0)
    props.append(_prop(neg, dags[0][1], nw))
    seed0.append(2 * 10**6)
    ns.append(200)
    batch = m.Batch(props, seed0, ns)
    assert batch.items == sum((n + 31) // 32 for n in ns)
    for rep in range(2):
        batch.run()
        for i, p in enumerate(props):
            got = batch.stats(i, hist=True)
            ref = p.run_stats(n=ns[i], seed0=seed0[i], hist=True)
            for k in ("mean", "p50", "p90", "p99", "p_on_time", "hist"):
                assert np.array_equal(got[k], ref[k]), (rep, i, k)


def test_batch_rejects_mixed_warps(cuda):
    flat, gen = W.config0()
    a = _prop(flat, gen, 4)
    b = _prop(flat, gen, 8)
    with pytest.raises(ValueError, match="same n_warps"):
        m.Batch([a, b], [0, 0], [64, 64])


@pytest.mark.parametrize("nw", [2, 8])
def test_batch_many_layouts_per_cta(cuda, nw):
    """Persistent CTAs that run tiles of many DAGs in turn, each with its own
    shared-memory layout (window, staging buffers and tables at different
    offsets): every DAG still gets exactly its single-DAG statistics."""
    dags = W.mixed_dags(seed=2, n_dags=40, ev_lo=100, ev_hi=20000, s_lo=300, s_hi=2500, five_types=True)
    props, seed0, ns = [], [], []
    for flat, gen, n, sb in dags:
        props.append(_prop(flat, gen, nw))
        seed0.append(sb)
        ns.append(n)
    offsets = {p.info()["smem_bytes"] for p in props}
    assert len(offsets) > 10
    batch = m.Batch(props, seed0, ns)
    assert batch.items > 4 * batch.grid  # most CTAs take several items
    for rep in range(2):
        batch.run()
        for i, p in enumerate(props):
            got = batch.stats(i)
            ref = p.run_stats(n=ns[i], seed0=seed0[i])
            for k in ("mean", "p50", "p90", "p99", "p_on_time"):
                assert np.array_equal(got[k], ref[k]), (rep, i, k)


def test_window_place_option_and_tuner(cuda, tmp_path, monkeypatch):
    """The window-place compile option: a DAG whose window fits in shared memory
    compiled with window="global" keeps it in global rows and gives the same
    statistics (exact); a batch of such DAGs equals their single runs; the
    autotuner times every (warps, window) pair of a class and the runner uses its
    choice."""
    from mc_dagprop_gb300 import batching

    monkeypatch.setenv("MCD_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    dags = W.mixed_dags(seed=27, n_dags=6, ev_lo=100, ev_hi=2000, s_lo=64, s_hi=2000, five_types=True)
    props = []
    for flat, gen, n, s0 in dags:
        a = batching.compile_dag(flat, gen, 8, "auto")
        g = batching.compile_dag(flat, gen, 8, "global")
        assert a.info()["window_in_smem"] and not g.info()["window_in_smem"]
        sa, sg = a.run_stats(n=n, seed0=s0), g.run_stats(n=n, seed0=s0)
        for k in ("mean", "p50", "p90", "p99", "p_on_time"):
            np.testing.assert_array_equal(sa[k], sg[k])
        props.append(g)
    b = m.Batch(props, [d[3] for d in dags], [d[2] for d in dags])
    b.run()
    for i, (flat, gen, n, s0) in enumerate(dags):
        alone = props[i].run_stats(n=n, seed0=s0)
        np.testing.assert_array_equal(b.stats(i)["mean"], alone["mean"])
    runner = batching.BatchRunner([(f, g, n, s0) for f, g, n, s0 in dags], use_cache=True)
    for c, secs in runner.tuning.items():
        assert set(secs) == {f"{w}/{p}" for w in batching.CLASS_CANDIDATES[c] for p in ("auto", "global")}
        assert runner.window[c] in ("auto", "global")
    runner.run()
    for i, (flat, gen, n, s0) in enumerate(dags):
        alone = batching.compile_dag(flat, gen, 8).run_stats(n=n, seed0=s0)
        np.testing.assert_array_equal(runner.stats(i)["mean"], alone["mean"])


def test_tuner_choice_holds_on_held_out_dags(cuda):
    """The (warps per CTA, window place) the tuner picks on calibration DAGs is
    within 25 % of the fastest candidate timed on a disjoint held-out set of the
    same width class (every candidate timed on both sets, nothing cached; the
    margin covers run-to-run noise of millisecond batches)."""
    from mc_dagprop_gb300 import batching as B

    dags = W.mixed_dags(seed=41, n_dags=160, ev_lo=200, ev_hi=8000, s_lo=500, s_hi=4000, five_types=True,
                        fast=True)
    by_class = {}
    for flat, gen, n, _ in dags:
        c = B.width_class(B.compile_dag(flat, gen).info()["n_warps"])
        by_class.setdefault(c, []).append((flat, gen, n))
    c, members = max(by_class.items(), key=lambda kv: len(kv[1]))
    assert len(members) >= 40
    cal, held = members[0::2], members[1::2]
    cand = B.CLASS_CANDIDATES[c]
    nw, win, cal_t = B.tune_class([x[0] for x in cal], [x[1] for x in cal], [x[2] for x in cal], candidates=cand,
                                  use_cache=False)
    assert set(cal_t) == {f"{w}/{p}" for w in cand for p in B.WINDOW_CANDIDATES}
    _, _, held_t = B.tune_class([x[0] for x in held], [x[1] for x in held], [x[2] for x in held], candidates=cand,
                                use_cache=False)
    best = min(held_t.values())
    assert held_t[f"{nw}/{win}"] <= 1.25 * best, (c, nw, win, cal_t, held_t)


def test_batch_all_eight_kernel_variants(cuda):
    """A batch whose DAGs need all eight kernel variants (window on chip or in
    global rows, positive times or not, distribution tables in shared or global
    memory): eight persistent launches, each with its own queue head; over two
    runs every DAG gets exactly its single-DAG statistics."""
    from mc_dagprop_gb300 import batching

    rng = np.random.default_rng(8)
    small = W.gen_five_types(rng)
    big = [g if g[1] != 4 else ("empirical_absolute", 4, np.arange(1000) * 0.3, rng.random(1000) + 0.01)
           for g in small]
    props, seed0, ns, variants = [], [], [], set()
    k = 0
    for window in ("auto", "global"):
        for positive in (True, False):
            for gen in (small, big):
                flat = W.layered_dag(60 + k, 8, 24, 2, [1, 2, 3, 4, 5], 1800.0)
                if not positive:
                    flat = dict(flat, earliest=flat["earliest"] - 400.0)
                p = batching.compile_dag(flat, gen, 8, window)
                info = p.info()
                variants.add((info["window_in_smem"], info["positive"], info["tables_in_smem"]))
                props.append(p)
                seed0.append(1000 * k)
                ns.append(96 + 40 * k)
                k += 1
    assert len(variants) == 8
    batch = m.Batch(props, seed0, ns)
    for rep in range(2):
        batch.run()
        for i, p in enumerate(props):
            got = batch.stats(i)
            ref = p.run_stats(n=ns[i], seed0=seed0[i])
            for key in ("mean", "p50", "p90", "p99", "p_on_time"):
                assert np.array_equal(got[key], ref[key]), (rep, i, key)
