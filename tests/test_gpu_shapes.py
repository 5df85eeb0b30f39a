"""Edge shapes of the DAG and of the sample batch, bit-exact against the oracle:
a lone event, events without any precedence, a star whose one target has more
predecessor records than a staging buffer holds, a level far wider than a
CTA's warps with a window too large for shared memory, ragged sample counts
(1, 31, 33, 65) and a gap-filled activity array, each through the given-durations
path (oracle durations in, realized and cause_event compared bit for bit) and the
sampled path (its durations propagated by the oracle)."""
from __future__ import annotations

import numpy as np
import pytest

import mc_dagprop_gb300 as m
import oracle
from mc_dagprop_gb300 import workloads as W
from mcd_testlib import propagator_from_flat

pytestmark = pytest.mark.gpu

GEN = [("constant", 1, 0.5), ("exponential", 2, 0.2, 4.0), ("empirical_absolute", 3, [0.0, 5.0, 9.0],
                                                              [0.2, 0.5, 0.3])]


def _bits(a):
    return np.asarray(a, np.float64).view(np.int64)


def _flat(earliest, links, prec, max_delay):
    """links: list of (act_idx, duration, type); prec: list of (target, [(src, act_idx), ...])."""
    t, off, src, act = [], [0], [], []
    for tgt, plist in prec:
        t.append(tgt)
        for s, a in plist:
            src.append(s)
            act.append(a)
        off.append(len(src))
    return {"earliest": np.asarray(earliest, np.float64),
            "act_idx": np.asarray([x[0] for x in links], np.int32),
            "act_duration": np.asarray([x[1] for x in links], np.float64),
            "act_type": np.asarray([x[2] for x in links], np.int32),
            "target": np.asarray(t, np.int32), "pred_offsets": np.asarray(off, np.int64),
            "pred_src": np.asarray(src, np.int32), "pred_act": np.asarray(act, np.int32),
            "max_delay": float(max_delay)}


def _star(n_src):
    """n_src sources, one target reached from each (2,000 predecessor records of 32 B
    exceed a 40 KB staging buffer)."""
    rng = np.random.default_rng(n_src)
    earliest = list(rng.uniform(0, 50, n_src).round(1)) + [10.0]
    links = [(i, float(rng.uniform(1, 30)), 1 + i % 3) for i in range(n_src)]
    return _flat(earliest, links, [(n_src, [(i, i) for i in range(n_src)])], 500.0)


def _wide(width):
    """One level of `width` sources, a second level where each event reads 3 of them,
    and a join: the window (all sources live until the second level) exceeds shared
    memory for width 1,000 and the level exceeds any CTA's warps."""
    rng = np.random.default_rng(width)
    earliest = list(rng.uniform(0, 20, width)) + list(rng.uniform(20, 40, width)) + [60.0]
    links, prec, a = [], [], 0
    for j in range(width):
        srcs = rng.choice(width, 3, replace=False)
        plist = []
        for s in srcs:
            links.append((a, float(rng.uniform(1, 20)), 1 + a % 3))
            plist.append((int(s), a))
            a += 1
        prec.append((width + j, plist))
    join = []
    for j in range(0, width, 7):
        links.append((a, 1.0, 2))
        join.append((width + j, a))
        a += 1
    prec.append((2 * width, join))
    return _flat(earliest, links, prec, 100.0)


def _gaps():
    """Activity indices with gaps (the dense link array holds zero-duration gaps) and a
    link no precedence entry uses."""
    links = [(0, 3.0, 1), (4, 2.0, 2), (9, 7.0, 3), (12, 1.0, 2)]
    return _flat([0.0, 1.0, 2.0, 3.0], links, [(1, [(0, 0)]), (2, [(1, 4)]), (3, [(0, 9), (2, 4)])], 50.0)


SHAPES = {
    "lone_event": lambda: _flat([4.5], [], [], 10.0),
    "no_precedence": lambda: _flat([1.0, 2.0, 3.0], [(0, 5.0, 1), (1, 2.0, 2)], [], 10.0),
    "star_2000": lambda: _star(2000),
    "wide_1000": lambda: _wide(1000),
    "wide_40": lambda: _wide(40),
    "gaps": _gaps,
}


@pytest.mark.parametrize("shape", list(SHAPES))
@pytest.mark.parametrize("n", [1, 31, 33, 65])
def test_shapes_given_and_sampled_bitexact(cuda, shape, n):
    flat = SHAPES[shape]()
    sim = oracle.OracleSim(flat, GEN)
    prop = propagator_from_flat(m, flat, GEN)
    E, L = sim.node_count(), sim.activity_count()
    assert (prop.node_count(), prop.activity_count()) == (E, L)
    rng = np.random.default_rng(n)
    seeds = rng.integers(-2**31, 2**31 - 1, n)
    _, dur_o, _ = sim.run_many(seeds)
    dur_o = np.asarray(dur_o, np.float64).reshape(n, L)
    real_o, cause_o = sim.propagate_given(dur_o)
    real, cause = prop.propagate(dur_o)
    assert np.array_equal(_bits(real), _bits(real_o))
    assert np.array_equal(cause, cause_o)
    # sampled: the GPU's own durations, propagated by the oracle
    r, d, c = prop.run_many_arrays(seeds)
    assert r.shape == (n, E) and d.shape == (n, L) and c.shape == (n, E)
    ro, co = sim.propagate_given(d)
    assert np.array_equal(_bits(r), _bits(ro))
    assert np.array_equal(c, co)
    if shape == "gaps":  # gap links have duration 0 (_core.cpp:287-288 dense array)
        assert (d[:, [1, 2, 3, 5, 6, 7, 8, 10, 11]] == 0.0).all()


def test_wide_level_uses_global_window(cuda):
    prop = propagator_from_flat(m, _wide(1000), GEN)
    info = prop.info()
    assert info["window_in_smem"] is False
    assert propagator_from_flat(m, _wide(40), GEN).info()["window_in_smem"] is True


def test_zero_samples_and_empty_seed_lists(cuda):
    flat, gen = W.config0()
    prop = propagator_from_flat(m, flat, gen)
    r, d, c = prop.run_many_arrays(np.zeros(0, np.int64))
    assert r.shape == (0, prop.node_count()) and d.shape == (0, prop.activity_count()) and c.shape == r.shape
    assert prop.run_many([]) == []


def test_tables_in_global_memory(cuda):
    """Distribution tables too large for shared memory (a 1,000-bin empirical table)
    run the kernels that read them from global memory: bit-exact propagation of the
    sampled durations, durations that are the reference's base + value, and draw
    frequencies that follow the weights."""
    rng = np.random.default_rng(77)
    values = np.arange(1000, dtype=np.float64) * 0.5
    weights = rng.random(1000) + 0.05
    gen = [("empirical_absolute", 1, values, weights), ("exponential", 2, 0.2, 4.0)]
    flat = W.layered_dag(3, 20, 30, 2, [1, 2], 100.0)
    prop = propagator_from_flat(m, flat, gen)
    assert prop.info()["tables_in_smem"] is False
    sim = oracle.OracleSim(flat, gen)
    seeds = np.arange(20_000, dtype=np.int64)
    r, d, c = prop.run_many_arrays(seeds)
    ro, co = sim.propagate_given(d)
    assert np.array_equal(_bits(r), _bits(ro))
    assert np.array_equal(c, co)
    emp = np.asarray(flat["act_type"]) == 1
    idx = np.asarray(flat["act_idx"])[emp]
    base = np.asarray(flat["act_duration"])[emp]
    delay = d[:, idx] - base[None, :]
    k = np.rint(delay / 0.5).astype(np.int64)
    assert np.all((k >= 0) & (k < 1000))
    assert np.array_equal(_bits(d[:, idx]), _bits(base[None, :] + values[k]))  # base + v, as the reference adds
    freq = np.bincount(k.ravel(), minlength=1000) / k.size
    p = weights / weights.sum()
    assert np.max(np.abs(freq - p)) < 8 * np.sqrt(p.max() / k.size)
