"""The two GPU engines against each other, as the reference's parity suite
(test/test_parity_suite.py) checks its Monte Carlo propagator against its analytic
one: integer-valued empirical delays on a zero base, TRUNCATE flow rules and event
bounds [earliest, earliest + max_delay], where the analytic PMF of every event is
the exact law of the Monte Carlo realized time.  200,000 samples per case (the
reference takes 8,000-14,000), so the tolerances are tighter: probabilities within
0.006 and means within 0.05 (about 4.5 standard errors)."""
from __future__ import annotations

import numpy as np
import pytest

import mc_dagprop_gb300 as m
from mc_dagprop_gb300 import analytic as AN

pytestmark = pytest.mark.gpu

N = 200_000


def _engines(earliest, arcs, max_delay):
    """arcs: [(src, dst, values, probs)]; one activity type per arc.  Returns (analytic
    results, Monte Carlo realized (N, E))."""
    E = len(earliest)
    events = tuple(m.Event(f"E{i}", m.EventTimestamp(float(e), float(e) + max_delay, float(e)))
                   for i, e in enumerate(earliest))
    by_target: dict[int, list] = {}
    an_acts, mc_acts = {}, {}
    gen = m.GenericDelayGenerator()
    for k, (s, d, v, p) in enumerate(arcs):
        an_acts[(s, d)] = (k, AN.AnalyticActivity(k, AN.DiscretePMF(np.asarray(v, float), np.asarray(p, float),
                                                                     step=1)))
        mc_acts[(s, d)] = m.Activity(idx=k, minimal_duration=0.0, activity_type=k + 1)
        gen.add_empirical_absolute(k + 1, [float(x) for x in v], [float(x) for x in p])
        by_target.setdefault(d, []).append((s, k))
    prec = sorted(by_target.items())
    ctx = AN.AnalyticContext(events=events, activities=an_acts,
                             precedence_list=tuple((t, tuple(pl)) for t, pl in prec), step=1,
                             underflow_rule=AN.UnderflowRule.TRUNCATE, overflow_rule=AN.OverflowRule.TRUNCATE,
                             max_delay=float(max_delay))
    analytic = AN.create_analytic_propagator(ctx).run()
    dag = m.DagContext(events=list(events), activities=mc_acts, precedence_list=[(t, list(pl)) for t, pl in prec],
                       max_delay=float(max_delay))
    real, _, _ = m.MonteCarloPropagator(dag, gen).run_many_arrays(np.arange(N, dtype=np.int64), durations=False)
    assert real.shape == (N, E)
    return analytic, real


def _check(analytic, real, events, p_atol=0.006, mean_atol=0.05):
    for e in events:
        pmf = analytic[e].pmf
        vals = np.asarray(pmf.values)
        col = real[:, e]
        assert np.all(col == np.round(col)), "integer delays give integer times"
        assert set(np.unique(col)) <= set(vals.tolist()), (e, np.unique(col), vals)
        freq = np.array([(col == v).mean() for v in vals])
        np.testing.assert_allclose(freq, pmf.probabilities, rtol=0, atol=p_atol, err_msg=f"event {e}")
        assert abs(col.mean() - float(np.dot(vals, pmf.probabilities))) <= mean_atol, e
        assert float(analytic[e].underflow) == 0.0 and float(analytic[e].overflow) == 0.0


def test_chain_parity(cuda):
    a = ([0, 1, 2, 3], [0.1, 0.3, 0.4, 0.2])
    b = ([0, 1, 2, 3], [0.15, 0.35, 0.3, 0.2])
    an, real = _engines([0, 0, 0], [(0, 1, *a), (1, 2, *b)], 120.0)
    _check(an, real, [1, 2], mean_atol=0.02)


def test_branching_parity(cuda):
    left = ([0, 1, 2, 3, 4], [0.15, 0.2, 0.25, 0.25, 0.15])
    right = ([0, 1, 2, 3], [0.2, 0.35, 0.3, 0.15])
    an, real = _engines([0, 0, 0, 0], [(0, 1, *left), (0, 2, *right), (1, 3, *right), (2, 3, *left)], 200.0)
    _check(an, real, [1, 2, 3], mean_atol=0.02)


def test_long_chain_parity(cuda):
    step = ([0, 1, 2], [0.2, 0.5, 0.3])
    an, real = _engines([0] * 101, [(i, i + 1, *step) for i in range(100)], 1000.0)
    _check(an, real, [1, 10, 50, 100])


def test_max_delay_truncation_parity(cuda):
    an, real = _engines([10, 12], [(0, 1, [3, 4, 5, 6], [0.25, 0.25, 0.3, 0.2])], 4.0)
    assert real[:, 1].max() <= 12 + 4.0
    _check(an, real, [1], mean_atol=0.02)


def test_merge_tree_parity(cuda):
    """A merge tree (the analytic engine's maximum assumes independent arrivals, so the
    two laws agree exactly when no two predecessors share an ancestor): 27 sources
    with random earliest times joined in twos and threes down to one sink; delays on
    contiguous grids of 0..6 with some zero weights; max_delay 12 truncates."""
    rng = np.random.default_rng(41)
    earliest = rng.integers(0, 4, 27).tolist()
    level = list(range(27))
    arcs = []
    while len(level) > 1:
        nxt = []
        i = 0
        while i < len(level):
            k = 3 if len(level) - i in (3, 5) or (len(level) - i > 3 and rng.random() < 0.5) else 2
            k = min(k, len(level) - i)
            t = len(earliest)
            earliest.append(int(max(earliest[s] for s in level[i:i + k]) + rng.integers(0, 3)))
            for s in level[i:i + k]:
                lo = int(rng.integers(0, 3))
                n = int(rng.integers(2, 5))
                w = rng.random(n) + 0.2
                w[rng.random(n) < 0.25] = 0.0  # gaps in the support
                if w.sum() == 0.0:
                    w[0] = 1.0
                arcs.append((s, t, list(range(lo, lo + n)), (w / w.sum()).tolist()))
            nxt.append(t)
            i += k
        level = nxt
    an, real = _engines(earliest, arcs, 12.0)
    _check(an, real, list(range(27, len(earliest))))
