"""GPU delay sampler: draw-for-draw against the numpy model, in distribution
against the reference's laws, and propagated statistics against the oracle
(which reproduces the reference's run_many bit for bit).

Tolerances stated here:
  * model parity: empirical draws exact; exponential within 2e-6 relative (the
    kernel's FP32 logarithm is the MUFU approximation);
  * distribution tests: Kolmogorov-Smirnov / chi-square at alpha = 0.01 on fixed seeds;
  * propagated statistics vs the oracle on the same DAG: per-event two-sample KS at
    alpha = 0.01 (at most 3% of events may reject, 1% expected by chance) and
    per-event means within 3 standard errors (at most 1% outside, 0.27% expected).
"""
from __future__ import annotations

import math
import os

import numpy as np
import pytest
from scipy import stats

import mc_dagprop_gb300 as m
import oracle
import philox_model as PM
from mc_dagprop_gb300 import workloads as W
from mcd_testlib import flat_from_lists, propagator_from_flat

pytestmark = pytest.mark.gpu


def _one_link(base=100.0):
    """Two events, one link of the given base duration, no clamping."""
    return flat_from_lists([0.0, 0.0], {(0, 1): (0, base, 1)}, [(1, [(0, 0)])], 1e12)


def _draw(gen, seeds, base=100.0, link=0):
    prop = propagator_from_flat(m, _one_link(base), gen)
    _, dur, _ = prop.run_many_arrays(np.asarray(seeds, np.int64))
    return dur[:, link]


SEEDS = np.concatenate([np.arange(-2000, 2000), np.random.default_rng(5).integers(-2**62, 2**62, 4000)])


def test_constant_exact(cuda):
    d = _draw([("constant", 1, 1.5)], SEEDS[:100], base=37.3)
    assert (d == 37.3 + 37.3 * 1.5).all()


@pytest.mark.parametrize("kind", ["empirical_absolute", "empirical_relative"])
def test_empirical_matches_model_exactly(cuda, kind):
    values = np.array([0.0, 3.5, 7.25, 100.0, 0.125])
    weights = np.array([0.1, 0.0, 2.0, 0.7, 1.2])
    d = _draw([(kind, 1, values, weights)], SEEDS, base=40.0)
    expect = PM.empirical_durations(SEEDS, 0, 40.0, values, weights, kind == "empirical_relative")
    assert np.array_equal(d, expect)


def test_exponential_matches_model(cuda):
    for lam, ms in ((0.1, math.inf), (2.0, 0.5), (1.0, 3.0)):
        d = _draw([("exponential", 1, lam, ms)], SEEDS, base=10.0)
        ref = PM.exponential_durations(SEEDS, 0, 10.0, lam, ms)
        np.testing.assert_allclose(d, ref, rtol=2e-6)
        assert (d >= 10.0).all() and (d <= 10.0 * (1 + ms)).all()


def test_exponential_distribution(cuda):
    n = 200_000
    seeds = np.arange(n) + 123_456
    for lam, ms in ((0.1, math.inf), (2.0, 0.5)):
        x = (_draw([("exponential", 1, lam, ms)], seeds, base=1.0) - 1.0)
        if math.isinf(ms):
            p = stats.kstest(x, stats.expon(scale=lam).cdf).pvalue
        else:
            p = stats.kstest(x, stats.truncexpon(b=ms / lam, scale=lam).cdf).pvalue
        assert p > 0.01, (lam, ms, p)


@pytest.mark.parametrize("shape,scale,ms", [(2.0, 0.05, math.inf), (0.4, 1.5, math.inf), (2.0, 1.0, 0.5),
                                            (9.0, 0.3, 3.0)])
def test_gamma_distribution(cuda, shape, scale, ms):
    n = 200_000
    x = _draw([("gamma", 1, shape, scale, ms)], np.arange(n) + 77, base=1.0) - 1.0
    assert (x >= 0.0).all() and (x <= ms).all()
    g = stats.gamma(shape, scale=scale)
    if math.isinf(ms):
        cdf = g.cdf
    else:
        cut = g.cdf(ms)
        cdf = lambda t: np.minimum(g.cdf(t) / cut, 1.0)  # noqa: E731
    assert stats.kstest(x, cdf).pvalue > 0.01


def _shared_block_dag():
    """Event 10 reads ten links of mixed kinds from events 0-9; event 11 reads two of
    the same links again (later references recompute the same words)."""
    kinds = [2, 4, 5, 2, 1, 3, 4, 2, 6, 5]  # types: 1 constant, 2 exp, 3 gamma, 4 emp abs, 5 emp rel, 6 big table
    links = {(i, 10): (i, 10.0 + i, kinds[i]) for i in range(10)}
    links[(10, 11)] = (10, 1.0, 1)
    prec = [(10, [(i, i) for i in range(10)]), (11, [(10, 10), (3, 3), (2, 2)])]
    return flat_from_lists([0.0] * 12, links, prec, 1e12)


BIG = (np.arange(5000) * 0.01, np.random.default_rng(11).random(5000) + 0.01)
SHARED_GEN = [("constant", 1, 0.5), ("exponential", 2, 0.3, math.inf), ("gamma", 3, 2.0, 0.05, math.inf),
              ("empirical_absolute", 4, np.array([0.0, 3.5, 7.25, 100.0]), np.array([1.0, 0.5, 2.0, 0.3])),
              ("empirical_relative", 5, np.array([0.0, 0.25, 0.5]), np.array([0.2, 0.3, 0.5])),
              ("empirical_absolute", 6, BIG[0], BIG[1])]


def test_shared_philox_blocks_match_model(cuda):
    """Links first referenced by one event share Philox blocks of four words:
    one-word links (exponential, small tables) take a word, shape-2 gamma two; a
    5,000-bin table owns its block.  Every link's draws match the model at its
    (block, word)."""
    flat = _shared_block_dag()
    prop = propagator_from_flat(m, flat, SHARED_GEN)
    block, word = prop.link_streams()
    one_word = [0, 1, 2, 3, 6, 7, 9]  # links of types 2, 4, 5 in precedence order
    assert list(block[one_word]) == [0, 0, 0, 0, 5, 5, 9] and list(word[one_word]) == [0, 1, 2, 3, 2, 3, 0]
    assert block[4] == -1 and block[10] == -1  # constant
    assert (block[5], word[5]) == (5, 0)  # shape-2 gamma: words 0 and 1 of block 5
    assert (block[8], word[8]) == (8, -1)  # big table
    _, dur, _ = prop.run_many_arrays(SEEDS)
    gen = {g[1]: g for g in SHARED_GEN}
    kinds = flat["act_type"]
    for l in range(10):
        g, base = gen[int(kinds[l])], float(flat["act_duration"][l])
        if g[0] == "exponential":
            ref = PM.exponential_durations(SEEDS, l, base, g[2], g[3], block=block[l], word=word[l])
            np.testing.assert_allclose(dur[:, l], ref, rtol=2e-6)
        elif g[0].startswith("empirical"):
            ref = PM.empirical_durations(SEEDS, l, base, g[2], g[3], g[0] == "empirical_relative",
                                         block=block[l], word=max(0, word[l]))
            assert np.array_equal(dur[:, l], ref), l


def test_shared_block_words_independent(cuda):
    """Links sharing a block are independent draws: pairwise correlation of their
    uniforms and a chi-square of the joint bins of two small tables."""
    flat = _shared_block_dag()
    prop = propagator_from_flat(m, flat, SHARED_GEN)
    n = 200_000
    _, dur, _ = prop.run_many_arrays(np.arange(n, dtype=np.int64) + 5)
    x = dur[:, [0, 3, 7]] - flat["act_duration"][[0, 3, 7]]  # three exponentials of block 0 / 6
    c = np.corrcoef(x.T)
    assert np.abs(c[np.triu_indices(3, 1)]).max() < 0.01
    a = np.searchsorted([0.0, 3.5, 7.25, 100.0], dur[:, 1] - 11.0)      # empirical abs, word 1 of block 0
    b = np.searchsorted([0.0, 0.25, 0.5], (dur[:, 2] - 12.0) / 12.0)    # empirical rel, word 2 of block 0
    table = np.zeros((4, 3))
    np.add.at(table, (a, b), 1)
    assert stats.chi2_contingency(table).pvalue > 0.01


def test_empirical_frequencies(cuda):
    n = 200_000
    values = np.linspace(0.0, 300.0, 16)
    w = np.random.default_rng(3).dirichlet(np.ones(16))
    x = _draw([("empirical_absolute", 1, values, w)], np.arange(n), base=0.0)
    idx = np.searchsorted(values, x)
    counts = np.bincount(idx, minlength=16)
    assert stats.chisquare(counts, w * n).pvalue > 0.01


def test_gamma_rejection_cap_reports_error(cuda):
    """A truncation that accepts (almost) nothing ends in a RuntimeError, not a hang."""
    prop = propagator_from_flat(m, _one_link(1.0), [("gamma", 1, 60.0, 1.0, 1.0)])
    with pytest.raises(RuntimeError, match="gamma"):
        prop.run_many_arrays(np.arange(64))
    # the handle stays usable afterwards
    prop2 = propagator_from_flat(m, _one_link(1.0), [("gamma", 1, 2.0, 1.0)])
    assert np.isfinite(prop2.run_many_arrays(np.arange(64))[1]).all()


def _per_event_agreement(real_a, real_b, earliest):
    ks_fail = 0
    mean_fail = 0
    E = real_a.shape[1]
    for e in range(E):
        a, b = real_a[:, e], real_b[:, e]
        if np.all(a == a[0]) and np.all(b == b[0]):
            assert a[0] == b[0]
            continue
        if stats.ks_2samp(a, b).pvalue < 0.01:
            ks_fail += 1
        se = math.sqrt(a.var() / len(a) + b.var() / len(b))
        if abs(a.mean() - b.mean()) > 3.0 * se + 1e-9:
            mean_fail += 1
    return ks_fail / E, mean_fail / E


@pytest.mark.parametrize("cfg", ["config0", "five_types"])
def test_propagated_statistics_match_oracle(cuda, cfg):
    """Per-event realized distributions of the GPU sampler vs the reference's
    algorithm (the oracle) on the same DAG, independent seeds."""
    if cfg == "config0":
        flat, gen = W.config0()
    else:
        flat, gen = W.config1(seed=21, n_layers=25, width=40)
    n = 100_000
    prop = propagator_from_flat(m, flat, gen)
    real_g, _, _ = prop.run_many_arrays(np.arange(n, dtype=np.int64) + 10**9, durations=False)
    real_o, _, _ = oracle.OracleSim(flat, gen).run_many(np.arange(n), threads=os.cpu_count() or 1,
                                                          want=("realized",))
    ks_rate, mean_rate = _per_event_agreement(real_g, real_o, flat["earliest"])
    assert ks_rate <= 0.03, ks_rate
    assert mean_rate <= 0.01, mean_rate


def test_reference_suite_bounds_and_known_answers(cuda):
    """test/test_monte_carlo_extra.py:27-57 and test/test_simulator.py:37-137 on the GPU."""
    ev = [m.Event("0", m.EventTimestamp(0.0, 100.0, 0.0)), m.Event("1", m.EventTimestamp(0.0, 100.0, 0.0)),
          m.Event("2", m.EventTimestamp(0.0, 100.0, 0.0))]
    acts = {(0, 1): m.Activity(idx=0, minimal_duration=1.0, activity_type=1),
            (1, 2): m.Activity(idx=1, minimal_duration=2.0, activity_type=1)}
    ctx = m.DagContext(events=ev, activities=acts, precedence_list=[(1, [(0, 0)]), (2, [(1, 1)])], max_delay=1e6)
    g = m.GenericDelayGenerator()
    g.add_constant(activity_type=1, factor=1.0)
    r = m.Simulator(ctx, g).run(seed=42)
    np.testing.assert_allclose(r.durations, [2.0, 4.0])
    np.testing.assert_allclose(r.realized, [0.0, 2.0, 6.0])
    for add in (lambda gg: gg.add_exponential(activity_type=1, lambda_=2.0, max_scale=0.5),
                lambda gg: gg.add_gamma(activity_type=1, shape=2.0, scale=1.0, max_scale=0.5)):
        gg = m.GenericDelayGenerator()
        add(gg)
        sim = m.Simulator(ctx, gg)
        for res in sim.run_many(list(range(200))):
            assert 1.0 <= res.durations[0] <= 1.5 and 2.0 <= res.durations[1] <= 3.0
            assert res.realized[2] >= res.realized[1]
        batch = sim.run_many(list(range(5)))
        solo = [sim.run(s) for s in range(5)]
        for b, s in zip(batch, solo):
            np.testing.assert_array_equal(b.realized, s.realized)
            np.testing.assert_array_equal(b.durations, s.durations)
            np.testing.assert_array_equal(b.cause_event, s.cause_event)
    # six-event DAG with an unmapped type and reversed precedence (test_simulator.py:64-137)
    events = [m.Event(str(i), m.EventTimestamp(t, 100.0, 0.0)) for i, t in enumerate([0.0, 5.0, 10.0, 22.0, 20.0, 100.0])]
    links = {(0, 1): m.Activity(0, 3.0, 1), (1, 2): m.Activity(1, 5.0, 1), (1, 3): m.Activity(2, 5.0, 1),
             (2, 4): m.Activity(3, 15.0, 2), (3, 4): m.Activity(4, 10.0, 3)}
    prec = [(1, [(0, 0)]), (2, [(1, 1)]), (3, [(1, 2)]), (4, [(2, 3), (3, 4)])]
    g = m.GenericDelayGenerator()
    g.add_constant(activity_type=1, factor=1.0)
    g.add_constant(activity_type=3, factor=3.0)
    for pl in (prec, list(reversed(prec))):
        res = m.Simulator(m.DagContext(events, links, pl, 1e6), g).run_many(tuple(range(5)))[3]
        assert list(res.durations) == [6.0, 10.0, 10.0, 15.0, 40.0]
        assert list(res.realized) == [0.0, 6.0, 16.0, 22.0, 62.0, 100.0]
        assert list(res.cause_event) == [-1, 0, 1, -1, 3, -1]
    # empirical absolute: every realized value is one the table allows
    g = m.GenericDelayGenerator()
    g.add_empirical_absolute(activity_type=1, values=[10, 20, 40, 50], weights=[0.1, 0.2, 0.3, 0.4])
    sim = m.Simulator(m.DagContext(events, links, prec, 1e6), g)
    for res in sim.run_many(list(range(50))):
        assert res.realized[3] in (5.0 + 3.0 + 10 + 5.0 + d for d in (10, 20, 40, 50)) or res.realized[3] >= 22.0
        assert res.realized[5] == 100.0


def test_unstaged_stage_tables_and_draws(cuda):
    """An event with 3,000 predecessors: its stage's records exceed a staging buffer,
    so they (and the empirical links' duration tables) are read from global memory.
    Its draws still match the model at each link's (block, word), and the run is a
    propagation of its own durations."""
    from mcd_testlib import describe

    n = 3000
    kinds = [2, 4, 5, 3, 1]  # exp, emp abs, emp rel, gamma, constant
    links = {(i, n): (i, 20.0 + i % 7, kinds[i % 5]) for i in range(n)}
    flat = flat_from_lists([0.0] * (n + 1), links, [(n, [(i, i) for i in range(n)])], 1e12)
    gen = SHARED_GEN[:5]
    rc, info, _ = describe(flat, gen)
    assert rc == 0 and info.n_stages >= 2
    prop = propagator_from_flat(m, flat, gen)
    seeds = np.arange(64, dtype=np.int64) * 31 + 7
    real, dur, cause = prop.run_many_arrays(seeds)
    r2, c2 = prop.propagate(dur)
    assert np.array_equal(real.view(np.int64), r2.view(np.int64)) and np.array_equal(cause, c2)
    block, word = prop.link_streams()
    gmap = {g[1]: g for g in gen}
    for l in range(0, n, 37):
        g, base = gmap[kinds[l % 5]], float(flat["act_duration"][l])
        if g[0].startswith("empirical"):
            ref = PM.empirical_durations(seeds, l, base, g[2], g[3], g[0] == "empirical_relative",
                                         block=block[l], word=max(0, word[l]))
            assert np.array_equal(dur[:, l], ref), l
        elif g[0] == "exponential":
            ref = PM.exponential_durations(seeds, l, base, g[2], g[3], block=block[l], word=word[l])
            np.testing.assert_allclose(dur[:, l], ref, rtol=2e-6)


def _erlang_durations(seeds, base, shape, scale, block, word):
    """Shape-k Erlang gamma without truncation, the kernel's float32 formula:
    X = -scale * log(U_w * ... * U_{w+k-1}) from words w.. of the block,
    duration base * (1 + X)."""
    r = PM.words(seeds, block)
    prod = PM.u01_open0(r[word]).astype(np.float32)
    for j in range(1, shape):
        prod = (prod * PM.u01_open0(r[word + j])).astype(np.float32)
    X = np.maximum(-np.float32(scale) * np.log(prod), np.float32(0.0)).astype(np.float32)
    return np.array([PM.scale_by(base, np.float32(1.0) + x) for x in X])


def test_event_pairs_share_blocks_draw_for_draw(cuda):
    """Events of one level run in pairs whose draws share Philox blocks: on a
    layered five-kind DAG every sampled link's durations match the model at the
    (block, word) the compiled DAG reports, blocks are shared between links of
    two different events, and the draws are the same under other warps per CTA
    and with the window in global rows."""
    from mc_dagprop_gb300 import batching

    flat = W.layered_dag(41, 30, 40, 3, [1, 2, 3, 4, 5], 3600.0)
    gen = SHARED_GEN[:5]
    prop = propagator_from_flat(m, flat, gen)
    info = prop.info()
    assert info["n_event_pairs"] > 0.2 * info["n_events"]
    block, word = prop.link_streams()
    L = len(flat["act_duration"])
    event_of = np.full(L, -1, np.int64)
    off, tgt, act = flat["pred_offsets"], flat["target"], flat["pred_act"]
    for k in range(len(tgt)):
        event_of[act[off[k]:off[k + 1]]] = tgt[k]
    by_block = {}
    for l in range(L):
        if block[l] >= 0 and word[l] >= 0:
            by_block.setdefault(int(block[l]), set()).add(int(event_of[l]))
    assert sum(len(evs) > 1 for evs in by_block.values()) > 0.2 * info["n_event_pairs"]
    seeds = SEEDS[:2000]
    _, dur, _ = prop.run_many_arrays(seeds)
    kinds = flat["act_type"]
    gmap = {g[1]: g for g in gen}
    checked = 0
    for l in range(L):
        g, base = gmap[int(kinds[l])], float(flat["act_duration"][l])
        if g[0].startswith("empirical"):
            ref = PM.empirical_durations(seeds, l, base, g[2], g[3], g[0] == "empirical_relative",
                                         block=block[l], word=word[l])
            assert np.array_equal(dur[:, l], ref), l
        elif g[0] == "exponential":
            ref = PM.exponential_durations(seeds, l, base, g[2], g[3], block=block[l], word=word[l])
            np.testing.assert_allclose(dur[:, l], ref, rtol=2e-6)
        elif g[0] == "gamma":
            ref = _erlang_durations(seeds, base, int(g[2]), g[3], block[l], word[l])
            np.testing.assert_allclose(dur[:, l], ref, rtol=2e-6)
        else:
            continue
        checked += 1
    assert checked > 0.7 * L
    for n_warps, window in ((4, "auto"), (12, "global")):
        other = batching.compile_dag(flat, gen, n_warps, window)
        assert other.info()["n_event_pairs"] == info["n_event_pairs"]
        _, d2, _ = other.run_many_arrays(seeds[:256])
        assert np.array_equal(d2.view(np.int64), dur[:256].view(np.int64))
