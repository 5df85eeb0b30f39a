"""Analytic engine, CPU side: the oracle pinned to the reference's own results
(tests/golden/analytic_ref.npz), the PMF helpers and host utilities of
mc_dagprop_gb300.analytic, and the context validation errors."""
from __future__ import annotations

import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))

import analytic_oracle as AO  # noqa: E402
from mc_dagprop_gb300 import analytic as AN  # noqa: E402

GOLDEN = np.load(os.path.join(HERE, "golden", "analytic_ref.npz"))
KEYS = ["earliest", "latest", "pmf_off", "pmf_first", "pmf_probs", "target", "pred_off", "pred_src", "pred_pmf",
        "step", "max_delay", "underflow_rule", "overflow_rule"]


def golden_case(name):
    return {k: GOLDEN[f"{name}/{k}"] for k in KEYS}


@pytest.mark.parametrize("name", list(GOLDEN["cases"]))
def test_oracle_matches_reference_exactly(name):
    out = AO.run(golden_case(name))
    assert np.array_equal([o[0] for o in out], GOLDEN[f"{name}/out_first"])
    assert np.array_equal([len(o[1]) for o in out], GOLDEN[f"{name}/out_len"])
    assert np.array_equal(np.concatenate([o[1] for o in out]), GOLDEN[f"{name}/out_probs"])
    assert np.array_equal([o[2] for o in out], GOLDEN[f"{name}/out_under"])
    assert np.array_equal([o[3] for o in out], GOLDEN[f"{name}/out_over"])


def test_reference_rule_table_known_answers():
    """The reference's rule table (test/test_discrete_simulator.py:300-397): event 1
    of the one-edge case, inside values [0, 1, 2]."""
    expected = {(1, 1): ([0.45, 0.25, 0.30], 0.0, 0.0), (1, 2): ([0.45, 0.25, 0.10], 0.0, 0.20),
                (2, 1): ([0.20, 0.25, 0.30], 0.25, 0.0), (2, 2): ([0.20, 0.25, 0.10], 0.25, 0.20),
                (3, 3): ([0.36363636363636365, 0.4545454545454546, 0.18181818181818182], 0.0, 0.0)}
    for (u, o), (probs, under, over) in expected.items():
        first, p, uu, oo = AO.run(golden_case(f"rules_{u}{o}"))[1]
        assert first == 0.0 and len(p) == 3
        np.testing.assert_allclose(p, probs, rtol=0, atol=1e-12)
        assert uu == pytest.approx(under) and oo == pytest.approx(over)


def _layered_pmfs(seed, n_layers, width, step):
    """Rebuild the activity PMFs of tests/golden/make_golden_analytic.py's layered
    cases with this package's helpers (same random sequence)."""
    rng = np.random.default_rng(seed)
    E = n_layers * width
    rng.integers(0, 10, E)
    pmfs = []
    for k in range(1, n_layers):
        lo = max(0, k - 2) * width
        for _ in range(width):
            srcs = rng.choice(np.arange(lo, k * width), size=int(rng.integers(1, 4)), replace=False)
            for _ in srcs:
                kind = int(rng.integers(0, 4))
                base = 40 // step * step
                if kind == 0:
                    pmf = AN.exponential_pmf(scale=float(rng.uniform(5, 40)), step=step, start=base,
                                             stop=base + int(rng.integers(12, 40)) * step)
                elif kind == 1:
                    pmf = AN.gamma_pmf(shape=2.0, scale=float(rng.uniform(2, 10)), step=step, start=float(base),
                                       stop=float(base + int(rng.integers(8, 30)) * step))
                elif kind == 2:
                    n = int(rng.integers(2, 6))
                    pmf = AN.empirical_pmf(base + step * np.arange(n, dtype=float) + step * int(rng.integers(0, 5)),
                                           rng.random(n) + 0.1, step=step)
                else:
                    pmf = AN.constant_pmf(float(base + step * int(rng.integers(1, 8))), step=step)
                pmfs.append(pmf)
    return pmfs


@pytest.mark.parametrize("name,seed,layers,width,step", [("layered_tt", 11, 12, 8, 1), ("layered_step5", 14, 8, 6, 5)])
def test_pmf_helpers_match_reference(name, seed, layers, width, step):
    pmfs = _layered_pmfs(seed, layers, width, step)
    c = golden_case(name)
    assert len(pmfs) == len(c["pmf_first"])
    probs = np.concatenate([p.probabilities for p in pmfs])
    assert np.array_equal([p.values[0] for p in pmfs], c["pmf_first"])
    np.testing.assert_allclose(probs, c["pmf_probs"], rtol=1e-10, atol=1e-15)


def test_host_pmf_utilities():
    """DiscretePMF.convolve / maximum, including the reference's own cases
    (test/test_pmf.py), against the oracle's restatement of the reference's
    operations: the convolution bit for bit where both take the same extended-
    precision sum, the maximum (an increment of a CDF product here, a sum of two
    products in the reference) within 1e-15."""
    a = AN.DiscretePMF(np.array([0.0, 1.0]), np.array([0.5, 0.5]), step=1)
    r = a.maximum(a)
    np.testing.assert_allclose(r.values, [0.0, 1.0])
    np.testing.assert_allclose(r.probabilities, [0.25, 0.75])
    tiny = 5e-324
    t = AN.DiscretePMF(np.array([0.0, 1.0]), np.array([1.0 - tiny, tiny]), step=1)
    r = t.maximum(t)
    assert np.all(r.probabilities >= 0.0) and np.isclose(float(r.total_mass), 1.0, rtol=1e-12, atol=1e-15)
    u = AN.DiscretePMF(np.arange(256, dtype=float), np.full(256, 1.0 / 256.0), step=1)
    r = u.convolve(u)
    assert np.isclose(float(r.total_mass), 1.0, rtol=1e-12, atol=1e-15) and np.all(r.probabilities >= 0.0)
    rng = np.random.default_rng(3)
    for _ in range(20):
        n, m = int(rng.integers(1, 30)), int(rng.integers(1, 30))
        x = AN.DiscretePMF(float(rng.integers(0, 50)) + np.arange(n, dtype=float), rng.dirichlet(np.ones(n)), 1)
        y = AN.DiscretePMF(float(rng.integers(0, 50)) + np.arange(m, dtype=float), rng.dirichlet(np.ones(m)), 1)
        cf, cp = AO.convolve((x.values[0], x.probabilities), (y.values[0], y.probabilities))
        c = x.convolve(y)
        assert c.values[0] == cf and len(c.probabilities) == len(cp)
        np.testing.assert_allclose(c.probabilities, cp, rtol=1e-15, atol=1e-18)
        mf, mp = AO.maximum((x.values[0], x.probabilities), (y.values[0], y.probabilities), 1)
        mx = x.maximum(y)
        assert mx.values[0] == mf and len(mx.probabilities) == len(mp)
        np.testing.assert_allclose(mx.probabilities, mp, rtol=0, atol=1e-15)
        np.testing.assert_array_equal(mx.values, mf + np.arange(len(mp)))


def _events(pairs):
    from mc_dagprop_gb300 import Event, EventTimestamp

    return tuple(Event(str(i), EventTimestamp(e, l, e)) for i, (e, l) in enumerate(pairs))


def test_context_validation_errors():
    """The reference's validation errors (test/test_discrete_simulator.py:113-190, 259-292)."""
    act = AN.AnalyticActivity(0, AN.DiscretePMF(np.array([1.0, 2.0]), np.array([0.5, 0.5]), step=1))
    ev = _events([(0.0, 100.0)] * 3)
    base = dict(events=ev, activities={(0, 1): (0, act)}, precedence_list=((1, ((0, 0),)),), step=1,
                underflow_rule=AN.UnderflowRule.TRUNCATE, overflow_rule=AN.OverflowRule.TRUNCATE)
    for bad in (dict(step=2), dict(step=0, activities={}, precedence_list=()),
                dict(max_delay=-1.0, activities={}, precedence_list=()),
                dict(events=_events([(5.0, 4.0)]), activities={}, precedence_list=()),
                dict(activities={(0, 1): (0, AN.AnalyticActivity(0, AN.DiscretePMF(np.array([1.0, 2.5]),
                                                                                  np.array([0.5, 0.5]), 1)))}),
                dict(activities={(0, 1): (0, act), (1, 0): (1, act)},
                     precedence_list=((1, ((0, 0),)), (0, ((1, 1),))))):
        with pytest.raises(ValueError):
            from mc_dagprop_gb300.analytic._context import validate_context

            validate_context(AN.AnalyticContext(**{**base, **bad}))
