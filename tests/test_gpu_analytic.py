"""Analytic engine on the GPU against the reference's own results (golden
fixtures) and the oracle: supports exactly, probabilities and flow masses within
1e-12 (the reference accumulates in extended precision, the GPU in FP64)."""
from __future__ import annotations

import ctypes as C
import math
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))

import analytic_oracle as AO  # noqa: E402
from mc_dagprop_gb300 import Event, EventTimestamp  # noqa: E402
from mc_dagprop_gb300 import analytic as AN  # noqa: E402
from mc_dagprop_gb300.analytic import _propagator as PR  # noqa: E402

pytestmark = pytest.mark.gpu

GOLDEN = np.load(os.path.join(HERE, "golden", "analytic_ref.npz"))
KEYS = ["earliest", "latest", "pmf_off", "pmf_first", "pmf_probs", "target", "pred_off", "pred_src", "pred_pmf",
        "step", "max_delay", "underflow_rule", "overflow_rule"]
ATOL = 1e-12


def run_flat(ctx):
    """The C ABI on a flat context: (first, len, probs per event, under, over)."""
    flat = {k: np.ascontiguousarray(ctx[k]) for k in KEYS[:9]}
    flat["pmf_off"] = flat["pmf_off"].astype(np.int64)
    flat["pred_off"] = flat["pred_off"].astype(np.int64)
    if len(flat["pmf_probs"]) == 0:
        flat["pmf_probs"] = np.zeros(1)
    md = float(ctx["max_delay"])
    desc = PR._desc(flat, int(ctx["step"]), None if math.isnan(md) else md, int(ctx["underflow_rule"]),
                    int(ctx["overflow_rule"]))
    L = PR._api()
    h = C.c_void_p()
    PR._check(L.mcd_analytic_create(C.byref(desc), C.byref(h)))
    try:
        PR._check(L.mcd_analytic_run(h))
        E = len(flat["earliest"])
        first, under, over = np.empty(E), np.empty(E), np.empty(E)
        off, ln = np.empty(E, np.int64), np.empty(E, np.int64)
        probs = np.empty(max(1, L.mcd_analytic_bins(h)))
        p = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
        PR._check(L.mcd_analytic_fetch(h, p(first), p(off), p(ln), p(probs), p(under), p(over)))
    finally:
        L.mcd_analytic_destroy(h)
    return first, ln, [probs[o:o + n] for o, n in zip(off, ln)], under, over


def compare(got, want_first, want_len, want_probs, want_under, want_over):
    first, ln, probs, under, over = got
    assert np.array_equal(first, want_first)
    assert np.array_equal(ln, want_len)
    np.testing.assert_allclose(np.concatenate(probs), want_probs, rtol=0, atol=ATOL)
    np.testing.assert_allclose(under, want_under, rtol=0, atol=ATOL)
    np.testing.assert_allclose(over, want_over, rtol=0, atol=ATOL)


@pytest.mark.parametrize("name", list(GOLDEN["cases"]))
def test_gpu_matches_reference(cuda, name):
    ctx = {k: GOLDEN[f"{name}/{k}"] for k in KEYS}
    compare(run_flat(ctx), GOLDEN[f"{name}/out_first"], GOLDEN[f"{name}/out_len"], GOLDEN[f"{name}/out_probs"],
            GOLDEN[f"{name}/out_under"], GOLDEN[f"{name}/out_over"])


def random_context(seed, n_layers, width, pmf_len, step=1, urule=1, orule=1, max_delay=None):
    rng = np.random.default_rng(seed)
    E = n_layers * width
    earliest = (np.repeat(np.arange(n_layers) * 60, width) + rng.integers(0, 20, E)) // step * step * 1.0
    latest = earliest + 900.0
    acts, prec, idx = {}, [], 0
    for k in range(1, n_layers):
        lo = max(0, k - 3) * width
        for j in range(width):
            t = k * width + j
            plist = []
            for s in rng.choice(np.arange(lo, k * width), size=int(rng.integers(1, 5)), replace=False):
                n = int(rng.integers(1, pmf_len))
                acts[(int(s), t)] = (idx, step * (10 + np.arange(n, dtype=float)), rng.dirichlet(np.ones(n)))
                plist.append((int(s), idx))
                idx += 1
            prec.append((t, plist))
    return AO.flatten(earliest, latest, acts, prec, step, urule, orule, max_delay)


@pytest.mark.parametrize("urule,orule,max_delay", [(1, 1, None), (1, 3, 300.0), (3, 1, 500.0)])
def test_gpu_matches_oracle_large(cuda, urule, orule, max_delay):
    """A 600-event DAG with PMFs of up to 400 bins: event windows of 900 s, wide
    enough that the maximum's grid spans thousands of bins (global scratch)."""
    ctx = random_context(5, 30, 20, 400, urule=urule, orule=orule, max_delay=max_delay)
    ref = AO.run(ctx)
    compare(run_flat(ctx), [r[0] for r in ref], [len(r[1]) for r in ref], np.concatenate([r[1] for r in ref]),
            [r[2] for r in ref], [r[3] for r in ref])


def _ctx(events, acts, prec, u=AN.UnderflowRule.TRUNCATE, o=AN.OverflowRule.TRUNCATE, step=1, max_delay=None):
    ev = tuple(Event(str(i), EventTimestamp(e, l, e)) for i, (e, l) in enumerate(events))
    return AN.AnalyticContext(events=ev, activities=acts, precedence_list=prec, step=step, underflow_rule=u,
                              overflow_rule=o, max_delay=max_delay)


def test_python_api_rule_table(cuda):
    """The reference's rule table through the Python API (test/test_discrete_simulator.py:300-397)."""
    edge = AN.AnalyticActivity(0, AN.DiscretePMF(np.array([-2.0, -1.0, 0.0, 1.0, 2.0, 3.0]),
                                                 np.array([0.10, 0.15, 0.20, 0.25, 0.10, 0.20]), step=1))
    expected = {(1, 1): [0.45, 0.25, 0.30], (1, 2): [0.45, 0.25, 0.10], (1, 3): [0.5625, 0.3125, 0.1250],
                (2, 1): [0.20, 0.25, 0.30], (2, 2): [0.20, 0.25, 0.10],
                (2, 3): [0.2727272727272727, 0.3409090909090909, 0.13636363636363635],
                (3, 1): [0.26666666666666666, 0.3333333333333333, 0.4000000000000001],
                (3, 2): [0.2909090909090909, 0.36363636363636365, 0.14545454545454545],
                (3, 3): [0.36363636363636365, 0.4545454545454546, 0.18181818181818182]}
    for (u, o), probs in expected.items():
        ctx = _ctx([(0.0, 0.0), (0.0, 2.0)], {(0, 1): (0, edge)}, ((1, ((0, 0),)),), AN.UnderflowRule(u),
                   AN.OverflowRule(o))
        res = AN.create_analytic_propagator(ctx).run()
        assert all(isinstance(r, AN.SimulatedEvent) for r in res)
        np.testing.assert_allclose(res[1].pmf.values, [0.0, 1.0, 2.0])
        np.testing.assert_allclose(res[1].pmf.probabilities, probs, rtol=0, atol=1e-12)
        assert np.isclose(float(res[1].pmf.total_mass + res[1].underflow + res[1].overflow), 1.0,
                          rtol=1e-12, atol=1e-15)


def test_python_api_errors_and_repeat(cuda):
    """Clipping that leaves nothing (REMOVE on both sides of an all-outside PMF)
    and a missing lower-bound bin raise ValueError as in the reference; a second
    run() returns the same results."""
    edge = AN.AnalyticActivity(0, AN.DiscretePMF(np.array([20.0, 21.0]), np.array([0.5, 0.5]), step=1))
    ctx = _ctx([(0.0, 0.0), (0.0, 5.0)], {(0, 1): (0, edge)}, ((1, ((0, 0),)),), AN.UnderflowRule.REMOVE,
               AN.OverflowRule.REMOVE)
    with pytest.raises(ValueError):
        AN.create_analytic_propagator(ctx).run()
    edge5 = AN.AnalyticActivity(0, AN.DiscretePMF(np.array([0.0, 5.0]), np.array([0.5, 0.5]), step=5))
    ctx5 = _ctx([(0.0, 0.0), (3.0, 20.0)], {(0, 1): (0, edge5)}, ((1, ((0, 0),)),), step=5)
    with pytest.raises(ValueError):
        AN.create_analytic_propagator(ctx5).run()
    c = {k: GOLDEN[f"layered_tt/{k}"] for k in KEYS}
    a, b = run_flat(c), run_flat(c)
    assert np.array_equal(np.concatenate(a[2]), np.concatenate(b[2]))
    prop = AN.create_analytic_propagator(_ctx([(0.0, 10.0), (0.0, 10.0)], {(0, 1): (0, edge)}, ((1, ((0, 0),)),)))
    r1, r2 = prop.run(), prop.run()
    assert np.array_equal(r1[1].pmf.probabilities, r2[1].pmf.probabilities)
