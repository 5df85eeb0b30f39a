"""Fused per-event statistics (mean, p50/p90/p99, on-time fraction, histogram)
against numpy over the same samples' realized times (the reference's users'
pattern, demo/monte_carlo.py:48-49: stack run_many results, then reduce).

Tolerances: means within 1e-9 s (exact integer-tick accumulation); quantiles
within one histogram bin width of np.quantile (plus the gap between the two
order statistics numpy interpolates between); atoms (on time / capped) exact.
"""
from __future__ import annotations

import numpy as np
import pytest

import mc_dagprop_gb300 as m
from mc_dagprop_gb300 import workloads as W
from mcd_testlib import propagator_from_flat

pytestmark = pytest.mark.gpu


def _cases():
    yield "config0", W.config0()
    yield "five", W.config1(seed=8, n_layers=30, width=40)


@pytest.mark.parametrize("name,case", list(_cases()))
@pytest.mark.parametrize("window", ["smem", "global"])
def test_stats_match_numpy(cuda, name, case, window, monkeypatch):
    if window == "global":
        monkeypatch.setenv("MCD_NO_SMEM_WINDOW", "1")
    flat, gen = case
    prop = propagator_from_flat(m, flat, gen)
    n = 5000
    seeds = np.arange(n, dtype=np.int64) * 31 + 7
    real, _, _ = prop.run_many_arrays(seeds, durations=False)
    st = prop.run_stats(seeds=seeds, hist=True)
    earliest = flat["earliest"]
    ub = earliest + flat["max_delay"]
    np.testing.assert_allclose(st["mean"], real.mean(axis=0), rtol=0, atol=1e-9)
    w = st["bin_width"]
    assert 0 < w <= flat["max_delay"] / 256 * 1.01
    for key, p in (("p50", 0.5), ("p90", 0.9), ("p99", 0.99)):
        q = np.quantile(real, p, axis=0)
        # one bin, plus the gap between the two order statistics numpy interpolates
        gap = np.quantile(real, p, axis=0, method="higher") - np.quantile(real, p, axis=0, method="lower")
        assert np.all(np.abs(st[key] - q) <= w + gap + 1e-9), (key, np.max(np.abs(st[key] - q) - gap))
    on_time = (real == earliest[None, :]).mean(axis=0)
    np.testing.assert_array_equal(st["p_on_time"], on_time)
    h = st["hist"]
    assert (h.sum(axis=1)[:, None] >= 0).all()
    assert (h[:, :258].sum(axis=1) == n).all()
    np.testing.assert_array_equal(h[:, 256], (real == earliest[None, :]).sum(axis=0))
    capped = (real == ub[None, :]) & (real != earliest[None, :])
    np.testing.assert_array_equal(h[:, 257], capped.sum(axis=0))


def test_stats_seed_range_and_determinism(cuda):
    flat, gen = W.config1(seed=12, n_layers=40, width=50)
    prop = propagator_from_flat(m, flat, gen)
    a = prop.run_stats(n=3000, seed0=1000, hist=True)
    b = prop.run_stats(seeds=np.arange(1000, 4000), hist=True)
    c = prop.run_stats(n=3000, seed0=1000, hist=True)
    for k in ("mean", "p50", "p90", "p99", "p_on_time", "hist"):
        np.testing.assert_array_equal(a[k], b[k])
        np.testing.assert_array_equal(a[k], c[k])


def test_stats_large_sample_count(cuda):
    """65,536 samples of a mid-size DAG: the per-event mean equals the mean of the
    realized rows the plain path returns for the same seeds."""
    flat, gen = W.config1(seed=13, n_layers=100, width=100)
    prop = propagator_from_flat(m, flat, gen)
    n = 65_536
    st = prop.run_stats(n=n, seed0=0)
    acc = np.zeros(prop.node_count())
    for off in range(0, n, 8192):
        real, _, _ = prop.run_many_arrays(np.arange(off, off + 8192, dtype=np.int64), durations=False)
        acc += real.sum(axis=0)
    np.testing.assert_allclose(st["mean"], acc / n, rtol=1e-12, atol=1e-9)
