"""Per-type delay inspection on the GPU (the reference's demo/inspection.py:11-29)
against the same histograms computed by numpy from the propagator's own sampled
durations (same seeds): identical counts, moments to rounding."""
from __future__ import annotations

import numpy as np
import pytest

import mc_dagprop_gb300 as m
from mc_dagprop_gb300 import inspection
from mc_dagprop_gb300 import workloads as W
from mcd_testlib import propagator_from_flat

pytestmark = pytest.mark.gpu


def numpy_bins(x, lo, hi, nb):
    out = np.zeros(nb + 2, np.int64)
    b = np.where(~(x >= lo), 0, np.where(~(x < hi), nb + 1,
                                          1 + np.minimum(((x - lo) * nb / (hi - lo)).astype(np.int64), nb - 1)))
    np.add.at(out, b, 1)
    return out


def test_delay_histograms_match_numpy(cuda):
    flat, gen = W.config1(seed=4, n_layers=30, width=40)
    prop = propagator_from_flat(m, flat, gen)
    seeds = np.arange(3000, dtype=np.int64) + 17
    res = inspection.delay_histograms(prop, flat, seeds, bins=48)
    _, dur, _ = prop.run_many_arrays(seeds)
    idx, base, typ = flat["act_idx"], flat["act_duration"], flat["act_type"]
    assert sorted(res) == sorted(set(int(t) for t in typ))
    for t, entry in res.items():
        sel = typ == t
        d = dur[:, idx[sel]] - base[sel]
        b = base[sel]
        rel = (d / b)[:, b != 0.0]
        for name, x in (("absolute", d.ravel()), ("relative", rel.ravel())):
            e = entry[name]
            lo, hi = e["edges"][0], e["edges"][-1]
            want = numpy_bins(x, lo, hi, 48)
            got = np.concatenate([[e["under"]], e["counts"], [e["over"]]])
            assert np.array_equal(got, want), (t, name)
            assert e["count"] == x.size
            assert e["mean"] == pytest.approx(x.mean(), rel=1e-9, abs=1e-9)
            assert e["var"] == pytest.approx(x.var(), rel=1e-6, abs=1e-9)
    # the constant type: every delay equal (one bin), exponential/gamma: non-negative
    assert res[1]["absolute"]["counts"].sum() + res[1]["absolute"]["under"] + res[1]["absolute"]["over"] == \
        3000 * int((typ == 1).sum())


def test_delay_histograms_fixed_ranges_and_errors(cuda):
    flat, gen = W.config1(seed=5, n_layers=10, width=20)
    prop = propagator_from_flat(m, flat, gen)
    seeds = np.arange(500, dtype=np.int64)
    res = inspection.delay_histograms(prop, flat, seeds, bins=10, ranges={2: (0.0, 10.0, 0.0, 0.05)})
    e = res[2]["relative"]
    assert e["edges"][0] == 0.0 and e["edges"][-1] == 0.05
    assert e["counts"].sum() + e["under"] + e["over"] == e["count"]
    with pytest.raises(ValueError):
        inspection.delay_histograms(prop, flat, seeds, bins=100000)
