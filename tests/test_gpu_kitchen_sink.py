"""Every sampler path in one DAG (see mcd_testlib.kitchen_sink) through the
sampled kernel at several CTA widths, window places, time signs and predecessor
list lengths (events of up to 12 draw several Philox blocks each): realized
and cause_event equal the oracle's propagation of the durations the kernel
reports, bit for bit, and links no entry references get their durations."""
from __future__ import annotations

import numpy as np
import pytest

import mc_dagprop_gb300 as m
import oracle
from mc_dagprop_gb300 import workloads as W
from mcd_testlib import kitchen_sink

pytestmark = pytest.mark.gpu


def _prop(flat, gen, **kw):
    g = W.to_generator(m, gen)
    return m.MonteCarloPropagator.from_arrays(flat["earliest"], flat["act_idx"], flat["act_duration"],
                                              flat["act_type"], flat["target"], flat["pred_offsets"],
                                              flat["pred_src"], flat["pred_act"], flat["max_delay"], g, **kw)


def _bits(a):
    return np.ascontiguousarray(a, dtype=np.float64).view(np.int64)


@pytest.mark.parametrize("warps,window,shift,big,preds", [(24, "auto", 0.0, False, 4), (8, "global", 0.0, False, 4),
                                                          (24, "auto", -500.0, False, 4), (12, "auto", 0.0, True, 4),
                                                          (16, "auto", 0.0, False, 12)])
def test_kitchen_sink_outputs_are_the_oracle_propagation(cuda, warps, window, shift, big, preds):
    flat, gen = kitchen_sink(seed=5, n_layers=40, width=150, big_table=big, max_preds=preds)
    flat = dict(flat, earliest=flat["earliest"] + shift)
    prop = _prop(flat, gen, n_warps=warps, window=window)
    info = prop.info()
    assert info["n_warps"] == warps and info["window_in_smem"] == (window == "auto")
    assert info["positive"] == (shift == 0.0) and info["tables_in_smem"] == (not big)
    seeds = np.arange(300, dtype=np.int64) * 104729 + 17
    real, dur, cause = prop.run_many_arrays(seeds)
    ro, co = oracle.OracleSim(flat, gen).propagate_given(dur)
    assert np.array_equal(_bits(real), _bits(ro))
    assert np.array_equal(cause, co)
    P = len(flat["pred_act"])
    unref = dur[:, P:P + 20]  # activities no entry references are still drawn
    assert np.isfinite(unref).all() and (unref > 0).any()
    # the statistics mode sees the same samples
    st = prop.run_stats(seeds=seeds)
    np.testing.assert_allclose(st["mean"], real.mean(axis=0), rtol=0, atol=1e-9 * np.abs(real).max())
