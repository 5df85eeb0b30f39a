"""Adjoint gradient of J = mean_s sum_e (realized - earliest).

1. Against a CPU gradient built from the oracle's cause_event and realized times
   (the reference's propagation loop, _core.cpp:331-350, restated in C) for the
   same samples' durations (the GPU sampler's, which the adjoint differentiates):
   earliest-time derivatives are integer path counts / n, so they must match
   exactly; base-duration derivatives carry d(duration)/d(base) in float, so
   within 1e-5 relative.
2. Against central finite differences with common random numbers (the same
   seeds), step 1e-3 s, on random coordinates: within 1e-3 absolute + 1e-3 relative.
3. Through the torch.autograd.Function wrapper.
4. Every memory plan -- all winners kept, level blocks recomputed from window
   checkpoints, the window off chip (global rows), several sample chunks --
   gives the same bits.
5. At the single-large-DAG size (200,000 events, 1,434 levels): against the
   oracle's chains, between plans, and against central finite differences.
"""
from __future__ import annotations

import numpy as np
import pytest

import mc_dagprop_gb300 as m
import oracle
from mc_dagprop_gb300 import batching
from mc_dagprop_gb300 import workloads as W
from mcd_testlib import chain_gradient, chain_gradient_loop

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("max_delay", [1800.0, 150.0])
def test_gradient_matches_cpu_chain(cuda, max_delay):
    flat, gen = W.config1(seed=31, n_layers=20, width=30)
    flat["max_delay"] = max_delay
    prop = batching.compile_dag(flat, gen)
    n, seed0 = 3000, 12345
    g = prop.gradient(n, seed0)
    _, dur, _ = prop.run_many_arrays(np.arange(seed0, seed0 + n, dtype=np.int64))
    real, cause = oracle.OracleSim(flat, gen).propagate_given(dur)  # the reference's chains
    obj, ge, gl = chain_gradient_loop(flat, gen, real, dur, cause)
    assert abs(g["objective"] - obj) <= 1e-9 * max(1.0, abs(obj))
    np.testing.assert_array_equal(g["grad_earliest"], ge)
    np.testing.assert_allclose(g["grad_base"], gl, rtol=1e-5, atol=1e-9)
    if max_delay < 200:
        assert (ge > 0).any()  # clamped events pass the derivative to their own earliest time


def test_gradient_finite_differences(cuda):
    flat, gen = W.config3()
    n, seed0, h = 16384, 777, 1e-3
    prop = batching.compile_dag(flat, gen)
    g = prop.gradient(n, seed0)

    def J(f):
        st = batching.compile_dag(f, gen).run_stats(n=n, seed0=seed0)
        return float(np.sum(st["mean"] - f["earliest"]))

    rng = np.random.default_rng(0)
    ev = rng.choice(len(flat["earliest"]), 12, replace=False)
    acts = rng.choice(len(flat["act_idx"]), 12, replace=False)
    for e in ev:
        fp, fm = dict(flat), dict(flat)
        fp["earliest"] = flat["earliest"].copy()
        fm["earliest"] = flat["earliest"].copy()
        fp["earliest"][e] += h
        fm["earliest"][e] -= h
        fd = (J(fp) - J(fm)) / (2 * h)
        assert abs(fd - g["grad_earliest"][e]) <= 1e-3 + 1e-3 * abs(fd), (e, fd, g["grad_earliest"][e])
    for k in acts:
        l = flat["act_idx"][k]
        fp, fm = dict(flat), dict(flat)
        fp["act_duration"] = flat["act_duration"].copy()
        fm["act_duration"] = flat["act_duration"].copy()
        fp["act_duration"][k] += h
        fm["act_duration"][k] -= h
        fd = (J(fp) - J(fm)) / (2 * h)
        assert abs(fd - g["grad_base"][l]) <= 1e-3 + 1e-3 * abs(fd), (k, fd, g["grad_base"][l])


def test_torch_autograd_wrapper(cuda):
    import torch

    from mc_dagprop_gb300.torch_ops import expected_tardiness

    flat, gen = W.config1(seed=32, n_layers=10, width=20)
    e = torch.tensor(flat["earliest"], dtype=torch.float64, requires_grad=True)
    b = torch.tensor(flat["act_duration"], dtype=torch.float64, requires_grad=True)
    J = expected_tardiness(e, b, flat, gen, n=2048, seed0=5)
    J.backward()
    g = batching.compile_dag(flat, gen).gradient(2048, 5)
    assert abs(J.item() - g["objective"]) < 1e-12 * max(1, abs(J.item()))
    np.testing.assert_array_equal(e.grad.numpy(), g["grad_earliest"])
    np.testing.assert_array_equal(b.grad.numpy(), g["grad_base"][flat["act_idx"]])


def _same_bits(a, b):
    assert a["objective"] == b["objective"]
    np.testing.assert_array_equal(a["grad_earliest"], b["grad_earliest"])
    np.testing.assert_array_equal(a["grad_base"], b["grad_base"])


@pytest.mark.parametrize("mode", ["blocks", "chunks_blocks", "offchip", "offchip_blocks"])
def test_gradient_plans_agree_bitwise(cuda, mode, monkeypatch):
    flat, gen = W.config1(seed=33, n_layers=40, width=60)
    n, seed0 = 2000, 99
    ref = batching.compile_dag(flat, gen).gradient(n, seed0)
    assert ref["level_blocks"] == 1 and ref["samples_per_chunk"] == 2016
    if "blocks" in mode:
        monkeypatch.setenv("MCD_ADJ_BLOCK_EVENTS", "300")
    if "chunks" in mode:
        monkeypatch.setenv("MCD_ADJ_BUDGET_MB", "1")
    if "offchip" in mode:
        monkeypatch.setenv("MCD_NO_SMEM_WINDOW", "1")
    prop = batching.compile_dag(flat, gen)
    assert prop.info()["window_in_smem"] == ("offchip" not in mode)
    g = prop.gradient(n, seed0)
    if "blocks" in mode:
        assert g["level_blocks"] >= 8
    if "chunks" in mode:
        assert g["samples_per_chunk"] < 2000
    _same_bits(g, ref)


@pytest.fixture(scope="module")
def bench_dag_grad():
    """The single-large-DAG workload (bench.py's DAG) and its gradient over 256 samples."""
    flat, gen = W.config1(seed=1, n_layers=2000, width=100)
    prop = batching.compile_dag(flat, gen)
    assert prop.info()["n_events"] == 200_000 and prop.info()["window_in_smem"]
    n, seed0 = 256, 4242
    return flat, gen, prop, n, seed0, prop.gradient(n, seed0)


def test_gradient_200k_events_matches_oracle_chain(cuda, bench_dag_grad):
    flat, gen, prop, n, seed0, g = bench_dag_grad
    _, dur, _ = prop.run_many_arrays(np.arange(seed0, seed0 + n, dtype=np.int64))
    real, cause = oracle.OracleSim(flat, gen).propagate_given(dur)
    obj, ge, gl = chain_gradient(flat, gen, real, dur, cause)
    assert abs(g["objective"] - obj) <= 1e-9 * abs(obj)
    np.testing.assert_array_equal(g["grad_earliest"], ge)
    np.testing.assert_allclose(g["grad_base"], gl, rtol=1e-5, atol=1e-9)
    assert (ge != 0).sum() > 1000 and (gl != 0).sum() > 1000


@pytest.mark.parametrize("mode", ["blocks", "offchip"])
def test_gradient_200k_events_plans_agree(cuda, bench_dag_grad, mode, monkeypatch):
    flat, gen, _, n, seed0, ref = bench_dag_grad
    if mode == "blocks":
        monkeypatch.setenv("MCD_ADJ_BUDGET_MB", "128")  # the winners of 256 samples need 307 MB
    else:
        monkeypatch.setenv("MCD_NO_SMEM_WINDOW", "1")
    prop = batching.compile_dag(flat, gen)
    g = prop.gradient(n, seed0)
    if mode == "blocks":
        assert g["level_blocks"] > 1 and g["samples_per_chunk"] == 256
    else:
        assert not prop.info()["window_in_smem"]
    _same_bits(g, ref)


def test_gradient_200k_events_finite_differences(cuda, bench_dag_grad):
    """Central differences with common random numbers (step 1e-3 s) of the
    statistics path's objective, on three event times and three link bases."""
    flat, gen, prop, _, _, _ = bench_dag_grad
    n, seed0, h = 4096, 77, 1e-3
    g = prop.gradient(n, seed0)

    def J(f):
        st = batching.compile_dag(f, gen).run_stats(n=n, seed0=seed0)
        return float(np.sum(st["mean"] - f["earliest"]))

    rng = np.random.default_rng(5)
    ev = rng.choice(np.flatnonzero(g["grad_earliest"] != 0), 3, replace=False)
    links = rng.choice(np.flatnonzero(g["grad_base"] != 0), 3, replace=False)
    pos = {int(l): k for k, l in enumerate(flat["act_idx"])}
    for e in ev:
        fp, fm = dict(flat), dict(flat)
        fp["earliest"], fm["earliest"] = flat["earliest"].copy(), flat["earliest"].copy()
        fp["earliest"][e] += h
        fm["earliest"][e] -= h
        fd = (J(fp) - J(fm)) / (2 * h)
        assert abs(fd - g["grad_earliest"][e]) <= 1e-3 + 1e-3 * abs(fd), (e, fd, g["grad_earliest"][e])
    for l in links:
        k = pos[int(l)]
        fp, fm = dict(flat), dict(flat)
        fp["act_duration"], fm["act_duration"] = flat["act_duration"].copy(), flat["act_duration"].copy()
        fp["act_duration"][k] += h
        fm["act_duration"][k] -= h
        fd = (J(fp) - J(fm)) / (2 * h)
        assert abs(fd - g["grad_base"][l]) <= 1e-3 + 1e-3 * abs(fd), (l, fd, g["grad_base"][l])
