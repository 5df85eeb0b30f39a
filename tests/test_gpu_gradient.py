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
"""
from __future__ import annotations

import numpy as np
import pytest

import mc_dagprop_gb300 as m
import oracle
from mc_dagprop_gb300 import batching
from mc_dagprop_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def cpu_gradient(flat, gen, real, dur, cause):
    """Backward pass over the samples' winning chains (vectorised over samples)."""
    S, E = real.shape
    earliest = flat["earliest"]
    ub = earliest + flat["max_delay"]
    L = dur.shape[1]
    base = np.zeros(L)
    kind = np.zeros(L, dtype=object)
    types = {g[1]: g for g in gen}
    for i, d, t in zip(flat["act_idx"], flat["act_duration"], flat["act_type"]):
        base[i] = d
        kind[i] = types.get(int(t), ("none",))
    preds = {}
    off = flat["pred_offsets"]
    for k, t in enumerate(flat["target"]):
        preds[int(t)] = list(zip(flat["pred_src"][off[k]:off[k + 1]], flat["pred_act"][off[k]:off[k + 1]]))
    cnt = np.zeros((S, E), np.int64)
    ge = np.zeros(E, np.int64)
    gl = np.zeros(L)
    delayed = real > earliest[None, :]
    for e in range(E - 1, -1, -1):  # layered DAGs: index order is topological
        c = cnt[:, e] + delayed[:, e]
        ce = cause[:, e]
        pl = preds.get(e, [])
        clamped = np.zeros(S, bool)
        link = np.full(S, -1)
        for src, l in pl:
            sel = ce == src
            link[sel] = l
            clamped[sel] = real[sel, src] + dur[sel, l] > ub[e]
        ge[e] = np.sum(np.where((ce < 0) | clamped, c, 0)) - delayed[:, e].sum()
        flow = (ce >= 0) & ~clamped
        for src, l in pl:
            sel = flow & (ce == src)
            if not sel.any():
                continue
            np.add.at(cnt[:, src], np.nonzero(sel)[0], c[sel])
            spec = kind[l]
            if spec[0] in ("exponential", "gamma", "empirical_relative"):
                dfac = (dur[sel, l] / base[l]).astype(np.float32)
            elif spec[0] == "constant":
                dfac = np.float32(1.0 + spec[2])
            else:
                dfac = np.float32(1.0)
            gl[l] += np.sum(c[sel] * np.asarray(dfac, np.float64))
    obj = (real - earliest[None, :]).sum(axis=1).mean()
    return obj, ge / S, gl / S


@pytest.mark.parametrize("max_delay", [1800.0, 150.0])
def test_gradient_matches_cpu_chain(cuda, max_delay):
    flat, gen = W.config1(seed=31, n_layers=20, width=30)
    flat["max_delay"] = max_delay
    prop = batching.compile_dag(flat, gen)
    n, seed0 = 3000, 12345
    g = prop.gradient(n, seed0)
    _, dur, _ = prop.run_many_arrays(np.arange(seed0, seed0 + n, dtype=np.int64))
    real, cause = oracle.OracleSim(flat, gen).propagate_given(dur)  # the reference's chains
    obj, ge, gl = cpu_gradient(flat, gen, real, dur, cause)
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
