"""CPU restatement of the reference's analytic PMF propagator (test infrastructure).

This module is the oracle for the GPU analytic engine
(``mc_dagprop_gb300.analytic``): only tests, the golden-fixture script and
``bench.py``'s CPU baseline use it.  It restates, step for step, the algorithm of

  src/mc_dagprop/analytic/_pmf.py        DiscretePMF.convolve (:107-125), maximum (:127-148),
                                         _rescale (:82-94), _expected_mass (:96-105)
  src/mc_dagprop/analytic/_propagator.py AnalyticPropagator.run (:89-148), _event_bounds
                                         (:150-156), _convert_to_simulated_event (:158-265)

with a PMF held as (first value, step, probabilities): its values are
first + i * step.  Extended precision (``np.longdouble``) is used where the
reference uses it.  Parity with the reference itself is pinned by
``tests/test_oracle_pin.py`` against ``tests/golden/analytic_ref.npz``.

A context is given in flat form (see ``flatten``):
  earliest, latest   float64[E]
  pmf_off            int64[K+1]   activity PMFs, concatenated
  pmf_first          float64[K]   first value of each activity PMF
  pmf_probs          float64[...]
  target             int32[T], pred_off int64[T+1], pred_src int32[P], pred_pmf int32[P]
  step               int;  max_delay (nan: none);  underflow_rule, overflow_rule (1..3)
"""
from __future__ import annotations

import math

import numpy as np

TRUNCATE, REMOVE, REDISTRIBUTE = 1, 2, 3


def _close(a: float, b: float) -> bool:
    return bool(np.isclose(a, b, rtol=1e-12, atol=1e-15))


def _expected(m1: float, m2: float) -> float:
    return 1.0 if _close(m1, 1.0) and _close(m2, 1.0) else m1 * m2


def _rescale(probs: np.ndarray, expected: float) -> np.ndarray:
    total = probs.sum()
    if total > 0 and not _close(total, expected):
        probs = probs * (expected / total)
    return probs


def convolve(a, b):
    """(first, probs) of the PMF of X + Y; the step is a's (_pmf.py:107-125)."""
    (fa, pa), (fb, pb) = a, b
    if len(pa) == 1:
        first, probs = fb + fa, pb * pa[0]
    elif len(pb) == 1:
        first, probs = fa + fb, pa * pb[0]
    else:
        first = fa + fb
        probs = np.convolve(pa.astype(np.longdouble), pb.astype(np.longdouble)).astype(float)
    return first, _rescale(probs, _expected(float(pa.sum()), float(pb.sum())))


def maximum(a, b, step: int):
    """(first, probs) of max(X, Y) on the common grid (_pmf.py:127-148)."""
    (fa, pa), (fb, pb) = a, b
    lo = min(fa, fb)
    hi = max(fa + step * (len(pa) - 1), fb + step * (len(pb) - 1))
    n = len(np.arange(lo, hi + step, step))
    oa = int(round((fa - lo) / step))
    ob = int(round((fb - lo) / step))
    xa = np.zeros(n, dtype=np.longdouble)
    xb = np.zeros(n, dtype=np.longdouble)
    xa[oa:oa + len(pa)] = pa
    xb[ob:ob + len(pb)] = pb
    ca = np.cumsum(xa, dtype=np.longdouble)
    cb = np.cumsum(xb, dtype=np.longdouble)
    ca_prev = np.concatenate((np.zeros(1, dtype=np.longdouble), ca[:-1]))
    probs = (xa * cb + xb * ca_prev).astype(float)
    return lo, _rescale(probs, _expected(float(pa.sum()), float(pb.sum())))


def event_bounds(earliest: float, latest: float, max_delay: float) -> tuple[int, int]:
    """_propagator.py:150-156: rounded bounds, the upper one capped by max_delay."""
    upper = latest if math.isnan(max_delay) else min(latest, earliest + max_delay)
    return int(np.round(earliest)), int(np.round(upper))


def clip(first: float, probs: np.ndarray, step: int, lo: int, hi: int, urule: int, orule: int):
    """_propagator.py:158-265: clip to [lo, hi] under the flow rules.
    Returns (first, probs, underflow, overflow); raises ValueError as the reference does."""
    if lo > hi:
        raise ValueError("min_value must not exceed max_value")
    vals = first + step * np.arange(len(probs), dtype=float)
    under = vals < lo
    over = vals > hi
    keep = ~(under | over)
    u_mass = float(probs[under].sum())
    o_mass = float(probs[over].sum())
    kv = vals[keep]
    kp = probs[keep].copy()
    red_u = 0.0
    if urule == TRUNCATE and u_mass > 0.0:
        if kv.size and np.isclose(kv[0], lo):
            kp[0] += u_mass
        elif kv.size == 0:
            kv, kp = np.array([float(lo)]), np.array([u_mass])
        else:
            raise ValueError("Underflow mass cannot be truncated: no lower-bound bin present.")
        u_mass = 0.0
    elif urule == REDISTRIBUTE and u_mass > 0.0:
        red_u, u_mass = u_mass, 0.0
    red_o = 0.0
    if orule == TRUNCATE and o_mass > 0.0:
        if kv.size and np.isclose(kv[-1], hi):
            kp[-1] += o_mass
        elif kv.size == 0:
            kv, kp = np.array([float(hi)]), np.array([o_mass])
        else:
            raise ValueError("Overflow mass cannot be truncated: no upper-bound bin present.")
        o_mass = 0.0
    elif orule == REDISTRIBUTE and o_mass > 0.0:
        red_o, o_mass = o_mass, 0.0
    red = red_u + red_o
    inside = kp.sum()
    if red > 0.0:
        if inside == 0.0:
            kv, kp = np.array([float(lo)]), np.array([red])
        else:
            kp = kp + red * (kp / inside)
    if kv.size == 0:
        raise ValueError("PMF must not be empty after clipping")
    target = max(0.0, 1.0 - (u_mass + o_mass))
    s = kp.sum()
    if s > 0.0:
        kp = kp / s
        kp = kp * target
    elif target > 0.0:
        kv, kp = np.array([float(lo)]), np.array([target])
    total = kp.sum() + u_mass + o_mass
    if not _close(total, 1.0):
        kp = kp * (1.0 / total if total > 0 else 1.0)
    return float(kv[0]), kp, u_mass, o_mass


def topo_order(E: int, target, pred_off, pred_src):
    """Kahn order with a FIFO queue (_propagator.py:15-45)."""
    from collections import deque

    preds = [None] * E
    indeg = [0] * E
    adj = [[] for _ in range(E)]
    for t_i, t in enumerate(target):
        srcs = [int(s) for s in pred_src[pred_off[t_i]:pred_off[t_i + 1]]]
        preds[int(t)] = t_i
        indeg[int(t)] = len(srcs)
        for s in srcs:
            adj[s].append(int(t))
    q = deque(i for i in range(E) if indeg[i] == 0)
    order = []
    while q:
        n = q.popleft()
        order.append(n)
        for d in adj[n]:
            indeg[d] -= 1
            if indeg[d] == 0:
                q.append(d)
    if len(order) != E:
        raise RuntimeError("Invalid DAG: cycle detected")
    return order, preds


def run(ctx: dict):
    """AnalyticPropagator.run (_propagator.py:89-148) on a flat context.
    Returns a list of (first, probs, underflow, overflow) per event."""
    E = len(ctx["earliest"])
    step = int(ctx["step"])
    order, preds = topo_order(E, ctx["target"], ctx["pred_off"], ctx["pred_src"])
    out = [None] * E
    for e in order:
        t_i = preds[e]
        lo_pred = ctx["pred_off"][t_i] if t_i is not None else 0
        hi_pred = ctx["pred_off"][t_i + 1] if t_i is not None else 0
        if t_i is None or hi_pred == lo_pred:
            v = round(float(ctx["earliest"][e]) / step) * step
            out[e] = (float(v), np.array([1.0]), 0.0, 0.0)
            continue
        combined = None
        for p in range(lo_pred, hi_pred):
            s = int(ctx["pred_src"][p])
            k = int(ctx["pred_pmf"][p])
            ep = (float(ctx["pmf_first"][k]), ctx["pmf_probs"][ctx["pmf_off"][k]:ctx["pmf_off"][k + 1]])
            conv = convolve((out[s][0], out[s][1]), ep)
            combined = conv if combined is None else maximum(combined, conv, step)
        lo, hi = event_bounds(float(ctx["earliest"][e]), float(ctx["latest"][e]), float(ctx["max_delay"]))
        out[e] = clip(combined[0], combined[1], step, lo, hi, int(ctx["underflow_rule"]), int(ctx["overflow_rule"]))
    return out


def flatten(earliest, latest, activities, precedence, step, urule, orule, max_delay=None):
    """Flat context from lists: activities {(src, dst): (idx, values, probs)},
    precedence [(target, [(src, idx), ...]), ...].  The PMF of a predecessor entry is
    the one of its (src, target) activity (_propagator.py:110)."""
    keys = list(activities.keys())
    slot = {k: i for i, k in enumerate(keys)}
    off = [0]
    first, probs = [], []
    for k in keys:
        _, v, p = activities[k]
        first.append(float(v[0]))
        probs.append(np.asarray(p, float))
        off.append(off[-1] + len(p))
    target, poff, psrc, ppmf = [], [0], [], []
    for t, plist in precedence:
        target.append(int(t))
        for s, _ in plist:
            psrc.append(int(s))
            ppmf.append(slot[(int(s), int(t))])
        poff.append(len(psrc))
    return {
        "earliest": np.asarray(earliest, float), "latest": np.asarray(latest, float),
        "pmf_off": np.asarray(off, np.int64), "pmf_first": np.asarray(first, float),
        "pmf_probs": np.concatenate(probs) if probs else np.zeros(0),
        "target": np.asarray(target, np.int32), "pred_off": np.asarray(poff, np.int64),
        "pred_src": np.asarray(psrc, np.int32), "pred_pmf": np.asarray(ppmf, np.int32),
        "step": int(step), "max_delay": float("nan") if max_delay is None else float(max_delay),
        "underflow_rule": int(urule), "overflow_rule": int(orule),
    }
