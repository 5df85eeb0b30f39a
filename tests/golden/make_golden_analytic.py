"""Generates ``analytic_ref.npz`` from the reference's own analytic PMF propagator.

Runs ``mc_dagprop.analytic.create_analytic_propagator(ctx).run()`` of the
reference (pure Python, loaded from its sources by ``oracle/ref_loader.py``) on
small contexts -- the cases of the reference's own tests
(test/test_discrete_simulator.py) and seeded layered DAGs with the reference's
PMF helpers -- and stores each context in flat form (``oracle/analytic_oracle.py``)
with the per-event results (first value, probabilities, underflow, overflow).

Usage:  python tests/golden/make_golden_analytic.py     (needs the reference sources)
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import analytic_oracle as AO  # noqa: E402
import ref_loader  # noqa: E402


def reference_run(an, core, case):
    """Build the reference context for a case and run it."""
    events = tuple(core.Event(str(i), core.EventTimestamp(float(e), float(l), float(e)))
                   for i, (e, l) in enumerate(zip(case["earliest"], case["latest"])))
    acts = {k: (idx, an.AnalyticActivity(idx, an.DiscretePMF(np.asarray(v, float), np.asarray(p, float),
                                                              step=int(st))))
            for k, (idx, v, p, st) in case["activities"].items()}
    prec = tuple((int(t), tuple((int(s), int(i)) for s, i in pl)) for t, pl in case["precedence"])
    ctx = an.AnalyticContext(events=events, activities=acts, precedence_list=prec, step=int(case["step"]),
                             underflow_rule=an.UnderflowRule(case["urule"]),
                             overflow_rule=an.OverflowRule(case["orule"]), max_delay=case.get("max_delay"))
    return an.create_analytic_propagator(ctx).run()


def layered_case(seed, n_layers, width, step, urule, orule, max_delay, an):
    rng = np.random.default_rng(seed)
    E = n_layers * width
    earliest = (np.repeat(np.arange(n_layers) * 30, width) + rng.integers(0, 10, E)) // step * step * 1.0
    latest = earliest + 300.0
    acts, prec = {}, []
    idx = 0
    for k in range(1, n_layers):
        lo = max(0, k - 2) * width
        for j in range(width):
            t = k * width + j
            srcs = rng.choice(np.arange(lo, k * width), size=int(rng.integers(1, 4)), replace=False)
            plist = []
            for s in srcs:
                kind = int(rng.integers(0, 4))
                base = 40 // step * step  # arrivals reach the target's window
                if kind == 0:
                    pmf = an.exponential_pmf(scale=float(rng.uniform(5, 40)), step=step, start=base,
                                             stop=base + int(rng.integers(12, 40)) * step)
                elif kind == 1:
                    pmf = an.gamma_pmf(shape=2.0, scale=float(rng.uniform(2, 10)), step=step, start=float(base),
                                       stop=float(base + int(rng.integers(8, 30)) * step))
                elif kind == 2:
                    n = int(rng.integers(2, 6))
                    pmf = an.empirical_pmf(base + step * np.arange(n, dtype=float) + step * int(rng.integers(0, 5)),
                                           rng.random(n) + 0.1, step=step)
                else:
                    pmf = an.constant_pmf(float(base + step * int(rng.integers(1, 8))), step=step)
                acts[(int(s), t)] = (idx, pmf.values, pmf.probabilities, step)
                plist.append((int(s), idx))
                idx += 1
            prec.append((t, plist))
    return {"earliest": earliest, "latest": latest, "activities": acts, "precedence": prec, "step": step,
            "urule": urule, "orule": orule, "max_delay": max_delay}


def cases(an):
    T, R, D = 1, 2, 3
    out = {}
    three = {"earliest": [0.0, 0.0, 0.0], "latest": [100.0, 100.0, 100.0], "step": 1,
             "activities": {(0, 1): (0, [1.0, 2.0], [0.5, 0.5], 1), (1, 2): (1, [0.0, 1.0], [0.5, 0.5], 1)},
             "precedence": [(1, [(0, 0)]), (2, [(1, 1)])], "urule": T, "orule": T}
    out["chain3"] = three
    out["bounds_overflow"] = dict(three, latest=[0.0, 2.0, 1.0])
    vals = [-2.0, -1.0, 0.0, 1.0, 2.0, 3.0]
    probs = [0.10, 0.15, 0.20, 0.25, 0.10, 0.20]
    for u in (T, R, D):
        for o in (T, R, D):
            out[f"rules_{u}{o}"] = {"earliest": [0.0, 0.0], "latest": [0.0, 2.0], "step": 1,
                                    "activities": {(0, 1): (0, vals, probs, 1)},
                                    "precedence": [(1, [(0, 0)])], "urule": u, "orule": o}
    zedge = {(0, 1): (0, [-1.0, 0.0, 1.0, 2.0], [0.5, 0.0, 0.0, 0.5], 1)}
    for u, o in ((T, T), (R, R), (R, T), (T, R)):
        out[f"zeros_{u}{o}"] = {"earliest": [0.0, 0.0], "latest": [10.0, 1.0], "step": 1, "activities": zedge,
                                "precedence": [(1, [(0, 0)])], "urule": u, "orule": o}
    uv = np.arange(-180.0, 1800.1, 1.0)
    up = np.ones_like(uv) / len(uv)
    pairs = [(0, 1), (0, 2), (1, 3), (2, 3), (2, 4), (3, 4)]
    out["uniform_network"] = {
        "earliest": [0.0] * 5, "latest": [2000.0] * 5, "step": 1,
        "activities": {p: (i, uv, up, 1) for i, p in enumerate(pairs)},
        "precedence": [(1, [(0, 0)]), (2, [(0, 1)]), (3, [(1, 2), (2, 3)]), (4, [(2, 4), (3, 5)])],
        "urule": T, "orule": T}
    # (the reference asserts that clipping keeps an event's incoming mass, which a
    # removed flow breaks one level further on, so REMOVE is covered by the one-edge cases)
    out["layered_tt"] = layered_case(11, 12, 8, 1, T, T, None, an)
    out["layered_td"] = layered_case(12, 12, 8, 1, T, D, 120.0, an)
    out["layered_dt"] = layered_case(13, 10, 6, 1, D, T, 200.0, an)
    out["layered_step5"] = layered_case(14, 8, 6, 5, T, T, None, an)
    return out


def main():
    core = ref_loader.load()
    an = ref_loader.load_analytic()
    store = {}
    names = []
    for name, case in cases(an).items():
        res = reference_run(an, core, case)
        acts = {k: (i, np.asarray(v, float), np.asarray(p, float)) for k, (i, v, p, _) in case["activities"].items()}
        flat = AO.flatten(case["earliest"], case["latest"], acts, case["precedence"], case["step"], case["urule"],
                          case["orule"], case.get("max_delay"))
        for k, v in flat.items():
            store[f"{name}/{k}"] = np.asarray(v)
        store[f"{name}/out_first"] = np.array([float(r.pmf.values[0]) for r in res])
        store[f"{name}/out_len"] = np.array([len(r.pmf.probabilities) for r in res], np.int64)
        store[f"{name}/out_probs"] = np.concatenate([np.asarray(r.pmf.probabilities, float) for r in res])
        store[f"{name}/out_under"] = np.array([float(r.underflow) for r in res])
        store[f"{name}/out_over"] = np.array([float(r.overflow) for r in res])
        names.append(name)
    store["cases"] = np.array(names)
    np.savez_compressed(os.path.join(HERE, "analytic_ref.npz"), **store)
    print("wrote", len(names), "cases")


if __name__ == "__main__":
    main()
