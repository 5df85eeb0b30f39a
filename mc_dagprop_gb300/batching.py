"""Batched runs of many DAGs in one persistent launch, with a small autotuner.

A batch compiles every DAG with the same number of warps per CTA (the CTA size
of the persistent launch) and runs all (DAG, 32-sample tile) work items in one
CUDA graph (``mc_dagprop_gb300.Batch``).  The warps per CTA trade work per
stage against barrier and idle time: wide DAGs want many warps, narrow ones few.
``tune_warps`` times the candidates on a calibration subset of the batch and
keeps the fastest; results are cached per shape class in a JSON file
(``$MCD_AUTOTUNE_CACHE``, default ``~/.cache/mc_dagprop_gb300/autotune.json``).
"""
from __future__ import annotations

import json
import math
import os
import time

import numpy as np

from . import _core
from . import workloads as W

CANDIDATE_WARPS = (4, 8, 16)


def _cache_path() -> str:
    return os.environ.get("MCD_AUTOTUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "mc_dagprop_gb300", "autotune.json"))


def shape_class(flats: list, ns: list) -> str:
    """Coarse key of a batch: log2 of the mean events, mean level width and mean samples."""
    ev = np.mean([len(f["earliest"]) for f in flats])
    width = np.mean([len(f["earliest"]) / max(1, _levels(f)) for f in flats])
    return f"E{int(round(math.log2(max(ev, 1))))}-W{int(round(math.log2(max(width, 1))))}-S{int(round(math.log2(max(np.mean(ns), 1))))}"


def _levels(flat: dict) -> int:
    """Number of levels (longest path) of a flat DAG, for the shape class."""
    E = len(flat["earliest"])
    level = np.zeros(E, np.int64)
    off, tgt, src = flat["pred_offsets"], flat["target"], flat["pred_src"]
    order = np.argsort(tgt, kind="stable")  # layered generators list targets in topological order
    for k in order:
        b, e = off[k], off[k + 1]
        if e > b:
            level[tgt[k]] = 1 + level[src[b:e]].max()
    return int(level.max()) + 1


def compile_dag(flat: dict, gen: list, n_warps: int = 0):
    g = W.to_generator(_core, gen)
    return _core.MonteCarloPropagator.from_arrays(
        flat["earliest"], flat["act_idx"], flat["act_duration"], flat["act_type"], flat["target"],
        flat["pred_offsets"], flat["pred_src"], flat["pred_act"], flat["max_delay"], g, n_warps=n_warps)


def _time_batch(props, seed0, ns, reps: int = 2) -> float:
    b = _core.Batch(props, seed0, ns)
    b.run()  # records the graph
    t0 = time.perf_counter()
    for _ in range(reps):
        b.run()
    return (time.perf_counter() - t0) / reps


def tune_warps(flats: list, gens: list, ns: list, candidates=CANDIDATE_WARPS, sample_cap: int = 4096,
               subset: int = 48, use_cache: bool = True) -> int:
    """Warps per CTA for a batch: the fastest candidate on up to `subset` DAGs of
    the batch (spread over its sizes) with samples capped at `sample_cap`."""
    key = shape_class(flats, ns)
    path = _cache_path()
    cache = {}
    if use_cache and os.path.exists(path):
        try:
            with open(path) as f:
                cache = json.load(f)
        except (OSError, ValueError):
            cache = {}
        if key in cache:
            return int(cache[key]["n_warps"])
    idx = np.linspace(0, len(flats) - 1, num=min(subset, len(flats))).astype(int)
    cal_ns = [min(int(ns[i]), sample_cap) for i in idx]
    timings = {}
    for nw in candidates:
        props = [compile_dag(flats[i], gens[i], nw) for i in idx]
        timings[nw] = _time_batch(props, [0] * len(idx), cal_ns)
    best = min(timings, key=timings.get)
    if use_cache:
        cache[key] = {"n_warps": int(best), "seconds": {str(k): v for k, v in timings.items()}}
        try:
            os.makedirs(os.path.dirname(path), exist_ok=True)
            with open(path, "w") as f:
                json.dump(cache, f, indent=1)
        except OSError:
            pass
    return int(best)


class BatchRunner:
    """Compiles a list of (flat DAG, generator, samples, seed0) and runs them as one
    batch; ``n_warps=None`` asks the autotuner."""

    def __init__(self, items: list, n_warps: int | None = None, use_cache: bool = True):
        flats = [it[0] for it in items]
        gens = [it[1] for it in items]
        self.ns = [int(it[2]) for it in items]
        self.seed0 = [int(it[3]) for it in items]
        self.n_warps = n_warps or tune_warps(flats, gens, self.ns, use_cache=use_cache)
        self.props = [compile_dag(f, g, self.n_warps) for f, g in zip(flats, gens)]
        self.batch = _core.Batch(self.props, self.seed0, self.ns)

    def run(self, wait: bool = True) -> None:
        self.batch.run(wait)

    def stats(self, i: int, hist: bool = False) -> dict:
        return self.batch.stats(i, hist)
