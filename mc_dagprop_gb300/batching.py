"""Batched runs of many DAGs in persistent launches, with a small autotuner.

A ``Batch`` compiles every DAG with the same number of warps per CTA (the CTA
size of its persistent launch) and runs all (DAG, 32-sample tile) work items in
one CUDA graph.  The warps per CTA trade work per stage against barrier and idle
time: wide DAGs want many warps, narrow ones few (and more CTAs per SM); where
the propagation window lives trades shared memory (fewer CTAs per SM) against
global-memory reads of predecessor times.
``BatchRunner`` therefore splits a mixed stream into width classes -- by the
warps the compiler would pick for each DAG alone -- and each width class by the
CTAs per SM its DAGs' shared-memory layouts allow (a launch runs at the
occupancy of its largest layout, so one wide window would otherwise throttle
every narrow DAG of the batch).  It runs one batch per class, all launched
together on their own streams so their CTAs share the SMs.  For each width
class ``tune_class`` times every (warps per CTA, window place) candidate on a
calibration subset and keeps the fastest; results are cached per shape class in
a JSON file (``$MCD_AUTOTUNE_CACHE``, default
``~/.cache/mc_dagprop_gb300/autotune.json``).  Samples per warp (32, one per
lane) and the work item ((DAG, 32-sample tile): a tile's levels run in order, so
cutting it into level blocks would not shorten it) are fixed by the kernel's
design, not tuned.
"""
from __future__ import annotations

import json
import math
import os
import time

import numpy as np

from . import _core
from . import workloads as W

CANDIDATE_WARPS = (4, 8, 12, 24)
# warps per CTA tried for each width class: block sizes that divide the 24 warps
# an SM holds at the batch kernel's register count
CLASS_CANDIDATES = {4: (2, 4, 8), 8: (4, 8, 12), 12: (6, 12, 24), 24: (12, 24)}


def _cache_path() -> str:
    return os.environ.get("MCD_AUTOTUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "mc_dagprop_gb300", "autotune.json"))


def shape_class(flats: list, ns: list, widths: list | None = None) -> str:
    """Coarse key of a batch: log2 of the mean events, mean level width and mean samples."""
    ev = np.mean([len(f["earliest"]) for f in flats])
    if widths is None:
        widths = [len(f["earliest"]) / max(1, _levels(f)) for f in flats]
    width = np.mean(widths)
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


def compile_dag(flat: dict, gen: list, n_warps: int = 0, window: str = "auto"):
    """Propagator of a flat DAG (n_warps: warps per CTA, 0 automatic; window:
    "auto" keeps the propagation window in shared memory when it fits, "global"
    in global rows)."""
    g = W.to_generator(_core, gen)
    return _core.MonteCarloPropagator.from_arrays(
        flat["earliest"], flat["act_idx"], flat["act_duration"], flat["act_type"], flat["target"],
        flat["pred_offsets"], flat["pred_src"], flat["pred_act"], flat["max_delay"], g, n_warps=n_warps,
        window=window)


def width_class(auto_warps: int) -> int:
    """Width class of a DAG from the warps the compiler picks for it alone."""
    return 4 if auto_warps <= 4 else 8 if auto_warps <= 8 else 12 if auto_warps <= 12 else 24


def _time_batch(props, seed0, ns, reps: int = 2) -> float:
    b = _core.Batch(props, seed0, ns)
    b.run()  # records the graph
    t0 = time.perf_counter()
    for _ in range(reps):
        b.run()
    return (time.perf_counter() - t0) / reps


WINDOW_CANDIDATES = ("auto", "global")


def tune_class(flats: list, gens: list, ns: list, candidates=CANDIDATE_WARPS, windows=WINDOW_CANDIDATES,
               sample_cap: int = 4096, subset: int = 48, use_cache: bool = True,
               widths: list | None = None) -> tuple:
    """(warps per CTA, window place) for a batch: the fastest candidate pair on up
    to `subset` DAGs of the batch (spread over its sizes) with samples capped at
    `sample_cap`.  Returns (n_warps, window, seconds per candidate)."""
    key = ("w" + "-".join(str(c) for c in candidates) + ":p" + "-".join(windows) + ":" +
           shape_class(flats, ns, widths))
    path = _cache_path()
    cache = {}
    if use_cache and os.path.exists(path):
        try:
            with open(path) as f:
                cache = json.load(f)
        except (OSError, ValueError):
            cache = {}
        if key in cache and "window" in cache[key]:
            return int(cache[key]["n_warps"]), str(cache[key]["window"]), cache[key]["seconds"]
    idx = np.linspace(0, len(flats) - 1, num=min(subset, len(flats))).astype(int)
    cal_ns = [min(int(ns[i]), sample_cap) for i in idx]
    timings = {}
    for nw in candidates:
        for win in windows:
            props = [compile_dag(flats[i], gens[i], nw, win) for i in idx]
            timings[f"{nw}/{win}"] = _time_batch(props, [0] * len(idx), cal_ns)
    best = min(timings, key=timings.get)
    nw, win = best.split("/")
    if use_cache:
        cache[key] = {"n_warps": int(nw), "window": win, "seconds": timings}
        try:
            os.makedirs(os.path.dirname(path), exist_ok=True)
            with open(path, "w") as f:
                json.dump(cache, f, indent=1)
        except OSError:
            pass
    return int(nw), win, timings


def tune_warps(flats: list, gens: list, ns: list, candidates=CANDIDATE_WARPS, sample_cap: int = 4096,
               subset: int = 48, use_cache: bool = True, widths: list | None = None) -> int:
    """Warps per CTA alone (the window where it fits): tune_class over warps."""
    return tune_class(flats, gens, ns, candidates, ("auto",), sample_cap, subset, use_cache, widths)[0]


class BatchRunner:
    """Compiles a list of (flat DAG, generator, samples, seed0) and runs them as one
    batch per width class (``n_warps`` given: a single batch with that many warps;
    ``tune=True``: each class's warps from the autotuner)."""

    def __init__(self, items: list, n_warps: int | None = None, tune: bool = True, use_cache: bool = True):
        flats = [it[0] for it in items]
        gens = [it[1] for it in items]
        self.ns = [int(it[2]) for it in items]
        self.seed0 = [int(it[3]) for it in items]
        window = {}         # width class -> window place chosen by the tuner
        self.tuning = {}    # width class -> seconds per "warps/window" candidate
        if n_warps:
            classes = {n_warps: list(range(len(items)))}
            warps = {n_warps: n_warps}
        else:
            classes = {}
            widths = []
            for i, (f, g) in enumerate(zip(flats, gens)):
                info = compile_dag(f, g).info()
                widths.append(info["n_events"] / max(1, info["n_levels"]))
                classes.setdefault(width_class(info["n_warps"]), []).append(i)
            warps = {}
            for c, idx in classes.items():
                cand = CLASS_CANDIDATES[c]
                if tune:
                    nw, win, secs = tune_class([flats[i] for i in idx], [gens[i] for i in idx],
                                               [self.ns[i] for i in idx], candidates=cand, use_cache=use_cache,
                                               widths=[widths[i] for i in idx])
                    warps[c] = nw
                    window[c] = win
                    self.tuning[c] = secs
                else:
                    warps[c] = c
        self.props = [None] * len(items)
        self.where = {}
        self.batches = []
        for c in sorted(classes):
            nw = warps[c]
            groups = {}
            for i in classes[c]:
                p = compile_dag(flats[i], gens[i], nw, window.get(c, "auto"))
                self.props[i] = p
                groups.setdefault(_core.Batch.occupancy(nw, p.info()["smem_bytes"]), []).append(i)
            for per_sm in sorted(groups, reverse=True):
                idx = groups[per_sm]
                for j, i in enumerate(idx):
                    self.where[i] = (len(self.batches), j)
                self.batches.append((nw, per_sm, idx, _core.Batch([self.props[i] for i in idx],
                                                                  [self.seed0[i] for i in idx],
                                                                  [self.ns[i] for i in idx])))

        self.window = window

    @property
    def classes(self) -> list:
        """(warps per CTA, CTAs per SM, DAG count, work items) of each class batch."""
        return [(w, per_sm, len(idx), b.items) for w, per_sm, idx, b in self.batches]

    def run(self, wait: bool = True) -> None:
        for *_, b in self.batches:  # one launch per class, all in flight together
            b.run(False)
        if wait:
            self.sync()

    def sync(self) -> None:
        for *_, b in self.batches:
            b.sync()

    def stats(self, i: int, hist: bool = False) -> dict:
        k, j = self.where[i]
        return self.batches[k][3].stats(j, hist)
