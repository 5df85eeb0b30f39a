"""Per-type delay inspection on the GPU (the reference's demo/inspection.py:11-29).

The reference lists, for every activity type, the delays ``durations[idx] -
minimal_duration`` of all activities of that type (and the delays relative to
the base, for non-zero bases) over a set of results, then plots their
histograms.  ``delay_histograms`` computes those histograms directly on the
device over n samples (``mcd_delay_histograms``): the durations never leave the
GPU.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_LIB = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib", "libmcdagprop_gb300.so")
_lib = None


def _api():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB):
            raise ImportError(f"mc_dagprop_gb300.inspection requires the compiled library {_LIB}")
        L = C.CDLL(_LIB)
        P = C.c_void_p
        L.mcd_last_error.restype = C.c_char_p
        L.mcd_delay_histograms.argtypes = [P, P, C.c_int64, P, P, C.c_int32, C.c_int32, P, P, P]
        _lib = L
    return _lib


def _links(activities, n_links: int):
    """(class per link, base per link, sorted types) from a DagContext's activity map
    or the flat arrays (act_idx, act_duration, act_type)."""
    if isinstance(activities, dict) and "act_idx" in activities:
        idx = np.asarray(activities["act_idx"])
        dur = np.asarray(activities["act_duration"], float)
        typ = np.asarray(activities["act_type"])
    else:
        acts = list(activities.values())
        idx = np.array([a.idx for a in acts])
        dur = np.array([a.minimal_duration for a in acts], float)
        typ = np.array([a.activity_type for a in acts])
    types = sorted(set(int(t) for t in typ))
    cls = np.full(n_links, -1, np.int32)
    base = np.zeros(n_links)
    pos = {t: i for i, t in enumerate(types)}
    for i, d, t in zip(idx, dur, typ):
        if 0 <= i < n_links:
            cls[i] = pos[int(t)]
            base[i] = d
    return cls, base, types


def delay_histograms(propagator, activities, seeds, bins: int = 64, ranges: dict | None = None):
    """Histograms of absolute and relative delays per activity type over the
    samples of ``seeds`` (int64).  ``activities``: the DagContext's activity map, or
    flat arrays {act_idx, act_duration, act_type}.  ``ranges``: {type: (abs_lo,
    abs_hi, rel_lo, rel_hi)}; types left out get the range of a pilot run of up to
    256 samples (the same seeds).  Returns {type: {"absolute": {...}, "relative":
    {...}}}, each with "counts" (bins), "edges" (bins + 1), "under", "over",
    "count", "mean" and "var"."""
    seeds = np.ascontiguousarray(seeds, dtype=np.int64)
    L = propagator.activity_count()
    cls, base, types = _links(activities, L)
    nc = len(types)
    rng = np.zeros((nc, 4))
    missing = [c for c, t in enumerate(types) if not ranges or t not in ranges]
    if missing:
        _, dur, _ = propagator.run_many_arrays(seeds[:256])
        for c in missing:
            sel = cls == c
            d = dur[:, sel] - base[sel]
            b = base[sel]
            rel = (d / np.where(b != 0.0, b, 1.0))[:, b != 0.0]
            a_lo, a_hi = (float(d.min()), float(d.max())) if d.size else (0.0, 1.0)
            r_lo, r_hi = (float(rel.min()), float(rel.max())) if rel.size else (0.0, 1.0)
            pad_a, pad_r = max(1e-9, 1e-6 * (a_hi - a_lo)), max(1e-9, 1e-6 * (r_hi - r_lo))
            rng[c] = (a_lo, a_hi + pad_a, r_lo, r_hi + pad_r)
    for c, t in enumerate(types):
        if ranges and t in ranges:
            rng[c] = ranges[t]
    counts = np.zeros((nc, 2, bins + 2), np.uint64)
    moments = np.zeros((nc, 2, 3))
    p = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    rc = _api().mcd_delay_histograms(C.c_void_p(propagator._handle()), p(seeds), len(seeds), p(cls), p(base), nc,
                                     bins, p(rng), p(counts), p(moments))
    if rc != 0:
        raise (ValueError if rc == 1 else RuntimeError)(_api().mcd_last_error().decode())
    out = {}
    for c, t in enumerate(types):
        entry = {}
        for k, name in ((0, "absolute"), (1, "relative")):
            cnt, s, s2 = moments[c, k]
            mean = s / cnt if cnt else float("nan")
            entry[name] = {"counts": counts[c, k, 1:bins + 1].copy(), "under": int(counts[c, k, 0]),
                           "over": int(counts[c, k, bins + 1]),
                           "edges": np.linspace(rng[c, 2 * k], rng[c, 2 * k + 1], bins + 1), "count": int(cnt),
                           "mean": mean, "var": s2 / cnt - mean * mean if cnt else float("nan")}
        out[t] = entry
    return out
