"""Seeded synthetic workloads with the shapes of the benchmark configurations.

No public dataset is involved: every DAG is generated from ``numpy.random.
default_rng(seed)`` so the same seed gives the same DAG on every machine.

A DAG is returned in *flat* form, the array image of a ``DagContext``:

    earliest      float64[E]   EventTimestamp.earliest (latest = earliest+600, actual = earliest)
    act_idx       int32[K]     Activity.idx
    act_duration  float64[K]   Activity.minimal_duration
    act_type      int32[K]     Activity.activity_type
    act_src, act_dst int32[K]  the activity map's (src, dst) key
    target        int32[T]     precedence_list targets
    pred_offsets  int64[T+1]   CSR offsets into pred_src / pred_act
    pred_src      int32[P]     predecessor events
    pred_act      int32[P]     activity (link) indices
    max_delay     float

and a generator as a list of ``(kind, activity_type, *params)`` tuples.
"""
from __future__ import annotations

import math

import numpy as np

# Delay generators of the benchmark configurations.
GEN_TWO_TYPES = [("constant", 1, 1.5), ("exponential", 2, 0.1, math.inf)]


def gen_five_types(rng: np.random.Generator) -> list:
    """Five activity types: constant 1.2, exponential (mean 0.05 d), gamma(2, 0.05),
    empirical absolute (16 bins on 0-300 s) and empirical relative (8 bins on 0-0.5),
    the empirical weights drawn from Dirichlet(1)."""
    w16 = rng.dirichlet(np.ones(16))
    w8 = rng.dirichlet(np.ones(8))
    return [
        ("constant", 1, 1.2),
        ("exponential", 2, 0.05, math.inf),
        ("gamma", 3, 2.0, 0.05, math.inf),
        ("empirical_absolute", 4, np.linspace(0.0, 300.0, 16), w16),
        ("empirical_relative", 5, np.linspace(0.0, 0.5, 8), w8),
    ]


def layered_dag(seed: int, n_layers: int, width: int, back: int, types, max_delay: float,
                max_preds: int = 4) -> dict:
    """Layered DAG: event j of layer k has earliest = 60 k + U(0,30) s; each event in
    layer k > 0 takes 1..max_preds predecessors (uniform count) drawn without
    replacement from layers k-back .. k-1 (a uniform random subset, in random
    order); minimal_duration ~ U(30, 300) s; activity types uniform over ``types``."""
    rng = np.random.default_rng(seed)
    E = n_layers * width
    layer = np.repeat(np.arange(n_layers), width)
    earliest = 60.0 * layer + rng.uniform(0.0, 30.0, E)
    counts = np.zeros(E, np.int64)
    counts[width:] = rng.integers(1, max_preds + 1, E - width)
    srcs = []
    for k in range(1, n_layers):
        lo = max(0, k - back) * width
        pool = k * width - lo
        c = np.minimum(counts[k * width:(k + 1) * width], pool)
        counts[k * width:(k + 1) * width] = c
        m = int(min(max_preds, pool))
        # the m smallest of random keys per row: a uniform random m-subset, in random order
        keys = rng.random((width, pool))
        pick = np.argpartition(keys, m - 1, axis=1)[:, :m] if m < pool else np.argsort(keys, axis=1)
        order = np.take_along_axis(keys, pick, axis=1).argsort(axis=1)
        pick = np.take_along_axis(pick, order, axis=1)
        keep = np.arange(pick.shape[1])[None, :] < c[:, None]
        srcs.append(lo + pick[keep])
    pred_src = np.concatenate(srcs).astype(np.int32) if srcs else np.zeros(0, np.int32)
    P = len(pred_src)
    target = np.arange(width, E, dtype=np.int32)
    pred_offsets = np.zeros(len(target) + 1, np.int64)
    pred_offsets[1:] = np.cumsum(counts[width:])
    act_dst = np.repeat(target, counts[width:]).astype(np.int32)
    types = np.asarray(types, np.int32)
    return {
        "earliest": earliest,
        "act_idx": np.arange(P, dtype=np.int32),
        "act_duration": rng.uniform(30.0, 300.0, P),
        "act_type": types[rng.integers(0, len(types), P)],
        "act_src": pred_src.copy(),
        "act_dst": act_dst,
        "target": target,
        "pred_offsets": pred_offsets,
        "pred_src": pred_src,
        "pred_act": np.arange(P, dtype=np.int32),
        "max_delay": float(max_delay),
    }


def layered_dag_fast(rng: np.random.Generator, n_layers: int, width: int, back: int, types, max_delay: float,
                     max_preds: int = 4) -> dict:
    """The distribution of ``layered_dag`` (same layers, earliest times, predecessor
    counts and pools, durations and types), drawn with whole-array operations
    so that a serving benchmark can build a fresh DAG for every request (about a
    millisecond for 4,000 events).  Each event's predecessors are a uniform random subset
    of its pool (Floyd's sampling without replacement, one column per pick)
    in uniformly random order.  It is another random stream than
    ``layered_dag``'s: equal in law, not in values."""
    E = n_layers * width
    layer = np.repeat(np.arange(n_layers), width)
    earliest = 60.0 * layer + rng.uniform(0.0, 30.0, E)
    tl = layer[width:]                                   # layers of the targets (events past layer 0)
    lo = np.maximum(0, tl - back) * width                # first event of each target's pool
    pool = tl * width - lo
    cnt = np.minimum(rng.integers(1, max_preds + 1, len(tl)), pool)
    k = max_preds
    pick = np.full((len(tl), k), -1, np.int64)
    for m in range(k):  # Floyd: for j = pool-cnt .. pool-1, take t in [0, j], or j when t is taken
        live = m < cnt
        j = pool - cnt + m
        t = np.floor(rng.random(len(tl)) * (j + 1)).astype(np.int64)
        taken = (pick[:, :m] == t[:, None]).any(axis=1)
        pick[:, m] = np.where(live, np.where(taken, j, t), -1)
    keys = np.where(pick >= 0, rng.random(pick.shape), 2.0)  # random order, unused slots last
    pick = np.take_along_axis(pick, np.argsort(keys, axis=1), axis=1)
    keep = pick >= 0
    pred_src = (lo[:, None] + pick)[keep].astype(np.int32)
    P = len(pred_src)
    target = np.arange(width, E, dtype=np.int32)
    pred_offsets = np.zeros(len(target) + 1, np.int64)
    pred_offsets[1:] = np.cumsum(cnt)
    types = np.asarray(types, np.int32)
    return {
        "earliest": earliest,
        "act_idx": np.arange(P, dtype=np.int32),
        "act_duration": rng.uniform(30.0, 300.0, P),
        "act_type": types[rng.integers(0, len(types), P)],
        "act_src": pred_src.copy(),
        "act_dst": np.repeat(target, cnt).astype(np.int32),
        "target": target,
        "pred_offsets": pred_offsets,
        "pred_src": pred_src,
        "pred_act": np.arange(P, dtype=np.int32),
        "max_delay": float(max_delay),
    }


def fresh_request(rng: np.random.Generator, ev_lo: int = 200, ev_hi: int = 20_000, s_lo: int = 4_096,
                  s_hi: int = 65_536) -> tuple:
    """One serving request of the serving configuration: a fresh DAG from the
    layered generator with events log-uniform in [ev_lo, ev_hi] (layer width
    log-uniform in 20-200, predecessors from the previous 3 layers), the five
    delay kinds (their empirical weights drawn anew), max_delay 1,800 s, a
    sample count log-uniform in [s_lo, s_hi] and a random seed base.
    Returns (flat, gen, n_samples, seed0)."""
    ev = int(round(math.exp(rng.uniform(math.log(ev_lo), math.log(ev_hi)))))
    width = int(round(math.exp(rng.uniform(math.log(20), math.log(200)))))
    width = max(1, min(width, ev // 2))
    n_layers = max(2, int(round(ev / width)))
    flat = layered_dag_fast(rng, n_layers, width, 3, [1, 2, 3, 4, 5], 1800.0)
    ns = int(round(math.exp(rng.uniform(math.log(s_lo), math.log(s_hi)))))
    return flat, gen_five_types(rng), ns, int(rng.integers(0, 2**40))


def config0(seed: int = 0):
    """1,000 events in 50 layers of 20, predecessors from the previous 1-3 layers,
    types {1: constant 1.5, 2: exponential mean 0.1 d}, max_delay 1800 s;
    run with seeds 0..9999."""
    return layered_dag(seed, 50, 20, 3, [1, 2], 1800.0), list(GEN_TWO_TYPES)


def config1(seed: int = 1, n_layers: int = 2000, width: int = 100):
    """200,000 events in 2,000 layers of 100, predecessors from the previous 1-5
    layers, the five activity types, max_delay 3600 s."""
    rng = np.random.default_rng(seed + 1000)
    return layered_dag(seed, n_layers, width, 5, [1, 2, 3, 4, 5], 3600.0), gen_five_types(rng)


def config3(seed: int = 3):
    """10,000 events (100 layers of 100), the five activity types, max_delay 1800 s."""
    rng = np.random.default_rng(seed + 1000)
    return layered_dag(seed, 100, 100, 3, [1, 2, 3, 4, 5], 1800.0), gen_five_types(rng)


def mixed_dags(seed: int, n_dags: int, ev_lo: int, ev_hi: int, s_lo: int, s_hi: int,
               five_types: bool, fast: bool = False):
    """A stream of DAGs with log-uniform event counts (layer width log-uniform in
    20-200) and log-uniform sample counts; each DAG gets its own seed range.
    fast: draw each DAG with ``layered_dag_fast`` (the same law, another stream)."""
    rng = np.random.default_rng(seed)
    out = []
    seed_base = 0
    for i in range(n_dags):
        ev = int(round(math.exp(rng.uniform(math.log(ev_lo), math.log(ev_hi)))))
        width = int(round(math.exp(rng.uniform(math.log(20), math.log(200)))))
        width = max(1, min(width, ev // 2))
        n_layers = max(2, int(round(ev / width)))
        ns = int(round(math.exp(rng.uniform(math.log(s_lo), math.log(s_hi)))))
        types = [1, 2, 3, 4, 5] if five_types else [1, 2]
        if fast:
            flat = layered_dag_fast(np.random.default_rng(seed * 100003 + i), n_layers, width, 3, types, 1800.0)
        else:
            flat = layered_dag(seed * 100003 + i, n_layers, width, 3, types, 1800.0)
        if five_types:
            gen = gen_five_types(np.random.default_rng(seed * 7919 + i))
        else:
            gen = list(GEN_TWO_TYPES)
        out.append((flat, gen, ns, seed_base))
        seed_base += ns
    return out


def config2(seed: int = 2, n_dags: int = 512, fast: bool = False):
    """512 DAGs, events log-uniform 100-50,000, samples log-uniform 1,000-100,000."""
    return mixed_dags(seed, n_dags, 100, 50_000, 1_000, 100_000, five_types=False, fast=fast)


def config4_requests(seed: int = 4, n_requests: int = 120_000):
    """Serving requests: events log-uniform 200-20,000, samples log-uniform
    4,096-65,536, the five activity types."""
    return mixed_dags(seed, n_requests, 200, 20_000, 4_096, 65_536, five_types=True)


def sample_edges(flat: dict, n_samples: int) -> int:
    """Work units: one (sample, activity) pair per link of the dense activity array."""
    L = int(flat["act_idx"].max()) + 1 if len(flat["act_idx"]) else 0
    return int(n_samples) * L


def to_context(mod, flat: dict):
    """Build a DagContext of ``mod`` (this package or the reference) from flat form."""
    Event, EventTimestamp, Activity, DagContext = mod.Event, mod.EventTimestamp, mod.Activity, mod.DagContext
    e = flat["earliest"]
    events = [Event(str(i), EventTimestamp(float(x), float(x) + 600.0, float(x))) for i, x in enumerate(e)]
    src = flat.get("act_src")
    dst = flat.get("act_dst")
    if src is None:
        src = np.arange(len(flat["act_idx"]))
        dst = src
    acts = {(int(s), int(d)): Activity(int(i), float(du), int(t)) for s, d, i, du, t in
            zip(src, dst, flat["act_idx"], flat["act_duration"], flat["act_type"])}
    off = flat["pred_offsets"]
    prec = [(int(t), [(int(flat["pred_src"][p]), int(flat["pred_act"][p])) for p in range(off[k], off[k + 1])])
            for k, t in enumerate(flat["target"])]
    return DagContext(events, acts, prec, float(flat["max_delay"]))


def to_generator(mod, gen: list):
    g = mod.GenericDelayGenerator()
    for spec in gen:
        kind, t = spec[0], int(spec[1])
        if kind == "constant":
            g.add_constant(t, float(spec[2]))
        elif kind == "exponential":
            g.add_exponential(t, float(spec[2]), float(spec[3]))
        elif kind == "gamma":
            g.add_gamma(t, float(spec[2]), float(spec[3]), float(spec[4]) if len(spec) > 4 else math.inf)
        elif kind == "empirical_absolute":
            g.add_empirical_absolute(t, [float(x) for x in spec[2]], [float(x) for x in spec[3]])
        elif kind == "empirical_relative":
            g.add_empirical_relative(t, [float(x) for x in spec[2]], [float(x) for x in spec[3]])
        else:
            raise ValueError(kind)
    return g
