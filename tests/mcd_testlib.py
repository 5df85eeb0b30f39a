"""Test helpers: ctypes bindings of the C ABI, fixture loading, DAG builders."""
from __future__ import annotations

import ctypes as C
import json
import os
import re

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "mc_dagprop_gb300.h")
LIB = os.path.join(ROOT, "mc_dagprop_gb300", "_lib", "libmcdagprop_gb300.so")
GOLDEN = os.path.join(ROOT, "tests", "golden")

MCD_OK, MCD_ERR_INVALID, MCD_ERR_RUNTIME, MCD_ERR_CUDA, MCD_ERR_NOMEM, MCD_ERR_DEVICE = 0, 1, 2, 3, 4, 5


class DagDesc(C.Structure):
    _fields_ = [("n_events", C.c_int32), ("earliest", C.c_void_p), ("n_activities", C.c_int32),
                ("act_idx", C.c_void_p), ("act_duration", C.c_void_p), ("act_type", C.c_void_p),
                ("n_targets", C.c_int32), ("target", C.c_void_p), ("pred_offsets", C.c_void_p),
                ("pred_src", C.c_void_p), ("pred_act", C.c_void_p), ("max_delay", C.c_double)]


class DagInfo(C.Structure):
    _fields_ = [("n_events", C.c_int32), ("n_links", C.c_int32), ("n_levels", C.c_int32), ("n_warps", C.c_int32),
                ("n_preds", C.c_int64), ("window_slots", C.c_int32), ("window_in_smem", C.c_int32),
                ("n_orphan_links", C.c_int32), ("device", C.c_int32), ("device_bytes", C.c_int64),
                ("n_stages", C.c_int32), ("smem_bytes", C.c_int32), ("positive", C.c_int32),
                ("tables_in_smem", C.c_int32), ("cache_hit", C.c_int32), ("n_event_pairs", C.c_int32),
                ("block_draws", C.c_int64)]


class DagOptions(C.Structure):
    _fields_ = [("n_warps", C.c_int32), ("no_cache", C.c_int32), ("window", C.c_int32)]


def header_functions() -> list[str]:
    """Names of every function the public header declares."""
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(mcd_[a-z0-9_]+)\s*\(", src)))


_lib = None


def lib():
    global _lib
    if _lib is None:
        L = C.CDLL(LIB)
        P, I64, I32, D = C.c_void_p, C.c_int64, C.c_int32, C.c_double
        L.mcd_last_error.restype = C.c_char_p
        L.mcd_generator_create.argtypes = [C.POINTER(P)]
        L.mcd_generator_destroy.argtypes = [P]
        L.mcd_generator_set_seed.argtypes = [P, I64]
        L.mcd_generator_add_constant.argtypes = [P, I32, D]
        L.mcd_generator_add_exponential.argtypes = [P, I32, D, D]
        L.mcd_generator_add_gamma.argtypes = [P, I32, D, D, D]
        L.mcd_generator_add_empirical_absolute.argtypes = [P, I32, P, I64, P, I64]
        L.mcd_generator_add_empirical_relative.argtypes = [P, I32, P, I64, P, I64]
        L.mcd_dag_create.argtypes = [C.POINTER(DagDesc), P, C.POINTER(P)]
        L.mcd_dag_destroy.argtypes = [P]
        L.mcd_dag_node_count.argtypes = [P]
        L.mcd_dag_activity_count.argtypes = [P]
        L.mcd_dag_get_info.argtypes = [P, C.POINTER(DagInfo)]
        L.mcd_dag_describe.argtypes = [C.POINTER(DagDesc), P, C.POINTER(DagInfo)]
        L.mcd_dag_stream.argtypes = [P]
        L.mcd_dag_stream.restype = P
        L.mcd_run_many_host.argtypes = [P, P, I64, P, P, P]
        L.mcd_propagate_host.argtypes = [P, P, I64, P, P]
        L.mcd_run_device.argtypes = [P, P, I64, P, P, P, I64, P]
        L.mcd_propagate_device.argtypes = [P, P, I64, I64, P, P, I64, P]
        L.mcd_dag_check.argtypes = [P]
        L.mcd_host_alloc.argtypes = [C.c_size_t, C.POINTER(P)]
        L.mcd_host_free.argtypes = [P]
        _lib = L
    return _lib


def last_error() -> str:
    return lib().mcd_last_error().decode()


def ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def make_generator(gen: list):
    """C-ABI generator from a list of (kind, type, *params) tuples; returns (handle, rc, keepalive)."""
    L = lib()
    h = C.c_void_p()
    assert L.mcd_generator_create(C.byref(h)) == MCD_OK
    keep = []
    for spec in gen:
        kind, t = spec[0], int(spec[1])
        if kind == "constant":
            rc = L.mcd_generator_add_constant(h, t, float(spec[2]))
        elif kind == "exponential":
            rc = L.mcd_generator_add_exponential(h, t, float(spec[2]), float(spec[3]))
        elif kind == "gamma":
            rc = L.mcd_generator_add_gamma(h, t, float(spec[2]), float(spec[3]),
                                           float(spec[4]) if len(spec) > 4 else float("inf"))
        else:
            v = np.ascontiguousarray(spec[2], np.float64)
            w = np.ascontiguousarray(spec[3], np.float64)
            keep += [v, w]
            fn = L.mcd_generator_add_empirical_absolute if kind == "empirical_absolute" else \
                L.mcd_generator_add_empirical_relative
            rc = fn(h, t, ptr(v), len(v), ptr(w), len(w))
        if rc != MCD_OK:
            return h, rc, keep
    return h, MCD_OK, keep


def make_desc(flat: dict):
    arrs = {
        "earliest": np.ascontiguousarray(flat["earliest"], np.float64),
        "act_idx": np.ascontiguousarray(flat["act_idx"], np.int32),
        "act_duration": np.ascontiguousarray(flat["act_duration"], np.float64),
        "act_type": np.ascontiguousarray(flat["act_type"], np.int32),
        "target": np.ascontiguousarray(flat["target"], np.int32),
        "pred_offsets": np.ascontiguousarray(flat["pred_offsets"], np.int64),
        "pred_src": np.ascontiguousarray(flat["pred_src"], np.int32),
        "pred_act": np.ascontiguousarray(flat["pred_act"], np.int32),
    }
    d = DagDesc(len(arrs["earliest"]), ptr(arrs["earliest"]), len(arrs["act_idx"]), ptr(arrs["act_idx"]),
                ptr(arrs["act_duration"]), ptr(arrs["act_type"]), len(arrs["target"]), ptr(arrs["target"]),
                ptr(arrs["pred_offsets"]), ptr(arrs["pred_src"]), ptr(arrs["pred_act"]), float(flat["max_delay"]))
    return d, arrs


def describe(flat: dict, gen: list, env: dict | None = None):
    """Host-only compile of a flat DAG: (status, DagInfo, message)."""
    import os as _os

    old = {}
    for k, v in (env or {}).items():
        old[k] = _os.environ.get(k)
        _os.environ[k] = v
    try:
        gh, rc, keep = make_generator(gen)
        assert rc == MCD_OK
        d, arrs = make_desc(flat)
        info = DagInfo()
        rc = lib().mcd_dag_describe(C.byref(d), gh, C.byref(info))
        msg = last_error()
        lib().mcd_generator_destroy(gh)
        return rc, info, msg
    finally:
        for k, v in old.items():
            if v is None:
                _os.environ.pop(k, None)
            else:
                _os.environ[k] = v


def load_golden(name: str):
    z = np.load(os.path.join(GOLDEN, name))
    flat = {k: z[k] for k in ("earliest", "act_idx", "act_duration", "act_type", "act_src", "act_dst", "target",
                              "pred_offsets", "pred_src", "pred_act")}
    flat["max_delay"] = float(z["max_delay"])
    gen = [tuple([g[0], g[1]] + [np.asarray(p) if isinstance(p, list) else p for p in g[2:]])
           for g in json.loads(str(z["gen"]))]
    return flat, gen, z


def block_digests(rows: np.ndarray, block: int = 100) -> np.ndarray:
    """8-byte BLAKE2b digest of the raw bytes of each block of `block` consecutive
    rows (sample-major: one row per seed), as uint64 -- how the golden fixture
    config0_hashes_ref.npz pins the reference's full 10,000-seed run."""
    import hashlib

    rows = np.ascontiguousarray(rows)
    out = np.empty((len(rows) + block - 1) // block, np.uint64)
    for i in range(len(out)):
        h = hashlib.blake2b(rows[i * block:(i + 1) * block].tobytes(), digest_size=8)
        out[i] = np.frombuffer(h.digest(), np.uint64)[0]
    return out


def flat_from_lists(earliest, links, precedence, max_delay):
    """Flat DAG from python lists: links = {(src,dst): (idx, duration, type)}."""
    act_src = np.array([k[0] for k in links], np.int32)
    act_dst = np.array([k[1] for k in links], np.int32)
    vals = list(links.values())
    off = [0]
    src, act = [], []
    for _, preds in precedence:
        for s, a in preds:
            src.append(s)
            act.append(a)
        off.append(len(src))
    return {
        "earliest": np.asarray(earliest, np.float64),
        "act_idx": np.array([v[0] for v in vals], np.int32),
        "act_duration": np.array([v[1] for v in vals], np.float64),
        "act_type": np.array([v[2] for v in vals], np.int32),
        "act_src": act_src, "act_dst": act_dst,
        "target": np.array([t for t, _ in precedence], np.int32),
        "pred_offsets": np.array(off, np.int64),
        "pred_src": np.array(src, np.int32),
        "pred_act": np.array(act, np.int32),
        "max_delay": float(max_delay),
    }


def propagator_from_flat(mod, flat, gen):
    from mc_dagprop_gb300 import workloads as W

    g = W.to_generator(mod, gen)
    return mod.MonteCarloPropagator.from_arrays(flat["earliest"], flat["act_idx"], flat["act_duration"],
                                                flat["act_type"], flat["target"], flat["pred_offsets"],
                                                flat["pred_src"], flat["pred_act"], flat["max_delay"], g)


# The 6-event DAG of the reference's test_simulator.py:11-35.
def six_event_flat():
    earliest = [0.0, 5.0, 10.0, 22.0, 20.0, 100.0]
    links = {(0, 1): (0, 3.0, 1), (1, 2): (1, 5.0, 1), (1, 3): (2, 5.0, 1), (2, 4): (3, 15.0, 2),
             (3, 4): (4, 10.0, 3)}
    prec = [(1, [(0, 0)]), (2, [(1, 1)]), (3, [(1, 2)]), (4, [(2, 3), (3, 4)])]
    return flat_from_lists(earliest, links, prec, 1e6)


def event_levels(flat: dict) -> np.ndarray:
    """Level of every event (longest path from a source) of a DAG whose
    precedence targets come in topological order (the layered generators')."""
    lvl = np.zeros(len(flat["earliest"]), np.int64)
    off, src = flat["pred_offsets"], flat["pred_src"]
    for k, t in enumerate(flat["target"]):
        if off[k + 1] > off[k]:
            lvl[t] = lvl[src[off[k]:off[k + 1]]].max() + 1
    return lvl


def _link_tables(flat: dict, gen: list, L: int):
    """Per link: base duration, how its d(duration)/d(base) is formed (1: the
    sampled factor duration / base -- exponential, gamma, relative tables; 2:
    1 + factor -- constants; 0: 1 -- absolute tables and unmapped types), and the
    constant factor."""
    base = np.zeros(L)
    code = np.zeros(L, np.int8)
    factor = np.zeros(L)
    types = {g[1]: g for g in gen}
    for i, d, t in zip(flat["act_idx"], flat["act_duration"], flat["act_type"]):
        base[i] = d
        spec = types.get(int(t), ("none",))
        if spec[0] in ("exponential", "gamma", "empirical_relative"):
            code[i] = 1
        elif spec[0] == "constant":
            code[i] = 2
            factor[i] = spec[2]
    return base, code, factor


def chain_gradient(flat: dict, gen: list, real: np.ndarray, dur: np.ndarray, cause: np.ndarray):
    """CPU pathwise gradient of J = mean_s sum_e (realized - earliest) from the
    samples' realized times, durations and cause_event (the winning predecessor of
    the reference's propagation loop, _core.cpp:331-350): a sample's derivative
    flows back along its winning chain with slope 1 while the winner is not
    clamped at earliest + max_delay.  Levels are walked from the last to the
    first, all events of a level at once.  Assumes distinct predecessors per event
    (the layered generators').  Returns (objective, grad_earliest, grad_base)."""
    S, E = real.shape
    L = dur.shape[1]
    earliest = np.asarray(flat["earliest"], np.float64)
    ub = earliest + flat["max_delay"]
    off = np.asarray(flat["pred_offsets"])
    tgt = np.asarray(flat["target"])
    ev_of = np.repeat(tgt, np.diff(off))  # the event each precedence entry belongs to
    src = np.asarray(flat["pred_src"], np.int64)
    link = np.asarray(flat["pred_act"], np.int64)
    lvl = event_levels(flat)
    delayed = real > earliest[None, :]
    cnt = np.zeros((E, S), np.int64)  # event-major for np.add.at over rows
    ge = np.zeros(E, np.int64)
    gl = np.zeros(L)
    entry_lvl = lvl[ev_of]
    base, code, factor = _link_tables(flat, gen, L)
    for lv in range(int(lvl.max()), -1, -1):
        evs = np.flatnonzero(lvl == lv)
        c = cnt[evs] + delayed[:, evs].T  # (events of the level, S)
        ent = np.flatnonzero(entry_lvl == lv)
        e_ent = ev_of[ent]
        pos = np.searchsorted(evs, e_ent)  # row of each entry's event in c
        win = cause[:, e_ent].T == src[ent][:, None]  # (entries, S)
        valid = link[ent] < L
        dsum = np.where(valid[:, None], dur[:, np.minimum(link[ent], L - 1)].T, 0.0)
        clamped = win & (real[:, src[ent]].T + dsum > ub[e_ent][:, None])
        flow = win & ~clamped
        won = np.zeros((len(evs), S), bool)
        np.logical_or.at(won, pos, flow)
        ge[evs] = np.where(won, 0, c).sum(axis=1) - delayed[:, evs].sum(axis=0)
        contrib = np.where(flow, c[pos], 0)
        np.add.at(cnt, src[ent], contrib)
        ok = valid & flow.any(axis=1)
        if ok.any():  # d(duration)/d(base) as the GPU records it, in float32
            lk = link[ent][ok]
            sampled = (dur[:, lk] / base[lk]).astype(np.float32).astype(np.float64).T
            fixed = np.where(code[lk] == 2, np.float32(1.0) + factor[lk].astype(np.float32), np.float32(1.0))
            dfac = np.where((code[lk] == 1)[:, None], sampled, fixed.astype(np.float64)[:, None])
            np.add.at(gl, lk, (contrib[ok] * dfac).sum(axis=1))
    obj = (real - earliest[None, :]).sum(axis=1).mean()
    return obj, ge / S, gl / S


def chain_gradient_loop(flat, gen, real, dur, cause):
    """chain_gradient written event by event (the definition, for small DAGs)."""
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
        for src, l in pl:
            sel = ce == src
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


def kitchen_sink(seed: int = 3, n_layers: int = 60, width: int = 120, big_table: bool = False,
                 max_preds: int = 4):
    """A layered DAG drawing on every sampler path: constant, truncated
    exponential, Erlang shapes 1 (truncated: redraws), 2 and 3, Marsaglia-Tsang
    shapes 2.5 (truncated) and 0.5, empirical tables with per-link duration
    tables (16 bins) and without them (40 and 300 bins), a type with no
    distribution; links referenced by two entries, entries past the last link
    (duration 0) and links no entry references.  big_table: the 300-bin table
    becomes 5,000 bins (two random words per draw; the tables block then lives
    in global memory).  max_preds: predecessors per event, 1 to max_preds."""
    import numpy as np

    from mc_dagprop_gb300 import workloads as W

    rng = np.random.default_rng(seed)
    flat = W.layered_dag(seed, n_layers, width, 3, list(range(1, 12)), 600.0, max_preds=max_preds)
    P = len(flat["pred_act"])
    pa = flat["pred_act"].copy()
    k = np.arange(100, P)
    dup = k[rng.random(len(k)) < 0.05]
    pa[dup] = pa[dup - 50]                    # a link read by two entries
    extra = 20                                # activities no entry references
    past = np.arange(200, P, 997)
    pa[past] = P + extra + 100                # past the last link: duration 0
    flat["pred_act"] = pa.astype(np.int32)
    flat["act_idx"] = np.arange(P + extra, dtype=np.int32)
    flat["act_duration"] = np.concatenate([flat["act_duration"], rng.uniform(30.0, 300.0, extra)])
    flat["act_type"] = np.concatenate([flat["act_type"], rng.integers(1, 12, extra)]).astype(np.int32)
    nb = 5000 if big_table else 300
    gen = [
        ("constant", 1, 0.3),
        ("exponential", 2, 0.05, 0.2),
        ("gamma", 3, 2.0, 0.05, float("inf")),
        ("gamma", 4, 2.5, 0.04, 0.5),
        ("gamma", 5, 0.5, 0.1, float("inf")),
        ("gamma", 6, 1.0, 0.1, 0.15),
        ("gamma", 7, 3.0, 0.02, float("inf")),
        ("empirical_absolute", 8, np.linspace(0.0, 300.0, 16), rng.dirichlet(np.ones(16))),
        ("empirical_relative", 9, np.linspace(0.0, 0.8, 40), rng.dirichlet(np.ones(40))),
        ("empirical_absolute", 10, np.linspace(0.0, 600.0, nb), rng.dirichlet(np.ones(nb))),
    ]  # type 11: no distribution (fixed at its base)
    return flat, gen
