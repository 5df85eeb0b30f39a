"""C-ABI boundary and API surface, without a GPU.

The library must load and export every function the public header declares;
all validation happens in the host DAG compiler before any CUDA call, so the
reference's error cases (test/test_monte_carlo_extra.py:60-92) are checked here.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import math

import numpy as np
import pytest

import mc_dagprop_gb300 as m
from mcd_testlib import (MCD_ERR_INVALID, MCD_ERR_RUNTIME, MCD_OK, flat_from_lists, header_functions, last_error,
                         lib, make_desc, make_generator, six_event_flat)


def test_library_exports_every_header_symbol():
    names = header_functions()
    assert len(names) >= 20
    L = C.CDLL(lib()._name)
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_abi_version_and_last_error():
    L = lib()
    L.mcd_abi_version.restype = C.c_int
    assert L.mcd_abi_version() == 4
    assert isinstance(last_error(), str)


def _create(flat, gen):
    L = lib()
    gh, rc, keep = make_generator(gen)
    if rc != MCD_OK:
        L.mcd_generator_destroy(gh)
        return rc, last_error()
    d, arrs = make_desc(flat)
    h = C.c_void_p()
    rc = L.mcd_dag_create(C.byref(d), gh, C.byref(h))
    msg = last_error()
    L.mcd_generator_destroy(gh)
    if rc == MCD_OK:
        L.mcd_dag_destroy(h)
    return rc, msg


def _three():
    return flat_from_lists([0.0, 0.0, 0.0], {(0, 1): (0, 1.0, 1), (1, 2): (1, 2.0, 1)},
                           [(1, [(0, 0)]), (2, [(1, 1)])], 1e6)


def test_reference_runtime_errors_via_capi():
    cyc = flat_from_lists([0.0, 0.0], {(0, 1): (0, 1.0, 1), (1, 0): (1, 1.0, 1)}, [(1, [(0, 0)]), (0, [(1, 1)])], 1e6)
    rc, msg = _create(cyc, [("constant", 1, 0.0)])
    assert rc == MCD_ERR_RUNTIME and msg == "Invalid DAG: cycle detected in precedence list"
    rc, msg = _create(_three(), [("constant", -1, 0.0)])
    assert rc == MCD_ERR_RUNTIME and msg == "Activity type -1 is reserved for no delay"
    neg = dict(_three(), max_delay=-1.0)
    rc, msg = _create(neg, [("constant", 1, 0.0)])
    assert rc == MCD_ERR_RUNTIME and msg == "max_delay must be non-negative"
    rc, msg = _create(_three(), [("empirical_absolute", 1, [1.0, 2.0], [1.0])])
    assert rc == MCD_ERR_RUNTIME and "same length" in msg


@pytest.mark.parametrize("gen,frag", [
    ([("exponential", 1, 1.0, -1.0)], "max_scale"),
    ([("exponential", 1, -1.0, 1.0)], "lambda_"),
    ([("gamma", 1, 2.0, 1.0, 0.0)], "max_scale"),
    ([("gamma", 1, 0.0, 1.0)], "shape"),
    ([("empirical_absolute", 1, [], [])], "at least one"),
    ([("empirical_relative", 1, [1.0, 2.0], [0.0, 0.0])], "zero"),
    ([("empirical_relative", 1, [1.0, 2.0], [1.0, -1.0])], "non-negative"),
])
def test_non_terminating_or_undefined_parameters_rejected(gen, frag):
    """Parameters for which the reference's loops never end, or that are
    undefined behaviour there, are rejected up front."""
    rc, msg = _create(_three(), gen)
    assert rc == MCD_ERR_INVALID and frag in msg


def test_index_validation():
    f = _three()
    bad = dict(f, pred_src=np.array([0, 7], np.int32))
    assert _create(bad, [])[0] == MCD_ERR_INVALID
    dup = flat_from_lists([0.0, 0.0, 0.0], {(0, 2): (0, 1.0, 1), (1, 2): (1, 2.0, 1)},
                          [(2, [(0, 0)]), (2, [(1, 1)])], 1e6)
    rc, msg = _create(dup, [])
    assert rc == MCD_ERR_INVALID and "twice" in msg
    negact = dict(f, pred_act=np.array([0, -1], np.int32))
    assert _create(negact, [])[0] == MCD_ERR_INVALID


def test_python_errors_and_types():
    ev = [m.Event("0", m.EventTimestamp(0.0, 100.0, 0.0)), m.Event("1", m.EventTimestamp(0.0, 100.0, 0.0))]
    acts = {(0, 1): m.Activity(idx=0, minimal_duration=1.0, activity_type=1),
            (1, 0): m.Activity(idx=1, minimal_duration=1.0, activity_type=1)}
    ctx = m.DagContext(events=ev, activities=acts, precedence_list=[(1, [(0, 0)]), (0, [(1, 1)])], max_delay=1e6)
    g = m.GenericDelayGenerator()
    g.add_constant(1, 0.0)
    with pytest.raises(RuntimeError, match="cycle detected"):
        m.Simulator(ctx, g)
    g2 = m.GenericDelayGenerator()
    g2.add_constant(-1, 0.0)
    with pytest.raises(RuntimeError, match="reserved"):
        m.Simulator(ctx, g2)
    with pytest.raises(RuntimeError, match="same length"):
        g.add_empirical_relative(2, [1.0, 2.0], [1.0])


def test_api_surface_matches_reference():
    """Names, aliases, dataclass behaviour and reprs of _core.pyi / _core.cpp:366-552."""
    assert m.MonteCarloPropagator.__name__ == "MonteCarloPropagator"
    assert m.Simulator is m.MonteCarloPropagator
    from mc_dagprop_gb300 import core, monte_carlo, types

    assert monte_carlo.Simulator is m.MonteCarloPropagator
    assert core.DagContext is m.DagContext
    assert types.Second.__name__ == "Second"
    ts = m.EventTimestamp(1.0, 2.0, 3.0)
    assert dataclasses.is_dataclass(ts)
    assert repr(ts) == "EventTimestamp(earliest=1.0, latest=2.0, actual=3.0)"
    with pytest.raises(dataclasses.FrozenInstanceError):
        ts.earliest = 5.0
    assert ts == m.EventTimestamp(1.0, 2.0, 3.0) and hash(ts) == hash(m.EventTimestamp(1.0, 2.0, 3.0))
    e = m.Event("a", ts)
    assert repr(e) == "Event(event_id='a', timestamp=EventTimestamp(earliest=1.0, latest=2.0, actual=3.0))"
    a = m.Activity(idx=3, minimal_duration=2.5, activity_type=7)
    assert (a.idx, a.minimal_duration, a.activity_type) == (3, 2.5, 7)
    assert repr(a) == "Activity(idx=3, minimal_duration=2.5, activity_type=7)"
    ctx = m.DagContext(events=(e,), activities={(0, 0): a}, precedence_list=((0, ()),), max_delay=10.0)
    assert ctx.max_delay == 10.0 and ctx.activities[(0, 0)] == a and ctx.precedence_list == [(0, [])]
    gen = m.GenericDelayGenerator()
    gen.set_seed(3)
    gen.add_gamma(1, 2.0, 0.5)  # max_scale defaults to inf
    gen.add_exponential(activity_type=2, lambda_=1.0, max_scale=math.inf)
    gen.add_empirical_absolute(activity_type=3, values=np.array([1.0, 2.0]), weights=[1, 1])


def test_reference_and_workload_generators_agree_on_shapes():
    from mc_dagprop_gb300 import workloads as W

    flat, gen = W.config0()
    assert len(flat["earliest"]) == 1000
    assert 2000 < len(flat["act_idx"]) < 3000
    flat1, gen1 = W.config1(n_layers=20)
    assert len(flat1["earliest"]) == 2000 and len(gen1) == 5
    f6 = six_event_flat()
    assert list(f6["target"]) == [1, 2, 3, 4]


def test_compiler_layout_decisions():
    """Host compile of the benchmark DAG shapes: window on chip, staged records,
    shared memory within the per-CTA limit, positive-time fast path."""
    from mc_dagprop_gb300 import workloads as W
    from mcd_testlib import describe

    for flat, gen in (W.config0(), W.config1(n_layers=200)):
        rc, info, msg = describe(flat, gen)
        assert rc == MCD_OK, msg
        assert info.window_in_smem == 1 and info.positive == 1 and info.tables_in_smem == 1
        assert info.n_stages >= info.n_levels
        assert 0 < info.smem_bytes <= 227 * 1024
        assert info.window_slots * 256 < info.smem_bytes
        assert info.device == -1
    # a window too large for shared memory falls back to global rows, staging stays on
    flat = W.layered_dag(3, 6, 1500, 1, [1], 10.0)
    rc, info, msg = describe(flat, [("constant", 1, 1.0)])
    assert rc == MCD_OK and info.window_in_smem == 0 and info.window_slots >= 1500
    assert info.n_stages > info.n_levels  # wide levels are split into stages
    # negative times disable the positive fast path
    f6 = six_event_flat()
    f6["earliest"] = f6["earliest"] - 50.0
    rc, info, msg = describe(f6, [("constant", 1, 1.0)])
    assert rc == MCD_OK and info.positive == 0
    # an event with more predecessors than a staging buffer holds
    n = 2000
    big = flat_from_lists([0.0] * (n + 1), {(i, n): (i, 1.0, 1) for i in range(n)}, [(n, [(i, i) for i in range(n)])], 1e6)
    rc, info, msg = describe(big, [("constant", 1, 1.0)])
    assert rc == MCD_OK and info.n_levels == 2
    # distribution tables beyond 16 KB stay in global memory (the kTablesGlobal kernels)
    vals = np.arange(1000, dtype=np.float64)
    rc, info, msg = describe(W.config0()[0], [("empirical_absolute", 1, vals, np.ones(1000)), ("constant", 2, 0.5)])
    assert rc == MCD_OK and info.tables_in_smem == 0
    rc, info, msg = describe(W.config0()[0], [("empirical_absolute", 1, vals[:100], np.ones(100)), ("constant", 2, 0.5)])
    assert rc == MCD_OK and info.tables_in_smem == 1


def _block_draws_per_event(flat: dict, gen: list) -> float:
    """Philox blocks per event when every event is its own work unit: the links an
    event references first share blocks of four words in predecessor order (one
    word for exponential and small tables, shape-k Erlang gamma k words), other
    random links draw blocks of their own.  A restatement of the compiler's rule
    without event pairs, for the five-kind layered DAGs (each link referenced once)."""
    words = {"exponential": 1, "empirical_absolute": 1, "empirical_relative": 1}
    per_type = {}
    for g in gen:
        if g[0] == "gamma":
            per_type[g[1]] = int(g[2]) if float(g[2]) in (1.0, 2.0, 3.0) else -1
        else:
            per_type[g[1]] = words.get(g[0], 0)
    draws = 0
    off, act, typ = flat["pred_offsets"], flat["pred_act"], flat["act_type"]
    for k in range(len(flat["target"])):
        used = None
        for a in act[off[k]:off[k + 1]]:
            w = per_type.get(int(typ[a]), 0)
            if w < 0:
                draws += 1
            elif w > 0:
                if used is None or used + w > 4:
                    draws += 1
                    used = 0
                used += w
    return draws / len(flat["earliest"])


def test_event_pairs_share_philox_blocks():
    """The compiler runs pairs of events of one level whose draws fit one block of
    four words back to back on one warp, so they draw one block between them: on
    the five-kind benchmark shape the blocks a sample draws fall by about 30 %
    against one unit per event, and the fixed-duration DAG draws none."""
    from mc_dagprop_gb300 import workloads as W
    from mcd_testlib import describe

    flat, gen = W.config1(n_layers=200)
    rc, info, msg = describe(flat, gen)
    assert rc == MCD_OK, msg
    E = info.n_events
    single = _block_draws_per_event(flat, gen)
    assert 1.0 < single < 1.1
    assert info.n_event_pairs > 0.3 * E
    assert info.block_draws / E < 0.75 * single
    # the units depend on the levels alone: the same under other warps per CTA and
    # with the window in global rows (other stage splits)
    for env in ({"MCD_WARPS": "3"}, {"MCD_NO_SMEM_WINDOW": "1"}):
        rc, other, msg = describe(flat, gen, env=env)
        assert rc == MCD_OK, msg
        assert (other.n_warps, other.window_in_smem, other.n_stages) != (info.n_warps, info.window_in_smem,
                                                                         info.n_stages)
        assert (other.n_event_pairs, other.block_draws) == (info.n_event_pairs, info.block_draws)
    rc, info, msg = describe(flat, [("constant", t, 1.0) for t in range(1, 6)])
    assert rc == MCD_OK and info.block_draws == 0 and info.n_event_pairs == 0


def test_serving_stream_compiles():
    """500 requests of the serving stream (fresh layered DAGs of 200-20,000 events,
    five delay kinds) compile on the host -- event pairs, stages and the layout
    check of every compile included -- and most of them pair events."""
    from mc_dagprop_gb300 import workloads as W
    from mcd_testlib import describe

    rng = np.random.default_rng(4)
    paired = 0
    for _ in range(500):
        flat, gen, _, _ = W.fresh_request(rng)
        rc, info, msg = describe(flat, gen)
        assert rc == MCD_OK, msg
        assert 2 * info.n_event_pairs <= info.n_events and info.block_draws <= info.n_preds
        paired += info.n_event_pairs > 0
    assert paired > 400
