"""GPU parity: propagation bit-exact against the reference and the oracle.

Given the reference's own durations (golden fixtures) or the oracle's durations,
the CUDA propagation must reproduce realized and cause_event bit for bit.
"""
from __future__ import annotations

import ctypes as C
import math
import os

import numpy as np
import pytest

import mc_dagprop_gb300 as m
import oracle
from mc_dagprop_gb300 import workloads as W
from mcd_testlib import (MCD_OK, flat_from_lists, last_error, lib, load_golden, propagator_from_flat, ptr,
                         six_event_flat)

pytestmark = pytest.mark.gpu


def _bits(a):
    return np.asarray(a, np.float64).view(np.int64)


def assert_bits_equal(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    assert a.shape == b.shape
    bad = np.argwhere(_bits(a) != _bits(b))
    assert len(bad) == 0, f"{len(bad)} mismatches, first {bad[:3].tolist()}: {a[tuple(bad[0])]} vs {b[tuple(bad[0])]}"


@pytest.fixture(params=["smem", "global"])
def window_mode(request, monkeypatch):
    """Both the on-chip window and the global re-read path."""
    if request.param == "global":
        monkeypatch.setenv("MCD_NO_SMEM_WINDOW", "1")
    else:
        monkeypatch.delenv("MCD_NO_SMEM_WINDOW", raising=False)
    return request.param


@pytest.mark.parametrize("name", ["config0_ref.npz", "five_types_ref.npz", "gamma_state_ref.npz"])
def test_given_reference_durations_bitexact(cuda, name, window_mode):
    flat, gen, z = load_golden(name)
    prop = propagator_from_flat(m, flat, gen)
    assert prop.info()["window_in_smem"] == (window_mode == "smem")
    real, cause = prop.propagate(z["durations"])
    assert_bits_equal(real, z["realized"])
    assert np.array_equal(cause, z["cause"])


@pytest.mark.parametrize("warps", ["1", "3", "16"])
def test_given_oracle_durations_bitexact_config0(cuda, warps, monkeypatch):
    monkeypatch.setenv("MCD_WARPS", warps)
    flat, gen = W.config0()
    sim = oracle.OracleSim(flat, gen)
    real_o, dur_o, cause_o = sim.run_many(np.arange(2000), threads=os.cpu_count() or 1)
    prop = propagator_from_flat(m, flat, gen)
    assert prop.info()["n_warps"] == int(warps)
    real, cause = prop.propagate(dur_o)
    assert_bits_equal(real, real_o)
    assert np.array_equal(cause, cause_o)


def test_given_durations_device_capi(cuda):
    """The device entry point, sample-minor buffers with a padded leading dimension."""
    import torch

    flat, gen, z = load_golden("config0_ref.npz")
    prop = propagator_from_flat(m, flat, gen)
    h = C.c_void_p(prop._handle())
    S, E, L = z["durations"].shape[0], prop.node_count(), prop.activity_count()
    ld = 64
    dur = torch.zeros((L, ld), dtype=torch.float64, device=cuda)
    dur[:, :S] = torch.from_numpy(np.ascontiguousarray(z["durations"].T)).to(cuda)
    real = torch.full((E, ld), -7.0, dtype=torch.float64, device=cuda)
    cause = torch.full((E, ld), -7, dtype=torch.int32, device=cuda)
    torch.cuda.synchronize()
    rc = lib().mcd_propagate_device(h, dur.data_ptr(), ld, S, real.data_ptr(), cause.data_ptr(), ld, None)
    assert rc == MCD_OK, last_error()
    assert lib().mcd_dag_check(h) == MCD_OK, last_error()
    r = real.cpu().numpy()
    assert_bits_equal(r[:, :S].T, z["realized"])
    assert np.array_equal(cause.cpu().numpy()[:, :S].T, z["cause"])
    assert (r[:, S:] == -7.0).all()  # padding untouched


def _edge_flats():
    yield six_event_flat()
    yield flat_from_lists([0.0, 0.0, 0.0, 0.0], {(0, 3): (0, 5.0, 9), (1, 3): (1, 5.0, 9), (2, 3): (2, 5.0, 9)},
                          [(3, [(0, 0), (1, 1), (2, 2)])], 1e6)
    yield flat_from_lists(
        [math.nan, -0.0, math.inf, 0.0, -math.inf, 3.0, 1.0],
        {(0, 3): (0, 1.0, 1), (1, 3): (2, -0.0, 9), (2, 5): (5, 1.0, 1), (3, 5): (6, 2.0, 2), (4, 6): (7, 1.0, 1),
         (1, 6): (9, 0.0, 9)},
        [(3, [(0, 0), (1, 2)]), (5, [(2, 5), (3, 6)]), (6, [(4, 7), (1, 9)])], 1e6)
    yield flat_from_lists([0.0, 1.0, 2.0], {(0, 1): (0, 10.0, 1), (1, 2): (1, 10.0, 1)},
                          [(1, [(0, 0)]), (2, [(1, 1)])], 0.0)
    yield flat_from_lists([0.0, 1.0, 2.0], {(0, 1): (0, 10.0, 1), (1, 2): (1, 10.0, 1)},
                          [(1, [(0, 0)]), (2, [(1, 1)])], math.nan)
    yield W.layered_dag(5, 30, 7, 4, [1, 2], 50.0)
    # longer predecessor lists (the given-durations kernel reads them four at a
    # time): up to 11 per event, and one event with 37
    yield W.layered_dag(6, 20, 12, 3, [1, 2], 80.0, max_preds=11)
    yield flat_from_lists([0.0] * 38, {(k, 37): (k, 1.0 + k % 3, 1) for k in range(37)},
                          [(37, [(k, k) for k in range(37)])], 1e6)


def test_given_special_values_bitexact(cuda, window_mode):
    """NaN / +-inf / -0 / negative durations, ties, zero and NaN max_delay; long
    predecessor lists."""
    rng = np.random.default_rng(11)
    specials = np.array([math.nan, math.inf, -math.inf, -0.0, 0.0, -5.0, 1e308, 5e-324, 3.0])
    for flat in _edge_flats():
        sim = oracle.OracleSim(flat, [])
        prop = propagator_from_flat(m, flat, [])
        n, L = 300, sim.activity_count()
        dur = rng.uniform(0.0, 40.0, (n, L)).round(0)  # rounding makes ties frequent
        mask = rng.random((n, L)) < 0.15
        dur[mask] = rng.choice(specials, mask.sum())
        real_o, cause_o = sim.propagate_given(dur)
        real, cause = prop.propagate(dur)
        assert_bits_equal(real, real_o)
        assert np.array_equal(cause, cause_o)


def test_chain_10000_known_answer(cuda):
    """test/test_simulator.py:175-212 (chain of 10,000 events, constant delays, threads)."""
    from concurrent.futures import ThreadPoolExecutor
    from itertools import chain

    n = 10_000
    events = [m.Event(str(i), m.EventTimestamp(float(i), 100.0 + i, 0.0)) for i in range(n)]
    links = {(i, i + 1): m.Activity(idx=i, minimal_duration=3.0, activity_type=1) for i in range(n - 1)}
    prec = [(i, [(i - 1, i)]) for i in range(1, n)]
    ctx = m.DagContext(events=events, activities=links, precedence_list=prec, max_delay=1e6)
    gen = m.GenericDelayGenerator()
    gen.add_constant(activity_type=1, factor=1.0)
    sim = m.Simulator(ctx, gen)
    res = sim.run(seed=7)
    assert len(res.realized) == 10000 and len(res.durations) == 9999 and len(res.cause_event) == 10000
    assert res.realized[0] == 0.0 and res.realized[9999] == 59988.0
    sims = [m.Simulator(ctx, gen) for _ in range(4)]
    seeds = [[i + j for i in range(1000)] for j in range(4)]
    with ThreadPoolExecutor(max_workers=4) as pool:
        results = list(chain.from_iterable(pool.map(lambda a: a[0].run_many(a[1]), zip(sims, seeds))))
    assert len(results) == 4000
    for r in results[::97]:
        assert len(r.realized) == 10000 and len(r.durations) == 9999 and len(r.cause_event) == 10000
        assert r.realized[9999] == 59988.0


def test_sampled_outputs_are_a_propagation_of_their_durations(cuda):
    """realized/cause of a sampled run == propagation of that run's durations (bit-exact)."""
    for flat, gen in (W.config0(), W.config1(seed=3, n_layers=40, width=60)):
        prop = propagator_from_flat(m, flat, gen)
        seeds = np.arange(-500, 1500, dtype=np.int64) * 7919
        real, dur, cause = prop.run_many_arrays(seeds)
        real2, cause2 = prop.propagate(dur)
        assert_bits_equal(real, real2)
        assert np.array_equal(cause, cause2)
        # and the oracle's propagation of the same durations
        ro, co = oracle.OracleSim(flat, gen).propagate_given(dur)
        assert_bits_equal(real, ro)
        assert np.array_equal(cause, co)


def test_sample_keying_is_position_independent(cuda):
    """A sample's result depends on its seed only, not on batch, chunk or position."""
    flat, gen = W.config1(seed=4, n_layers=20, width=50)
    prop = propagator_from_flat(m, flat, gen)
    seeds = np.array([5, 17, -3, 2**40 + 1, 99, 5], dtype=np.int64)
    real, dur, cause = prop.run_many_arrays(seeds)
    for i, s in enumerate(seeds):
        r1, d1, c1 = prop.run_many_arrays(np.array([s]))
        assert_bits_equal(r1[0], real[i])
        assert_bits_equal(d1[0], dur[i])
    assert_bits_equal(real[0], real[5])


def test_simresult_views_like_reference(cuda):
    """SimResult properties are writable zero-copy numpy views owned by the result
    (_core.cpp:491-516); the buffer protocol exposes realized."""
    flat, gen = W.config0()
    prop = propagator_from_flat(m, flat, gen)
    res = prop.run_many([1, 2, 3])
    r = res[1]
    a = r.realized
    assert a.dtype == np.float64 and a.shape == (prop.node_count(),) and a.flags.writeable
    assert a.base is r
    assert r.durations.dtype == np.float64 and r.durations.shape == (prop.activity_count(),)
    assert r.cause_event.dtype == np.int32
    assert np.array_equal(np.asarray(memoryview(r)), r.realized)
    solo = prop.run(2)
    assert_bits_equal(solo.realized, r.realized)
    assert_bits_equal(solo.durations, r.durations)
    assert np.array_equal(solo.cause_event, r.cause_event)
    with pytest.raises(TypeError):
        prop.run_many([2**31])  # seeds are C ints, as in the reference


def test_large_sample_counts_chunk_correctly(cuda):
    """More samples than one host chunk: results must equal per-chunk runs."""
    flat, gen = W.config1(seed=9, n_layers=200, width=100)
    prop = propagator_from_flat(m, flat, gen)
    seeds = np.arange(1200, dtype=np.int64)
    real, _, cause = prop.run_many_arrays(seeds, durations=False)
    r2, _, c2 = prop.run_many_arrays(seeds[1000:], durations=False)
    assert_bits_equal(real[1000:], r2)
    assert np.array_equal(cause[1000:], c2)


def _pinned(nbytes):
    p = C.c_void_p()
    assert lib().mcd_host_alloc(nbytes, C.byref(p)) == MCD_OK, last_error()
    return p


def test_host_paths_pinned_and_pageable_agree(cuda):
    """The host-buffer entry points over several chunks: pinned buffers (written and
    read by the transpose kernels directly) and pageable buffers (staged copies)
    give the same bits, and a sample's result does not depend on its chunk."""
    flat, gen = W.config1(seed=5, n_layers=20, width=50)
    prop = propagator_from_flat(m, flat, gen)
    h = C.c_void_p(prop._handle())
    E, L = prop.node_count(), prop.activity_count()
    n = 32 * 152 + 1000  # more than two half-wave chunks on a 152-SM part
    seeds = np.arange(7, 7 + n, dtype=np.int64)
    real = np.empty((n, E)); dur = np.empty((n, L)); cause = np.empty((n, E), np.int32)
    assert lib().mcd_run_many_host(h, ptr(seeds), n, ptr(real), ptr(dur), ptr(cause)) == MCD_OK, last_error()
    bufs = [_pinned(n * 8), _pinned(n * E * 8), _pinned(n * L * 8), _pinned(n * E * 4)]
    try:
        ps = np.ctypeslib.as_array(C.cast(bufs[0], C.POINTER(C.c_int64)), (n,))
        pr = np.ctypeslib.as_array(C.cast(bufs[1], C.POINTER(C.c_double)), (n, E))
        pd = np.ctypeslib.as_array(C.cast(bufs[2], C.POINTER(C.c_double)), (n, L))
        pc = np.ctypeslib.as_array(C.cast(bufs[3], C.POINTER(C.c_int32)), (n, E))
        ps[:] = seeds
        pr.fill(-1.0); pd.fill(-1.0); pc.fill(-9)
        assert lib().mcd_run_many_host(h, bufs[0], n, bufs[1], bufs[2], bufs[3]) == MCD_OK, last_error()
        assert_bits_equal(pr, real)
        assert_bits_equal(pd, dur)
        assert np.array_equal(pc, cause)
        # propagation of the pinned durations, written into pinned outputs
        pr.fill(-1.0); pc.fill(-9)
        assert lib().mcd_propagate_host(h, bufs[2], n, bufs[1], bufs[3]) == MCD_OK, last_error()
        assert_bits_equal(pr, real)
        assert np.array_equal(pc, cause)
    finally:
        for b in bufs:
            lib().mcd_host_free(b)
    r2, d2, c2 = prop.run_many_arrays(seeds[-700:])
    assert_bits_equal(r2, real[-700:])
    assert_bits_equal(d2, dur[-700:])
    assert np.array_equal(c2, cause[-700:])


def test_host_paths_mixed_pinned_pageable_and_absent_outputs(cuda):
    """One call with a pinned, a pageable and an absent output (the chunk buffers then
    hold sample-major staging rows too), over several chunks of the two-stream
    pipeline, gives the bits of the all-pageable call."""
    flat, gen = W.config1(seed=6, n_layers=16, width=40)
    prop = propagator_from_flat(m, flat, gen)
    h = C.c_void_p(prop._handle())
    E, L = prop.node_count(), prop.activity_count()
    n = 32 * 152 * 2 + 77  # five half-wave chunks on a 152-SM part
    seeds = np.arange(100, 100 + n, dtype=np.int64)
    real = np.empty((n, E)); dur = np.empty((n, L)); cause = np.empty((n, E), np.int32)
    assert lib().mcd_run_many_host(h, ptr(seeds), n, ptr(real), ptr(dur), ptr(cause)) == MCD_OK, last_error()
    bufs = [_pinned(n * E * 8), _pinned(n * L * 8)]
    try:
        pr = np.ctypeslib.as_array(C.cast(bufs[0], C.POINTER(C.c_double)), (n, E))
        pd = np.ctypeslib.as_array(C.cast(bufs[1], C.POINTER(C.c_double)), (n, L))
        pr.fill(-1.0)
        d_pageable = np.full((n, L), -1.0)
        assert lib().mcd_run_many_host(h, ptr(seeds), n, bufs[0], ptr(d_pageable), None) == MCD_OK, last_error()
        assert_bits_equal(pr, real)
        assert_bits_equal(d_pageable, dur)
        # given pageable durations into a pinned realized row set and a pageable cause
        pd[:] = dur
        pr.fill(-1.0)
        c_pageable = np.full((n, E), -9, np.int32)
        assert lib().mcd_propagate_host(h, ptr(dur), n, bufs[0], ptr(c_pageable)) == MCD_OK, last_error()
        assert_bits_equal(pr, real)
        assert np.array_equal(c_pageable, cause)
        # given pinned durations into pageable outputs
        r_pageable = np.full((n, E), -1.0)
        assert lib().mcd_propagate_host(h, bufs[1], n, ptr(r_pageable), None) == MCD_OK, last_error()
        assert_bits_equal(r_pageable, real)
    finally:
        for b in bufs:
            lib().mcd_host_free(b)
