"""mcd_stats_device_noalloc: per-event statistics without any device allocation.

Some callers cannot call cudaMalloc: their GPU memory already belongs to another
allocator (for example a framework's caching allocator that has reserved the
device), or an allocation would synchronise the device in the middle of their
latency-critical loop.  For them the library keeps the statistics accumulators
in one fixed 34 MiB device array (DAGs up to MCD_NOALLOC_MAX_EVENTS events).

This test calls the entry point through the C ABI on a freshly created handle,
before anything else ran on that handle, twice in a row (the array keeps the
previous call's contents, so the second call checks that each call starts from
zero), and checks that the device's free memory is the same before and after
those calls (so nothing was allocated behind the caller's back).  It then
compares every output with the allocating entry point mcd_stats_device, run on a
second handle of the same DAG with the same seeds: the statistics are
deterministic (exact integer accumulation), so the tolerance is zero.  It lives in
its own file, collected last, and works alone or after the other tests.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import mc_dagprop_gb300 as m
from mc_dagprop_gb300 import workloads as W
from mcd_testlib import MCD_OK, last_error, lib, propagator_from_flat

pytestmark = pytest.mark.gpu

HIST_STRIDE = 260


class Stats(C.Structure):
    _fields_ = [("mean", C.c_void_p), ("p50", C.c_void_p), ("p90", C.c_void_p), ("p99", C.c_void_p),
                ("p_on_time", C.c_void_p), ("hist", C.c_void_p)]


def _outputs(torch, E, dev):
    t = {k: torch.full((E,), -1.0, dtype=torch.float64, device=dev) for k in ("mean", "p50", "p90", "p99", "pot")}
    t["hist"] = torch.zeros((E, HIST_STRIDE), dtype=torch.int32, device=dev)
    s = Stats(t["mean"].data_ptr(), t["p50"].data_ptr(), t["p90"].data_ptr(), t["p99"].data_ptr(),
              t["pot"].data_ptr(), t["hist"].data_ptr())
    return t, s


def _bind(L):
    L.mcd_stats_device.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_int64, C.POINTER(Stats), C.c_void_p]
    L.mcd_stats_device_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_int64, C.POINTER(Stats),
                                           C.c_void_p]


def test_noalloc_stats_match_allocating_entry_point(cuda):
    import torch

    L = lib()
    _bind(L)
    # Load the kernels this path launches (and look the fixed array up) on a small
    # DAG of the same delay kinds first: a module loaded lazily on its first launch
    # takes device memory, which is not an allocation of the entry point.
    wflat, wgen = W.config1(seed=16, n_layers=4, width=8)
    warm = propagator_from_flat(m, wflat, wgen)
    wout, wout_s = _outputs(torch, warm.node_count(), cuda)
    assert L.mcd_stats_device_noalloc(C.c_void_p(warm._handle()), None, 0, 64, C.byref(wout_s), None) == MCD_OK, \
        last_error()
    assert L.mcd_dag_check(C.c_void_p(warm._handle())) == MCD_OK, last_error()

    flat, gen = W.config1(seed=17, n_layers=60, width=80)
    prop = propagator_from_flat(m, flat, gen)  # a fresh handle: no workspace yet
    h = C.c_void_p(prop._handle())
    E = prop.node_count()
    seeds = torch.arange(3000, dtype=torch.int64, device=cuda) * 7 + 11
    outs = [_outputs(torch, E, cuda) for _ in range(2)]
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info(cuda)[0]
    for out, out_s in outs:  # twice in a row: the fixed array must be cleared by each call
        rc = L.mcd_stats_device_noalloc(h, seeds.data_ptr(), 0, 3000, C.byref(out_s), None)
        assert rc == MCD_OK, last_error()
        assert L.mcd_dag_check(h) == MCD_OK, last_error()
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info(cuda)[0] == free_before, "device memory was allocated"

    # the allocating entry point on a second handle of the same DAG
    prop2 = propagator_from_flat(m, flat, gen)
    h2 = C.c_void_p(prop2._handle())
    ref, ref_s = _outputs(torch, E, cuda)
    assert L.mcd_stats_device(h2, seeds.data_ptr(), 0, 3000, C.byref(ref_s), None) == MCD_OK, last_error()
    assert L.mcd_dag_check(h2) == MCD_OK, last_error()
    for call, (out, _) in enumerate(outs):
        for k in ("mean", "p50", "p90", "p99", "pot", "hist"):
            a, b = out[k].cpu().numpy(), ref[k].cpu().numpy()
            assert np.array_equal(a, b), (call, k)
    assert (ref["hist"].cpu().numpy()[:, :258].sum(axis=1) == 3000).all()


def test_noalloc_rejects_too_many_events(cuda):
    L = lib()
    _bind(L)
    flat, gen = W.config1(seed=18, n_layers=400, width=100)  # 40,000 events
    prop = propagator_from_flat(m, flat, gen)
    s = Stats()
    rc = L.mcd_stats_device_noalloc(C.c_void_p(prop._handle()), None, 0, 64, C.byref(s), None)
    assert rc != MCD_OK and "at most 32000 events" in last_error()
