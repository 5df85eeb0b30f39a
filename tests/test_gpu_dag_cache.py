"""The compiled-DAG cache: handles created from identical inputs share one device
image; any difference in the inputs (an array element, a generator parameter,
n_warps, the compiler's environment overrides) gives a private compile; an image
outlives the handle that made it while another handle uses it; handles sharing an
image keep their own streams, workspace and error flag."""
from __future__ import annotations

import ctypes as C
import threading

import numpy as np
import pytest

import mc_dagprop_gb300 as m
from mc_dagprop_gb300 import workloads as W
from mcd_testlib import (MCD_OK, DagDesc, DagInfo, DagOptions, last_error, lib, make_desc, make_generator,
                         propagator_from_flat, ptr)

pytestmark = pytest.mark.gpu


def _create(flat, gen, n_warps=0, no_cache=0):
    L = lib()
    L.mcd_dag_create_ex.argtypes = [C.POINTER(DagDesc), C.c_void_p, C.POINTER(DagOptions), C.POINTER(C.c_void_p)]
    d, keep = make_desc(flat)
    g, rc, gkeep = make_generator(gen)
    assert rc == MCD_OK, last_error()
    h = C.c_void_p()
    opts = DagOptions(n_warps, no_cache)
    rc = L.mcd_dag_create_ex(C.byref(d), g, C.byref(opts), C.byref(h))
    L.mcd_generator_destroy(g)
    assert rc == MCD_OK, last_error()
    return h


def _info(h) -> DagInfo:
    i = DagInfo()
    assert lib().mcd_dag_get_info(h, C.byref(i)) == MCD_OK, last_error()
    return i


def _run(h, E, L, seeds):
    n = len(seeds)
    real = np.empty((n, E))
    dur = np.empty((n, L))
    cause = np.empty((n, E), np.int32)
    s = np.ascontiguousarray(seeds, np.int64)
    assert lib().mcd_run_many_host(h, ptr(s), n, ptr(real), ptr(dur), ptr(cause)) == MCD_OK, last_error()
    return real, dur, cause


@pytest.fixture
def dag():
    flat, gen = W.config1(seed=21, n_layers=12, width=30)
    return flat, gen


def test_identical_inputs_share_one_image(cuda, dag):
    flat, gen = dag
    L = lib()
    a = _create(flat, gen)
    b = _create(flat, gen)
    private = _create(flat, gen, no_cache=1)
    try:
        ia, ib, ip = _info(a), _info(b), _info(private)
        assert ia.cache_hit == 0 and ib.cache_hit == 1 and ip.cache_hit == 0
        assert ia.device_bytes == ib.device_bytes == ip.device_bytes
        E, Ln = ia.n_events, ia.n_links
        seeds = np.arange(3000, 3000 + 200)
        ra, da, ca = _run(a, E, Ln, seeds)
        rb, db, cb = _run(b, E, Ln, seeds)
        rp, dp, cp = _run(private, E, Ln, seeds)
        for x, y in ((ra, rb), (da, db), (ra, rp), (da, dp)):
            assert np.array_equal(x.view(np.int64), y.view(np.int64))
        assert np.array_equal(ca, cb) and np.array_equal(ca, cp)
        # the image outlives the handle that compiled it
        L.mcd_dag_destroy(a)
        a = None
        rb2, db2, cb2 = _run(b, E, Ln, seeds)
        assert np.array_equal(rb2.view(np.int64), ra.view(np.int64)) and np.array_equal(cb2, ca)
        c = _create(flat, gen)  # b still holds the image
        assert _info(c).cache_hit == 1
        L.mcd_dag_destroy(c)
    finally:
        for h in (a, b, private):
            if h is not None:
                L.mcd_dag_destroy(h)
    # every handle of these inputs is gone (the private one never was in the cache)
    d = _create(flat, gen)
    assert _info(d).cache_hit == 0
    L.mcd_dag_destroy(d)


def test_any_input_difference_compiles_anew(cuda, dag, monkeypatch):
    flat, gen = dag
    L = lib()
    base = _create(flat, gen)
    made = []
    try:
        def differs(f, g, **kw):
            h = _create(f, g, **kw)
            made.append(h)
            return _info(h).cache_hit == 0

        f2 = dict(flat)
        f2["earliest"] = np.array(flat["earliest"], np.float64)
        f2["earliest"][7] = np.nextafter(f2["earliest"][7], np.inf)  # one ulp
        assert differs(f2, gen)
        f3 = dict(flat)
        f3["pred_src"] = np.array(flat["pred_src"], np.int32)
        f3["pred_act"] = np.array(flat["pred_act"], np.int32)
        last = len(f3["pred_src"]) - 1  # swap the last target's predecessor order
        f3["pred_src"][last - 1:last + 1] = f3["pred_src"][last - 1:last + 1][::-1].copy()
        f3["pred_act"][last - 1:last + 1] = f3["pred_act"][last - 1:last + 1][::-1].copy()
        assert differs(f3, gen)
        assert differs(dict(flat, max_delay=flat["max_delay"] + 1.0), gen)
        g2 = [tuple(s) for s in gen]
        g2[0] = (g2[0][0], g2[0][1], float(g2[0][2]) * 1.5) + tuple(g2[0][3:])
        assert differs(flat, g2)
        assert differs(flat, gen, n_warps=8)
        monkeypatch.setenv("MCD_NO_SMEM_WINDOW", "1")
        assert differs(flat, gen)
        monkeypatch.delenv("MCD_NO_SMEM_WINDOW")
        h = _create(flat, gen)  # the same inputs again: shared
        made.append(h)
        assert _info(h).cache_hit == 1
    finally:
        for h in made:
            L.mcd_dag_destroy(h)
        L.mcd_dag_destroy(base)


def test_sharing_handles_run_concurrently(cuda, dag):
    """Two handles on one image, driven from two threads at once: each keeps its own
    streams and workspace, so both get the results of a lone run."""
    flat, gen = dag
    p1 = propagator_from_flat(m, flat, gen)
    p2 = propagator_from_flat(m, flat, gen)
    assert p2.info()["cache_hit"] and not p1.info()["cache_hit"]
    seeds = [np.arange(0, 6000), np.arange(50_000, 56_000)]
    want = [p1.run_many_arrays(s) for s in seeds]
    got = [None, None]

    def work(k, p):
        for _ in range(3):
            got[k] = p.run_many_arrays(seeds[k])

    ts = [threading.Thread(target=work, args=(0, p1)), threading.Thread(target=work, args=(1, p2))]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    for w, g in zip(want, got):
        for x, y in zip(w[:2], g[:2]):
            assert np.array_equal(np.asarray(x).view(np.int64), np.asarray(y).view(np.int64))
        assert np.array_equal(w[2], g[2])
