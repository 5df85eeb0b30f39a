"""Failure detection without a GPU fault: every wait in the kernels has a poll
limit, after which it latches an error flag and the kernel returns.  The test
makes a wait run out (a barrier phase that no copy completes) and checks that the
flag is latched, the kernel ran to its end, and the context still runs work."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import mc_dagprop_gb300 as m
import oracle
from mc_dagprop_gb300 import workloads as W
from mcd_testlib import MCD_OK, last_error, lib, propagator_from_flat

pytestmark = pytest.mark.gpu


def test_bounded_wait_gives_up_and_context_stays_usable(cuda):
    L = lib()
    L.mcd_selftest_bounded_wait.argtypes = [C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
    timed_out, returned = C.c_int32(-1), C.c_int32(-1)
    assert L.mcd_selftest_bounded_wait(C.byref(timed_out), C.byref(returned)) == MCD_OK, last_error()
    assert timed_out.value == 1 and returned.value == 1
    # the same process and context keep running kernels, with correct results
    flat, gen = W.config0()
    prop = propagator_from_flat(m, flat, gen)
    real, dur, cause = prop.run_many_arrays(np.arange(256, dtype=np.int64))
    ro, co = oracle.OracleSim(flat, gen).propagate_given(dur)
    assert np.array_equal(real.view(np.int64), ro.view(np.int64)) and np.array_equal(cause, co)
