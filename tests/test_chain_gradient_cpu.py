"""The CPU chain gradient the adjoint is checked against (test infrastructure):
the level-vectorised form equals the event-by-event definition, on the oracle's
samples, with and without clamping at earliest + max_delay."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from mc_dagprop_gb300 import workloads as W
from mcd_testlib import chain_gradient, chain_gradient_loop


@pytest.mark.parametrize("max_delay", [1800.0, 150.0, 30.0])
def test_vectorised_chain_gradient_equals_definition(max_delay):
    flat, gen = W.config1(seed=41, n_layers=25, width=30)
    flat["max_delay"] = max_delay
    real, dur, cause = oracle.OracleSim(flat, gen).run_many(np.arange(400))
    a = chain_gradient_loop(flat, gen, real, dur, cause)
    b = chain_gradient(flat, gen, real, dur, cause)
    assert a[0] == b[0]
    np.testing.assert_array_equal(a[1], b[1])
    np.testing.assert_allclose(a[2], b[2], rtol=1e-12, atol=0)
    assert (a[1] != 0).any() and (a[2] != 0).any()
