"""The reference's PMF and distribution-helper tests (test/test_pmf.py,
test/test_distributions.py), restated against ``import mc_dagprop``: the same
inputs and the same assertions, on the host helpers (no GPU)."""
from __future__ import annotations

import numpy as np

from mc_dagprop.analytic import constant_pmf, empirical_pmf, exponential_pmf, gamma_pmf
from mc_dagprop.analytic._pmf import DiscretePMF


def test_maximum_aligned():
    """test/test_pmf.py:10-15."""
    a = DiscretePMF(np.array([0.0, 1.0]), np.array([0.5, 0.5]), step=1)
    b = DiscretePMF(np.array([0.0, 1.0]), np.array([0.5, 0.5]), step=1)
    r = a.maximum(b)
    assert np.allclose(r.values, [0.0, 1.0])
    assert np.allclose(r.probabilities, [0.25, 0.75])


def test_maximum_tiny_tail_mass_stays_non_negative():
    """test/test_pmf.py:17-25: the smallest subnormal tail."""
    t = 5e-324
    a = DiscretePMF(np.array([0.0, 1.0]), np.array([1.0 - t, t]), step=1)
    b = DiscretePMF(np.array([0.0, 1.0]), np.array([1.0 - t, t]), step=1)
    r = a.maximum(b)
    assert np.all(r.probabilities >= 0.0)
    assert np.isclose(float(r.total_mass), 1.0, rtol=1e-12, atol=1e-15)


def test_convolve_keeps_small_probabilities_exact_in_mass():
    """test/test_pmf.py:27-35: two 256-bin uniforms."""
    p = np.full(256, 1.0 / 256.0)
    a = DiscretePMF(np.arange(256, dtype=float), p, step=1)
    b = DiscretePMF(np.arange(256, dtype=float), p, step=1)
    r = a.convolve(b)
    assert np.isclose(float(r.total_mass), 1.0, rtol=1e-12, atol=1e-15)
    assert np.all(r.probabilities >= 0.0)


def test_constant_pmf():
    """test/test_distributions.py:9-15."""
    pmf = constant_pmf(5.0, step=1)
    pmf.validate()
    pmf.validate_alignment(1.0)
    assert np.allclose(pmf.values, [5.0]) and np.allclose(pmf.probabilities, [1.0])


def test_empirical_pmf():
    """test/test_distributions.py:17-21."""
    pmf = empirical_pmf([0.0, 1.0, 2.0], [1, 1, 2], step=1)
    pmf.validate()
    pmf.validate_alignment(1.0)
    assert abs(pmf.probabilities.sum() - 1.0) < 5e-7


def test_exponential_pmf():
    """test/test_distributions.py:23-29."""
    pmf = exponential_pmf(scale=10.0, step=1, start=0.0, stop=300.0)
    pmf.validate()
    pmf.validate_alignment(1.0)
    assert abs(pmf.probabilities.sum() - 1.0) < 5e-7
    assert pmf.values[0] == 0.0 and pmf.step == 1.0


def test_gamma_pmf():
    """test/test_distributions.py:31-35."""
    pmf = gamma_pmf(shape=2.0, scale=2.0, step=1, start=0.0, stop=20.0)
    pmf.validate()
    pmf.validate_alignment(1.0)
    assert abs(pmf.probabilities.sum() - 1.0) < 5e-7
