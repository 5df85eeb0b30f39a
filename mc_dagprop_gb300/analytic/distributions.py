"""PMF constructors of the analytic API (the reference's ``analytic/distributions.py``:
``constant_pmf``, ``empirical_pmf``, ``exponential_pmf``, ``gamma_pmf``).

The discretisation rule is the reference's, so that these helpers give its PMFs:
a continuous law on ``[start, stop]`` is read at the grid edges ``start,
start + step, ...`` (numpy's ``arange(start, stop + step, step)``), bin ``k`` --
placed at edge ``k`` -- holds ``F(edge k+1) - F(edge k)``, and the bins are scaled
to unit mass; an empirical law puts ``weight / sum(weights)`` at each value.
Every PMF leaves through the same two checks of ``DiscretePMF`` (well formed,
aligned to the step).  Argument errors carry the reference's messages.

The CDFs: the exponential law's ``-expm1(-x / scale)``; the gamma law's is
the regularized lower incomplete gamma function ``P(shape, x / scale)``
(``scipy.special.gammainc``).
"""
from __future__ import annotations

from typing import Callable, Iterable

import numpy as np

from ..types import Second
from ._pmf import DiscretePMF


def _checked(values: np.ndarray, probs: np.ndarray, step: int) -> DiscretePMF:
    pmf = DiscretePMF(values, probs, step=step)
    pmf.validate()
    pmf.validate_alignment(step)
    return pmf


def _range_errors(step, start, stop) -> None:
    if step <= 0.0:
        raise ValueError("step must be positive")
    if stop < start:
        raise ValueError("stop must be greater or equal to start")


def _binned(cdf: Callable[[np.ndarray], np.ndarray], step: int, start, stop) -> DiscretePMF:
    """A continuous law on the grid: CDF differences between consecutive edges,
    scaled to unit mass, each bin at its left edge."""
    edges = np.arange(start, stop + step, step)
    mass = np.diff(cdf(edges))
    total = mass.sum()
    if total == 0.0:
        raise ValueError("zero probability mass in range")
    return _checked(edges[:-1], mass / total, step)


def constant_pmf(value: Second, step: int) -> DiscretePMF:
    """All mass at ``value``."""
    return _checked(np.array([value], dtype=float), np.ones(1), step)


def empirical_pmf(values: Iterable[Second], weights: Iterable[float], step: int) -> DiscretePMF:
    """Mass proportional to ``weights`` at ``values``."""
    v = np.fromiter(values, dtype=float)
    w = np.fromiter(weights, dtype=float)
    if len(v) != len(w):
        raise ValueError("values and weights must have same length")
    total = w.sum()
    if total <= 0.0:
        raise ValueError("weights must sum to a positive number")
    return _checked(v, w / total, step)


def exponential_pmf(scale: Second, step: int, start: int, stop: int) -> DiscretePMF:
    """The exponential law of mean ``scale`` restricted to ``[start, stop]``."""
    if scale <= 0.0:
        raise ValueError("scale must be positive")
    _range_errors(step, start, stop)
    return _binned(lambda x: -np.expm1(-x / scale), step, start, stop)


def gamma_pmf(shape: float, scale: Second, step: int, start: Second, stop: Second) -> DiscretePMF:
    """The gamma law of ``shape`` and ``scale`` restricted to ``[start, stop]``."""
    from scipy.special import gammainc

    if shape <= 0.0 or scale <= 0.0:
        raise ValueError("shape and scale must be positive")
    _range_errors(step, start, stop)

    def cdf(x: np.ndarray) -> np.ndarray:
        if (x < 0.0).any():  # the CDF is only defined on x >= 0
            raise ValueError("shape must be > 0 and x >= 0")
        return gammainc(shape, x / scale)

    return _binned(cdf, step, start, stop)
