"""PMF constructors (the reference's ``analytic/distributions.py``): constant,
empirical, and exponential / gamma laws discretised on [start, stop] by
differences of their CDF at the grid edges, normalised to unit mass."""
from __future__ import annotations

import math
from typing import Iterable

import numpy as np

from ..types import Second
from ._pmf import DiscretePMF


def constant_pmf(value: Second, step: int) -> DiscretePMF:
    pmf = DiscretePMF.delta(value, step)
    pmf.validate()
    pmf.validate_alignment(step)
    return pmf


def _regularized_gamma(shape: float, x: float) -> float:
    """P(shape, x), the regularized lower incomplete gamma function: its power
    series below shape + 1, the continued fraction of Q above (Numerical Recipes
    6.2), to 1e-12."""
    if shape <= 0.0 or x < 0.0:
        raise ValueError("shape must be > 0 and x >= 0")
    if x == 0.0:
        return 0.0
    lg = math.lgamma(shape)
    if x < shape + 1.0:
        term = total = 1.0 / shape
        a = shape
        for _ in range(200):
            a += 1.0
            term *= x / a
            total += term
            if abs(term) < abs(total) * 1e-12:
                break
        return total * math.exp(-x + shape * math.log(x) - lg)
    tiny = 1e-30
    b = x + 1.0 - shape
    c = 1.0 / tiny
    d = 1.0 / b
    h = d
    for i in range(1, 201):
        an = -i * (i - shape)
        b += 2.0
        d = an * d + b
        d = tiny if abs(d) < tiny else d
        c = b + an / c
        c = tiny if abs(c) < tiny else c
        d = 1.0 / d
        f = d * c
        h *= f
        if abs(f - 1.0) < 1e-12:
            break
    return 1.0 - math.exp(-x + shape * math.log(x) - lg) * h


def _from_cdf(cdf: np.ndarray) -> np.ndarray:
    diffs = np.diff(cdf)
    total = diffs.sum()
    if total == 0.0:
        raise ValueError("zero probability mass in range")
    return diffs / total


def exponential_pmf(scale: Second, step: int, start: int, stop: int) -> DiscretePMF:
    """Exponential law of mean ``scale`` restricted to [start, stop]."""
    if scale <= 0.0:
        raise ValueError("scale must be positive")
    if step <= 0.0:
        raise ValueError("step must be positive")
    if stop < start:
        raise ValueError("stop must be greater or equal to start")
    edges = np.arange(start, stop + step, step)
    pmf = DiscretePMF(edges[:-1], _from_cdf(1.0 - np.exp(-edges / scale)), step=step)
    pmf.validate()
    pmf.validate_alignment(step)
    return pmf


def gamma_pmf(shape: float, scale: Second, step: int, start: Second, stop: Second) -> DiscretePMF:
    """Gamma(shape, scale) restricted to [start, stop]."""
    if shape <= 0.0 or scale <= 0.0:
        raise ValueError("shape and scale must be positive")
    if step <= 0.0:
        raise ValueError("step must be positive")
    if stop < start:
        raise ValueError("stop must be greater or equal to start")
    edges = np.arange(start, stop + step, step)
    cdf = np.array([_regularized_gamma(shape, x / scale) for x in edges])
    pmf = DiscretePMF(edges[:-1], _from_cdf(cdf), step=step)
    pmf.validate()
    pmf.validate_alignment(step)
    return pmf


def empirical_pmf(values: Iterable[Second], weights: Iterable[float], step: int) -> DiscretePMF:
    """PMF at ``values`` with probabilities proportional to ``weights``."""
    v = np.array(list(values), dtype=float)
    w = np.array(list(weights), dtype=float)
    if v.size != w.size:
        raise ValueError("values and weights must have same length")
    if w.sum() <= 0.0:
        raise ValueError("weights must sum to a positive number")
    pmf = DiscretePMF(v, w / w.sum(), step=step)
    pmf.validate()
    pmf.validate_alignment(step)
    return pmf
