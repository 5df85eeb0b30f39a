"""Discrete PMFs on an integer step grid (the reference's ``analytic/_pmf.py``).

``DiscretePMF`` carries the data the GPU engine propagates; its ``convolve`` and
``maximum`` are host utilities for single pairs (the propagation itself runs on
the GPU, ``AnalyticPropagator.run``).  Validation rules and error messages follow
the reference (_pmf.py:26-67) so callers see the same exceptions.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from ..types import ProbabilityMass, Second


def _close(a: float, b: float) -> bool:
    return bool(np.isclose(a, b, rtol=1e-12, atol=1e-15))


@dataclass(frozen=True, slots=True)
class DiscretePMF:
    """Probability mass function on an equidistant grid: ``values`` (sorted,
    spaced by ``step`` seconds, an int) and their ``probabilities``."""

    values: np.ndarray
    probabilities: np.ndarray
    step: int

    def __post_init__(self) -> None:
        self.validate()
        if len(self.values) != len(self.probabilities):
            raise ValueError("values and probs must have same length")
        if self.step < 0.0:
            raise ValueError("step size must be non-negative")
        if not isinstance(self.step, int):
            raise OverflowError(f"step must be an integer number of seconds, got: {self.step} "
                                f"(type: {type(self.step)})")

    def validate(self) -> None:
        if len(self.values) == 0:
            raise ValueError("PMF values cannot be empty")
        if len(self.values) != len(self.probabilities):
            raise ValueError("values and probs must have same length")
        if len(self.values) > 1 and not np.all(self.values[1:] >= self.values[:-1]):
            raise ValueError("values must be sorted in non-decreasing order")
        s = self.probabilities.sum()
        if not (1.0 >= s or np.isclose(s, 1.0)):
            raise ValueError("Probabilities must sum to <= 1.0")

    def validate_alignment(self, step: Second) -> None:
        if not np.isclose(self.step, step):
            raise ValueError(f"PMF step {self.step} does not match expected {step}")
        if step <= 0.0:
            raise ValueError("step must be positive")
        if len(self.values) == 0:
            raise ValueError("PMF values cannot be empty")
        if len(self.values) > 1 and not np.allclose(np.diff(self.values), step):
            raise ValueError("PMF grid spacing does not match step")
        if self.values.size > 0 and not np.isclose(self.values[0] % step, 0.0):
            raise ValueError("PMF values are not aligned to step grid")

    @staticmethod
    def delta(v: Second, step: Second) -> "DiscretePMF":
        return DiscretePMF(np.array([v], dtype=float), np.array([1.0]), step=step)

    @property
    def total_mass(self) -> ProbabilityMass:
        return ProbabilityMass(self.probabilities.sum())

    def shift(self, delta: Second) -> "DiscretePMF":
        return DiscretePMF(self.values + delta, self.probabilities.copy(), step=self.step)

    # host utilities: the same operations the GPU engine applies per event
    def _with_mass(self, values: np.ndarray, probs: np.ndarray, m1: float, m2: float) -> "DiscretePMF":
        expected = 1.0 if _close(m1, 1.0) and _close(m2, 1.0) else m1 * m2
        total = probs.sum()
        if total > 0 and not _close(total, expected):
            probs = probs * (expected / total)
        return DiscretePMF(values, probs, step=self.step)

    def convolve(self, other: "DiscretePMF") -> "DiscretePMF":
        """PMF of X + Y (extended-precision accumulation, then mass correction)."""
        if len(self.values) == 1:
            vals, probs = other.values + self.values[0], other.probabilities * self.probabilities[0]
        elif len(other.values) == 1:
            vals, probs = self.values + other.values[0], self.probabilities * other.probabilities[0]
        else:
            probs = np.convolve(self.probabilities.astype(np.longdouble),
                                other.probabilities.astype(np.longdouble)).astype(float)
            vals = self.values[0] + other.values[0] + self.step * np.arange(len(probs))
        return self._with_mass(vals, probs, float(self.total_mass), float(other.total_mass))

    def maximum(self, other: "DiscretePMF") -> "DiscretePMF":
        """PMF of max(X, Y) from cumulative sums on the common grid."""
        lo = np.minimum(self.values[0], other.values[0])
        hi = np.maximum(self.values[-1], other.values[-1])
        grid = np.arange(lo, hi + self.step, self.step)
        a = np.zeros(len(grid), dtype=np.longdouble)
        b = np.zeros(len(grid), dtype=np.longdouble)
        oa = int(round((self.values[0] - lo) / self.step))
        ob = int(round((other.values[0] - lo) / self.step))
        a[oa:oa + len(self.probabilities)] = self.probabilities
        b[ob:ob + len(other.probabilities)] = other.probabilities
        ca = np.cumsum(a, dtype=np.longdouble)
        cb = np.cumsum(b, dtype=np.longdouble)
        ca_before = np.concatenate((np.zeros(1, dtype=np.longdouble), ca[:-1]))
        probs = (a * cb + b * ca_before).astype(float)
        return self._with_mass(grid, probs, float(self.total_mass), float(other.total_mass))
