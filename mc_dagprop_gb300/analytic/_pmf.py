"""Discrete PMFs on an equidistant integer grid (the reference's public
``DiscretePMF``, ``analytic/_pmf.py``).

``DiscretePMF`` carries what the GPU engine propagates.  Its construction checks
and their messages are the reference's (_pmf.py:26-67), because callers match on
them.  ``convolve`` and ``maximum`` are host utilities for one pair of PMFs (the
propagation itself runs on the GPU, ``AnalyticPropagator.run``); both work on the
operands' common integer grid in extended precision, as the GPU fold does:

* the sum of two variables is the discrete convolution of their masses, which
  starts at the sum of their first values;
* the maximum of two independent variables has the CDF ``F_a * F_b``, so its
  masses are the increments of that product on the grid spanning both operands.

A result then carries the mass its operands imply -- exactly 1 when both are
normalised (rounding drift is scaled away), else the product of their masses
-- and is rescaled only when its sum strays from that by more than 1e-12
relative (1e-15 absolute), the reference's tolerance.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from ..types import ProbabilityMass, Second

_RTOL, _ATOL = 1e-12, 1e-15


def _near(x: float, y: float) -> bool:
    return bool(np.isclose(x, y, rtol=_RTOL, atol=_ATOL))


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
        """Non-empty, equal lengths, sorted values, total mass at most 1."""
        v, p = self.values, self.probabilities
        if len(v) == 0:
            raise ValueError("PMF values cannot be empty")
        if len(v) != len(p):
            raise ValueError("values and probs must have same length")
        if len(v) > 1 and not (np.diff(v) >= 0).all():  # NaN fails too
            raise ValueError("values must be sorted in non-decreasing order")
        total = p.sum()
        if not total <= 1.0 and not np.isclose(total, 1.0):  # NaN fails too
            raise ValueError("Probabilities must sum to <= 1.0")

    def validate_alignment(self, step: Second) -> None:
        """Values spaced by ``step`` and on its grid."""
        if not np.isclose(self.step, step):
            raise ValueError(f"PMF step {self.step} does not match expected {step}")
        if step <= 0.0:
            raise ValueError("step must be positive")
        v = self.values
        if len(v) == 0:
            raise ValueError("PMF values cannot be empty")
        if len(v) > 1 and not np.allclose(np.diff(v), step):
            raise ValueError("PMF grid spacing does not match step")
        if not np.isclose(v[0] % step, 0.0):
            raise ValueError("PMF values are not aligned to step grid")

    @staticmethod
    def delta(v: Second, step: Second) -> "DiscretePMF":
        """Unit mass at ``v``."""
        return DiscretePMF(np.array([v], dtype=float), np.ones(1), step=step)

    @property
    def total_mass(self) -> ProbabilityMass:
        return ProbabilityMass(self.probabilities.sum())

    def shift(self, delta: Second) -> "DiscretePMF":
        return DiscretePMF(self.values + delta, self.probabilities.copy(), step=self.step)

    # ------------------------------------------------------------ host utilities
    def _implied_mass(self, other: "DiscretePMF") -> float:
        ma, mb = float(self.total_mass), float(other.total_mass)
        return 1.0 if _near(ma, 1.0) and _near(mb, 1.0) else ma * mb

    def _result(self, first: float, probs: np.ndarray, mass: float) -> "DiscretePMF":
        probs = np.asarray(probs, dtype=float)
        total = probs.sum()
        if total > 0 and not _near(total, mass):
            probs = probs * (mass / total)
        return DiscretePMF(first + self.step * np.arange(len(probs)), probs, step=self.step)

    def convolve(self, other: "DiscretePMF") -> "DiscretePMF":
        """PMF of X + Y for independent X ~ self, Y ~ other."""
        q = np.longdouble
        probs = np.convolve(self.probabilities.astype(q), other.probabilities.astype(q))
        return self._result(self.values[0] + other.values[0], probs, self._implied_mass(other))

    def maximum(self, other: "DiscretePMF") -> "DiscretePMF":
        """PMF of max(X, Y) for independent X ~ self, Y ~ other."""
        lo = min(self.values[0], other.values[0])
        hi = max(self.values[-1], other.values[-1])
        n = len(np.arange(lo, hi + self.step, self.step))
        cdf = np.ones(n, dtype=np.longdouble)
        for pmf in (self, other):
            k = int(round((pmf.values[0] - lo) / self.step))  # the operand's first grid point
            col = np.zeros(n, dtype=np.longdouble)
            col[k:k + len(pmf.probabilities)] = pmf.probabilities
            cdf *= np.cumsum(col)
        probs = np.diff(cdf, prepend=np.longdouble(0.0))  # a monotone product: no negative increments
        return self._result(lo, probs, self._implied_mass(other))
