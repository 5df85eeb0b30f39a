"""``mc_dagprop.monte_carlo`` (reference ``src/mc_dagprop/monte_carlo/__init__.py``):
the GPU Monte Carlo classes; ``mc_dagprop.monte_carlo._core`` names the compiled
module that holds them."""
from __future__ import annotations

import sys

from mc_dagprop_gb300 import _core
from mc_dagprop_gb300.monte_carlo import (  # noqa: F401
    Activity,
    Batch,
    DagContext,
    Event,
    EventTimestamp,
    GenericDelayGenerator,
    MonteCarloPropagator,
    Server,
    SimResult,
    Simulator,
)

sys.modules.setdefault(__name__ + "._core", _core)

__all__ = [
    "GenericDelayGenerator",
    "DagContext",
    "SimResult",
    "Event",
    "Activity",
    "MonteCarloPropagator",
    "Simulator",
    "EventTimestamp",
    "Batch",
    "Server",
]
