"""``mc_dagprop`` under its own name, served by the GB300 engine.

Callers of the reference write ``import mc_dagprop`` / ``from mc_dagprop import
Simulator`` / ``from mc_dagprop.monte_carlo import ...`` / ``mc_dagprop.types``
(reference ``src/mc_dagprop/__init__.py:5-49``); this package answers those
imports with the objects of ``mc_dagprop_gb300``, whose Monte Carlo and analytic
engines run on the GPU.  ``__version__`` is the reference version this package
stands in for, without the distribution metadata the reference reads.
"""
from __future__ import annotations

from mc_dagprop_gb300 import __version__  # noqa: F401

from .analytic import (  # noqa: F401
    AnalyticContext,
    AnalyticPropagator,
    DiscretePMF,
    OverflowRule,
    SimulatedEvent,
    UnderflowRule,
    create_analytic_propagator,
)
from .monte_carlo import (  # noqa: F401
    Activity,
    DagContext,
    Event,
    EventTimestamp,
    GenericDelayGenerator,
    MonteCarloPropagator,
    SimResult,
    Simulator,
)

__all__ = [
    "GenericDelayGenerator",
    "DagContext",
    "SimResult",
    "Event",
    "Activity",
    "Simulator",
    "MonteCarloPropagator",
    "EventTimestamp",
    "DiscretePMF",
    "SimulatedEvent",
    "UnderflowRule",
    "OverflowRule",
    "AnalyticContext",
    "AnalyticPropagator",
    "create_analytic_propagator",
    "__version__",
]
