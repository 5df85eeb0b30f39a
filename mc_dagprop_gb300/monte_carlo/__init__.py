"""Monte Carlo propagation on the GPU (the reference's ``mc_dagprop.monte_carlo``)."""
from __future__ import annotations

from .._core import Activity, Batch, DagContext, Server, Event, EventTimestamp, GenericDelayGenerator, MonteCarloPropagator, SimResult

Simulator = MonteCarloPropagator

__all__ = [
    "Batch",
    "Server",
    "GenericDelayGenerator",
    "DagContext",
    "SimResult",
    "Event",
    "Activity",
    "MonteCarloPropagator",
    "Simulator",
    "EventTimestamp",
]
