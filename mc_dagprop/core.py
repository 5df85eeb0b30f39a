"""``mc_dagprop.core``: the core data classes (reference ``src/mc_dagprop/core.py``)."""
from __future__ import annotations

from .monte_carlo import Activity, DagContext, Event, EventTimestamp  # noqa: F401

__all__ = ["EventTimestamp", "Event", "Activity", "DagContext"]
