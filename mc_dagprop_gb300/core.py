"""Re-exports of the core data classes (the reference's ``mc_dagprop.core``)."""
from __future__ import annotations

from .monte_carlo import Activity, DagContext, Event, EventTimestamp

__all__ = ["EventTimestamp", "Event", "Activity", "DagContext"]
