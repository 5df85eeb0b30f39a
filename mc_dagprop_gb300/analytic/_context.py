"""Analytic context types and validation (the reference's ``analytic/_context.py``).

Same classes, fields and checks (``validate_context``, _context.py:93-158), with
the reference's error messages."""
from __future__ import annotations

from collections import deque
from dataclasses import dataclass
from enum import IntEnum, unique

import numpy as np

from ..types import ActivityIndex, EventIndex, ProbabilityMass, Second
from ._pmf import DiscretePMF

PredecessorTuple = tuple[EventIndex, ActivityIndex]


@dataclass(frozen=True, slots=True)
class AnalyticActivity:
    """Edge with its delay distribution (``pmf``)."""

    idx: ActivityIndex
    pmf: DiscretePMF


@dataclass(frozen=True, slots=True)
class SimulatedEvent:
    """Propagated event: its time PMF and the mass below / above its bounds."""

    pmf: DiscretePMF
    underflow: ProbabilityMass
    overflow: ProbabilityMass


@unique
class UnderflowRule(IntEnum):
    """Mass below the lower bound: TRUNCATE onto the bound, REMOVE it, or
    REDISTRIBUTE it over the retained range."""

    TRUNCATE = 1
    REMOVE = 2
    REDISTRIBUTE = 3


@unique
class OverflowRule(IntEnum):
    """Mass above the upper bound: TRUNCATE onto the bound, REMOVE it, or
    REDISTRIBUTE it over the retained range."""

    TRUNCATE = 1
    REMOVE = 2
    REDISTRIBUTE = 3


@dataclass(frozen=True, slots=True)
class AnalyticContext:
    """The analytic network: events, activities {(src, dst): (idx, AnalyticActivity)},
    precedence list, grid step, flow rules and an optional delay cap relative to
    each event's earliest time."""

    events: tuple
    activities: dict
    precedence_list: tuple
    step: Second
    underflow_rule: UnderflowRule
    overflow_rule: OverflowRule
    max_delay: Second | None = None


def validate_context(context: AnalyticContext) -> None:
    """Structural checks: bounds, activity indices and PMFs, step, cycles."""
    n_events = len(context.events)
    if context.step <= 0.0:
        raise ValueError("step_size must be positive")
    if context.max_delay is not None and context.max_delay < 0.0:
        raise ValueError("max_delay must be non-negative when provided")
    for i, ev in enumerate(context.events):
        ts = ev.timestamp
        if ts.earliest > ts.latest:
            raise ValueError(f"event {i} has earliest > latest")
        if not (ts.earliest <= ts.actual <= ts.latest):
            raise ValueError(f"event {i} actual time outside bounds")
    for (src, dst), (_, edge) in context.activities.items():
        if not (0 <= src < n_events and 0 <= dst < n_events):
            raise ValueError(f"activity {(src, dst)} references invalid node")
        edge.pmf.validate()
        if not np.isclose(edge.pmf.step, context.step):
            raise ValueError(f"edge {(src, dst)} step {edge.pmf.step} does not match context step size {context.step}")
        edge.pmf.validate_alignment(context.step)
        if not np.isclose(edge.pmf.total_mass, 1.0):
            raise ValueError(f"activity {(src, dst)} PMF does not sum to 1, got {edge.pmf.total_mass}")
    adjacency: list[list[int]] = [[] for _ in range(n_events)]
    indegree = [0] * n_events
    for target, preds in context.precedence_list:
        if not (0 <= target < n_events):
            raise ValueError(f"target index {target} out of range")
        for src, link in preds:
            if not (0 <= src < n_events):
                raise ValueError(f"predecessor index {src} out of range")
            edge = context.activities.get((src, target))
            if edge is None:
                raise ValueError(f"missing activity for {(src, target)}")
            if edge[0] != link:
                raise ValueError(f"edge index {link} for {(src, target)} does not match context mapping {edge[0]}")
            adjacency[src].append(target)
            indegree[target] += 1
    q = deque(i for i, d in enumerate(indegree) if d == 0)
    seen = 0
    while q:
        node = q.popleft()
        seen += 1
        for dst in adjacency[node]:
            indegree[dst] -= 1
            if indegree[dst] == 0:
                q.append(dst)
    if seen != n_events:
        raise ValueError("precedence list contains a cycle")
