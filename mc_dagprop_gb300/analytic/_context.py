"""Analytic context types (the reference's ``analytic/_context.py``) and their
structural validation.

The dataclasses and enums are the reference's public types, with the same names,
fields and values.  ``validate_context`` reports the reference's errors
(_context.py:93-158) -- the same messages, and when a context has several
problems, the one the reference reports first -- but is organised as one ordered
stream of problems (``_problems``): vectorised checks over the events' bounds,
one check per activity and per precedence entry, and a cycle test that peels the
DAG level by level (every event whose predecessors are all peeled is peeled in
the same step; an event that never is lies on a cycle).
"""
from __future__ import annotations

from dataclasses import dataclass
from enum import IntEnum, unique
from typing import Iterator

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


def _event_problem(events) -> str | None:
    """The first event whose bounds are out of order or whose actual time lies
    outside them (NaN times fail the second test, as in a chained comparison)."""
    if not events:
        return None
    t = np.array([(e.timestamp.earliest, e.timestamp.latest, e.timestamp.actual) for e in events], dtype=float)
    early, late, act = t[:, 0], t[:, 1], t[:, 2]
    inverted = early > late
    outside = ~((early <= act) & (act <= late))
    bad = np.flatnonzero(inverted | outside)
    if not len(bad):
        return None
    i = int(bad[0])
    return f"event {i} has earliest > latest" if inverted[i] else f"event {i} actual time outside bounds"


def _activity_problem(key, edge: AnalyticActivity, n_events: int, step) -> str | None:
    """Checks of one activity: its endpoints, then its PMF (which raises its own
    errors), its step, its grid, its mass."""
    src, dst = key
    if not (0 <= src < n_events and 0 <= dst < n_events):
        return f"activity {(src, dst)} references invalid node"
    pmf = edge.pmf
    pmf.validate()
    if not np.isclose(pmf.step, step):
        return f"edge {(src, dst)} step {pmf.step} does not match context step size {step}"
    pmf.validate_alignment(step)
    if not np.isclose(pmf.total_mass, 1.0):
        return f"activity {(src, dst)} PMF does not sum to 1, got {pmf.total_mass}"
    return None


def _has_cycle(n_events: int, src: np.ndarray, dst: np.ndarray) -> bool:
    """Level peeling: repeatedly remove every event with no unremoved predecessor;
    the graph is acyclic exactly when every event is removed."""
    waiting = np.bincount(dst, minlength=n_events) if len(dst) else np.zeros(n_events, np.int64)
    order = np.argsort(src, kind="stable")
    out_dst = dst[order]
    out_start = np.searchsorted(src[order], np.arange(n_events + 1))
    level = np.flatnonzero(waiting == 0)
    removed = 0
    while len(level):
        removed += len(level)
        reach = np.concatenate([out_dst[out_start[v]:out_start[v + 1]] for v in level]) if len(dst) else []
        if not len(reach):
            break
        np.subtract.at(waiting, reach, 1)
        level = np.unique(reach[waiting[reach] == 0])
    return removed != n_events


def _problems(context: AnalyticContext) -> Iterator[str]:
    n_events = len(context.events)
    if context.step <= 0.0:
        yield "step_size must be positive"
    if context.max_delay is not None and context.max_delay < 0.0:
        yield "max_delay must be non-negative when provided"
    msg = _event_problem(context.events)
    if msg:
        yield msg
    for key, (_, edge) in context.activities.items():
        msg = _activity_problem(key, edge, n_events, context.step)
        if msg:
            yield msg
    src, dst = [], []
    for target, preds in context.precedence_list:
        if not (0 <= target < n_events):
            yield f"target index {target} out of range"
            continue
        for s, link in preds:
            if not (0 <= s < n_events):
                yield f"predecessor index {s} out of range"
                continue
            mapped = context.activities.get((s, target))
            if mapped is None:
                yield f"missing activity for {(s, target)}"
                continue
            if mapped[0] != link:
                yield f"edge index {link} for {(s, target)} does not match context mapping {mapped[0]}"
            src.append(s)
            dst.append(target)
    if _has_cycle(n_events, np.asarray(src, np.int64), np.asarray(dst, np.int64)):
        yield "precedence list contains a cycle"


def validate_context(context: AnalyticContext) -> None:
    """Raise ``ValueError`` with the first structural problem of ``context``:
    step and delay cap, event bounds, activities and their PMFs, the precedence
    list's indices and activity mapping, cycles."""
    for msg in _problems(context):
        raise ValueError(msg)
