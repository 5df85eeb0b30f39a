"""Analytic PMF propagation on the GPU (the reference's ``analytic/_propagator.py``).

``create_analytic_propagator`` validates the context (as the reference does,
_propagator.py:48-72), flattens it and compiles it on the device through the C
ABI (``mcd_analytic_create``); ``AnalyticPropagator.run`` propagates every event's
PMF on the GPU (``mcd_analytic_run``, one CTA per event of a level) and returns
the ``SimulatedEvent`` tuple in event order (_propagator.py:89-148).  There is no
CPU path: the compiled library is required.
"""
from __future__ import annotations

import ctypes as C
import math
import os
from dataclasses import dataclass, field

import numpy as np

from ..types import ProbabilityMass
from ._context import AnalyticContext, OverflowRule, SimulatedEvent, UnderflowRule, validate_context
from ._pmf import DiscretePMF

_LIB = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "_lib", "libmcdagprop_gb300.so")
_lib = None


class _Desc(C.Structure):
    _fields_ = [("n_events", C.c_int32), ("earliest", C.c_void_p), ("latest", C.c_void_p),
                ("n_pmfs", C.c_int32), ("pmf_off", C.c_void_p), ("pmf_first", C.c_void_p), ("pmf_probs", C.c_void_p),
                ("n_targets", C.c_int32), ("target", C.c_void_p), ("pred_off", C.c_void_p),
                ("pred_src", C.c_void_p), ("pred_pmf", C.c_void_p), ("step", C.c_int32),
                ("max_delay", C.c_double), ("underflow_rule", C.c_int32), ("overflow_rule", C.c_int32)]


def _api():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB):
            raise ImportError("mc_dagprop_gb300.analytic requires the compiled library "
                              f"{_LIB} (build it with `python mc_dagprop_gb300/_build.py`)")
        L = C.CDLL(_LIB)
        P, I64 = C.c_void_p, C.c_int64
        L.mcd_last_error.restype = C.c_char_p
        L.mcd_analytic_create.argtypes = [C.POINTER(_Desc), C.POINTER(P)]
        L.mcd_analytic_destroy.argtypes = [P]
        L.mcd_analytic_run.argtypes = [P]
        L.mcd_analytic_bins.argtypes = [P]
        L.mcd_analytic_bins.restype = I64
        L.mcd_analytic_fetch.argtypes = [P, P, P, P, P, P, P]
        _lib = L
    return _lib


def _check(rc: int) -> None:
    if rc != 0:
        msg = _api().mcd_last_error().decode()
        raise (RuntimeError if rc in (2, 3, 5) else ValueError)(msg)


def _flatten(context: AnalyticContext) -> dict:
    """The context as the C ABI takes it: activity PMFs concatenated, each
    predecessor entry pointing at its (source, target) activity's PMF."""
    keys = list(context.activities.keys())
    slot = {k: i for i, k in enumerate(keys)}
    probs = [np.asarray(context.activities[k][1].pmf.probabilities, dtype=np.float64) for k in keys]
    off = np.zeros(len(keys) + 1, np.int64)
    off[1:] = np.cumsum([len(p) for p in probs]) if probs else []
    first = np.array([float(context.activities[k][1].pmf.values[0]) for k in keys], np.float64)
    target, pred_off, pred_src, pred_pmf = [], [0], [], []
    for tgt, preds in context.precedence_list:
        target.append(int(tgt))
        for src, _ in preds:
            key = (int(src), int(tgt))
            if key not in slot:
                raise ValueError(f"missing activity for {key}")
            pred_src.append(int(src))
            pred_pmf.append(slot[key])
        pred_off.append(len(pred_src))
    ev = context.events
    return {
        "earliest": np.array([float(e.timestamp.earliest) for e in ev], np.float64),
        "latest": np.array([float(e.timestamp.latest) for e in ev], np.float64),
        "pmf_off": off, "pmf_first": first,
        "pmf_probs": np.concatenate(probs) if probs else np.zeros(1, np.float64),
        "target": np.array(target, np.int32), "pred_off": np.array(pred_off, np.int64),
        "pred_src": np.array(pred_src, np.int32), "pred_pmf": np.array(pred_pmf, np.int32),
    }


def _desc(flat: dict, step: int, max_delay, urule: int, orule: int) -> _Desc:
    p = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    return _Desc(len(flat["earliest"]), p(flat["earliest"]), p(flat["latest"]), len(flat["pmf_first"]),
                 p(flat["pmf_off"]), p(flat["pmf_first"]), p(flat["pmf_probs"]), len(flat["target"]),
                 p(flat["target"]), p(flat["pred_off"]), p(flat["pred_src"]), p(flat["pred_pmf"]), int(step),
                 math.nan if max_delay is None else float(max_delay), int(urule), int(orule))


def create_analytic_propagator(context: AnalyticContext, validate: bool = True) -> "AnalyticPropagator":
    """An ``AnalyticPropagator`` for ``context``, compiled on the current CUDA
    device; ``validate=False`` skips ``validate_context``."""
    if validate:
        validate_context(context)
    step = context.step
    if int(step) != step or step <= 0:
        raise ValueError("step_size must be positive")
    flat = _flatten(context)
    handle = C.c_void_p()
    _check(_api().mcd_analytic_create(C.byref(_desc(flat, int(step), context.max_delay, int(context.underflow_rule),
                                                      int(context.overflow_rule))), C.byref(handle)))
    return AnalyticPropagator(context=context, _handle=handle)


@dataclass(frozen=True, slots=True)
class AnalyticPropagator:
    """Propagates discrete PMFs through the DAG on the GPU."""

    context: AnalyticContext
    _handle: C.c_void_p = field(repr=False)

    def __del__(self):
        if _lib is not None and self._handle:
            _lib.mcd_analytic_destroy(self._handle)

    @property
    def underflow_rule(self) -> UnderflowRule:
        return self.context.underflow_rule

    @property
    def overflow_rule(self) -> OverflowRule:
        return self.context.overflow_rule

    def run_arrays(self):
        """The run's results as arrays: first value, offset and length of each
        event's probabilities in ``probs``, underflow, overflow (no Python objects)."""
        L = _api()
        _check(L.mcd_analytic_run(self._handle))
        E = len(self.context.events)
        first = np.empty(E)
        off = np.empty(E, np.int64)
        ln = np.empty(E, np.int64)
        under = np.empty(E)
        over = np.empty(E)
        probs = np.empty(max(1, L.mcd_analytic_bins(self._handle)))
        p = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
        _check(L.mcd_analytic_fetch(self._handle, p(first), p(off), p(ln), p(probs), p(under), p(over)))
        return first, off, ln, probs, under, over

    def run(self) -> tuple[SimulatedEvent, ...]:
        """Every event's PMF and its underflow/overflow masses, in event order."""
        first, off, ln, probs, under, over = self.run_arrays()
        step = self.context.step
        out = []
        for e in range(len(first)):
            pr = probs[off[e]:off[e] + ln[e]].copy()
            vals = first[e] + step * np.arange(ln[e], dtype=float)
            out.append(SimulatedEvent(DiscretePMF(vals, pr, step=step), ProbabilityMass(float(under[e])),
                                      ProbabilityMass(float(over[e]))))
        return tuple(out)
