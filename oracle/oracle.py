"""ctypes wrapper around the C oracle (``mcd_oracle.c``).

TEST INFRASTRUCTURE ONLY: tests, ``__graft_entry__.smoke()`` and the CPU-baseline
leg of ``bench.py`` use it as the oracle results are compared with.  The product
path never imports it.

The oracle restates the reference's ``Simulator`` (src/mc_dagprop/monte_carlo/
_core.cpp:161-362) and its libstdc++ distribution arithmetic in C; it is pinned
bit-for-bit against the reference compiled from source (tests/test_oracle_pin.py)
and against committed golden fixtures (tests/golden/).

A DAG is passed in flat form (a dict of numpy arrays, see ``FLAT_KEYS``) and a
generator as a list of tuples, e.g. ``("exponential", type, lambda_, max_scale)``.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liborc.so")

FLAT_KEYS = ("earliest", "act_idx", "act_duration", "act_type", "target",
             "pred_offsets", "pred_src", "pred_act", "max_delay")

KINDS = {"constant": 0, "exponential": 1, "gamma": 2, "empirical_absolute": 3, "empirical_relative": 4}


class _DistDesc(C.Structure):
    _fields_ = [("activity_type", C.c_int32), ("kind", C.c_int32),
                ("p0", C.c_double), ("p1", C.c_double), ("p2", C.c_double),
                ("n_table", C.c_int64), ("values", C.POINTER(C.c_double)),
                ("weights", C.POINTER(C.c_double))]


class _DagDesc(C.Structure):
    _fields_ = [("n_events", C.c_int32), ("earliest", C.POINTER(C.c_double)),
                ("n_activities", C.c_int32), ("act_idx", C.POINTER(C.c_int32)),
                ("act_duration", C.POINTER(C.c_double)), ("act_type", C.POINTER(C.c_int32)),
                ("n_targets", C.c_int32), ("target", C.POINTER(C.c_int32)),
                ("pred_offsets", C.POINTER(C.c_int64)), ("pred_src", C.POINTER(C.c_int32)),
                ("pred_act", C.POINTER(C.c_int32)), ("max_delay", C.c_double)]


def build(force: bool = False) -> str:
    if force or not os.path.exists(LIB_PATH) or (
            os.path.getmtime(LIB_PATH) < os.path.getmtime(os.path.join(HERE, "mcd_oracle.c"))):
        subprocess.run(["make", "-s", "-C", HERE, "_build/liborc.so"], check=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        L.orc_sim_create.argtypes = [C.POINTER(_DagDesc), C.POINTER(_DistDesc), C.c_int32,
                                     C.POINTER(C.c_void_p), C.c_char_p, C.c_size_t]
        L.orc_sim_create.restype = C.c_int
        L.orc_sim_destroy.argtypes = [C.c_void_p]
        L.orc_node_count.argtypes = [C.c_void_p]
        L.orc_node_count.restype = C.c_int32
        L.orc_activity_count.argtypes = [C.c_void_p]
        L.orc_activity_count.restype = C.c_int32
        P = C.c_void_p
        L.orc_run_many.argtypes = [P, P, C.c_int64, P, P, P]
        L.orc_run_many_mt.argtypes = [P, P, C.c_int64, C.c_int32, P, P, P]
        L.orc_propagate_given.argtypes = [P, P, C.c_int64, P, P]
        L.orc_eval_order.argtypes = [P, P]
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


class OracleError(RuntimeError):
    pass


class OracleSim:
    """The reference's MonteCarloPropagator, restated in C (one instance = one
    simulator with its own distribution state, like the reference)."""

    def __init__(self, flat: dict, gen: list):
        L = lib()
        self._keep = []
        f = {k: flat[k] for k in FLAT_KEYS}
        arr = {}
        for k, dt in (("earliest", np.float64), ("act_idx", np.int32), ("act_duration", np.float64),
                      ("act_type", np.int32), ("target", np.int32), ("pred_offsets", np.int64),
                      ("pred_src", np.int32), ("pred_act", np.int32)):
            arr[k] = np.ascontiguousarray(f[k], dtype=dt)
        self._keep.append(arr)
        d = _DagDesc()
        d.n_events = len(arr["earliest"])
        d.earliest = arr["earliest"].ctypes.data_as(C.POINTER(C.c_double))
        d.n_activities = len(arr["act_idx"])
        d.act_idx = arr["act_idx"].ctypes.data_as(C.POINTER(C.c_int32))
        d.act_duration = arr["act_duration"].ctypes.data_as(C.POINTER(C.c_double))
        d.act_type = arr["act_type"].ctypes.data_as(C.POINTER(C.c_int32))
        d.n_targets = len(arr["target"])
        d.target = arr["target"].ctypes.data_as(C.POINTER(C.c_int32))
        d.pred_offsets = arr["pred_offsets"].ctypes.data_as(C.POINTER(C.c_int64))
        d.pred_src = arr["pred_src"].ctypes.data_as(C.POINTER(C.c_int32))
        d.pred_act = arr["pred_act"].ctypes.data_as(C.POINTER(C.c_int32))
        d.max_delay = float(f["max_delay"])
        dists = (_DistDesc * max(1, len(gen)))()
        for i, spec in enumerate(gen):
            kind = spec[0]
            dd = dists[i]
            dd.activity_type = int(spec[1])
            dd.kind = KINDS[kind]
            if kind == "constant":
                dd.p0 = float(spec[2])
            elif kind == "exponential":
                dd.p0, dd.p1 = float(spec[2]), float(spec[3])
            elif kind == "gamma":
                dd.p0, dd.p1 = float(spec[2]), float(spec[3])
                dd.p2 = float(spec[4]) if len(spec) > 4 else float("inf")
            else:
                v = np.ascontiguousarray(spec[2], dtype=np.float64)
                w = np.ascontiguousarray(spec[3], dtype=np.float64)
                if len(v) != len(w):
                    name = "EmpiricalAbsoluteDist" if kind == "empirical_absolute" else "EmpiricalRelativeDist"
                    what = "values" if kind == "empirical_absolute" else "factors"
                    raise OracleError(f"{name}: {what} and weights must have same length")
                self._keep.append((v, w))
                dd.n_table = len(v)
                dd.values = v.ctypes.data_as(C.POINTER(C.c_double))
                dd.weights = w.ctypes.data_as(C.POINTER(C.c_double))
        h = C.c_void_p()
        err = C.create_string_buffer(512)
        rc = L.orc_sim_create(C.byref(d), dists, len(gen), C.byref(h), err, 512)
        if rc != 0:
            raise OracleError(err.value.decode())
        self._h = h
        self.E = L.orc_node_count(h)
        self.L = L.orc_activity_count(h)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and _lib is not None:
            _lib.orc_sim_destroy(h)
            self._h = None

    def node_count(self) -> int:
        return self.E

    def activity_count(self) -> int:
        return self.L

    def eval_order(self) -> np.ndarray:
        o = np.empty(self.E, np.int32)
        lib().orc_eval_order(self._h, _ptr(o))
        return o

    def run_many(self, seeds, threads: int = 1, want=("realized", "durations", "cause")):
        """Sample-major outputs: realized (S,E), durations (S,L), cause (S,E)."""
        seeds = np.ascontiguousarray(seeds, dtype=np.int64)
        n = len(seeds)
        real = np.empty((n, self.E), np.float64) if "realized" in want else None
        dur = np.empty((n, self.L), np.float64) if "durations" in want else None
        cause = np.empty((n, self.E), np.int32) if "cause" in want else None
        if threads <= 1:
            lib().orc_run_many(self._h, _ptr(seeds), n, _ptr(real), _ptr(dur), _ptr(cause))
        else:
            lib().orc_run_many_mt(self._h, _ptr(seeds), n, threads, _ptr(real), _ptr(dur), _ptr(cause))
        return real, dur, cause

    def propagate_given(self, durations: np.ndarray):
        durations = np.ascontiguousarray(durations, dtype=np.float64)
        n = durations.shape[0]
        assert durations.shape[1] == self.L
        real = np.empty((n, self.E), np.float64)
        cause = np.empty((n, self.E), np.int32)
        lib().orc_propagate_given(self._h, _ptr(durations), n, _ptr(real), _ptr(cause))
        return real, cause
