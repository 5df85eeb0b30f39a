"""Generates the golden fixtures in this folder from the reference itself.

Runs the reference's own ``MonteCarloPropagator.run_many`` (compiled from its
sources by ``oracle/build_ref.sh``, loaded by ``oracle/ref_loader.py``) on seeded
synthetic DAGs and stores inputs and outputs as compressed ``.npz`` files:

  config0_ref.npz   1,000-event / 2-type DAG (constant 1.5 + exponential), seeds 0..15
  five_types_ref.npz  1,200-event DAG with all five delay kinds, seeds 0..7
  gamma_state_ref.npz  the same DAG under a gamma-only generator, seeds 5,5,6 run in
                      sequence on one propagator (the reference's gamma draws carry
                      a cached normal across runs)
  config0_hashes_ref.npz  the 1,000-event DAG over all 10,000 seeds 0..9999: digests
                      (tests/mcd_testlib.py block_digests) of the reference's realized, durations
                      and cause_event rows, per block of 100 seeds -- the full run
                      pinned in a few KB

Usage:  python tests/golden/make_golden.py [name ...]   (needs the reference sources)
"""
from __future__ import annotations

import json
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, ROOT)

sys.path.insert(0, os.path.join(ROOT, "tests"))

import ref_loader  # noqa: E402
from mc_dagprop_gb300 import workloads as W  # noqa: E402
from mcd_testlib import block_digests  # noqa: E402


def encode_gen(gen):
    out = []
    for spec in gen:
        out.append([spec[0], int(spec[1])] + [
            [float(x) for x in p] if isinstance(p, (list, tuple, np.ndarray)) else float(p) for p in spec[2:]])
    return json.dumps(out)


def dump(name, flat, gen, seeds):
    ref = ref_loader.load()
    sim = ref.MonteCarloPropagator(W.to_context(ref, flat), W.to_generator(ref, gen))
    res = sim.run_many([int(s) for s in seeds])
    arrays = {k: np.asarray(v) for k, v in flat.items() if k != "max_delay"}
    np.savez_compressed(
        os.path.join(HERE, name),
        **arrays,
        max_delay=np.float64(flat["max_delay"]),
        gen=np.array(encode_gen(gen)),
        seeds=np.asarray(seeds, np.int64),
        realized=np.array([r.realized for r in res]),
        durations=np.array([r.durations for r in res]),
        cause=np.array([r.cause_event for r in res]),
        node_count=np.int64(sim.node_count()),
        activity_count=np.int64(sim.activity_count()),
    )
    print("wrote", name)


def dump_hashes(name, flat, gen, seeds):
    ref = ref_loader.load()
    sim = ref.MonteCarloPropagator(W.to_context(ref, flat), W.to_generator(ref, gen))
    res = sim.run_many([int(s) for s in seeds])
    np.savez_compressed(
        os.path.join(HERE, name),
        seeds=np.asarray(seeds, np.int64), block=np.int64(100),
        realized=block_digests(np.array([r.realized for r in res])),
        durations=block_digests(np.array([r.durations for r in res])),
        cause=block_digests(np.array([r.cause_event for r in res])),
    )
    print("wrote", name)


def main(names):
    flat0, gen0 = W.config0()
    flat5, gen5 = W.config1(seed=11, n_layers=30, width=40)
    jobs = {
        "config0_ref.npz": lambda n: dump(n, flat0, gen0, np.arange(16)),
        "five_types_ref.npz": lambda n: dump(n, flat5, gen5, np.arange(8)),
        "gamma_state_ref.npz": lambda n: dump(
            n, flat5, [("gamma", t, 2.0, 0.05, math.inf) for t in range(1, 6)], [5, 5, 6]),
        "config0_hashes_ref.npz": lambda n: dump_hashes(n, flat0, gen0, np.arange(10_000)),
    }
    for n in names or jobs:
        jobs[n](n)


if __name__ == "__main__":
    main(sys.argv[1:])
