"""The reference's own Monte Carlo test suite, restated against ``import mc_dagprop``
(this repository's drop-in package, served by the GPU engine).

Each test below follows one test of the reference (cited by file:line) with the
same inputs and the same assertions.  Three assertions of the reference check the
exact Xoshiro256++ stream of seed 7 (test/test_simulator.py:145, 154, 171:
68.0, 34.10 and 23.0624...); the GPU draws from Philox, so here those three check
that the realized time is one the table allows, and the exact values are pinned
against the oracle instead (tests/test_oracle_pin.py).
"""
from __future__ import annotations

from concurrent.futures import ThreadPoolExecutor
from itertools import chain

import numpy as np
import pytest

import mc_dagprop
from mc_dagprop import (Activity, DagContext, Event, EventTimestamp, GenericDelayGenerator, MonteCarloPropagator,
                        Simulator)
from mc_dagprop.monte_carlo import Simulator as MCSimulator
from mc_dagprop.types import ActivityIndex, EventId, Second

pytestmark = pytest.mark.gpu


# ---------------------------------------------------------------- test/test_simulator.py

EARLIEST6 = [0.0, 5.0, 10.0, 22.0, 20.0, 100.0]


def _six_event_context(reverse: bool = False) -> DagContext:
    """The fixture of test/test_simulator.py:11-35."""
    events = [Event(str(i), EventTimestamp(t, 100.0, 0.0)) for i, t in enumerate(EARLIEST6)]
    links = {
        (0, 1): Activity(idx=0, minimal_duration=3.0, activity_type=1),
        (1, 2): Activity(idx=1, minimal_duration=5.0, activity_type=1),
        (1, 3): Activity(idx=2, minimal_duration=5.0, activity_type=1),
        (2, 4): Activity(idx=3, minimal_duration=15.0, activity_type=2),
        (3, 4): Activity(idx=4, minimal_duration=10.0, activity_type=3),
    }
    prec = [(1, [(0, 0)]), (2, [(1, 1)]), (3, [(1, 2)]), (4, [(2, 3), (3, 4)])]
    if reverse:
        prec = list(reversed(prec))
    return DagContext(events=events, activities=links, precedence_list=prec, max_delay=1e6)


def test_constant_via_generic(cuda):
    """test/test_simulator.py:37-62."""
    gen = GenericDelayGenerator()
    gen.add_constant(activity_type=1, factor=1.0)
    sim = Simulator(_six_event_context(), gen)
    res = sim.run(seed=7)
    batch = sim.run_many([1, 2, 3])
    assert len(batch) == 3 and all(isinstance(b, type(res)) for b in batch)
    assert res.realized[1] == pytest.approx(6.0, abs=1e-6)
    assert res.realized[2] == pytest.approx(16.0, abs=1e-6)
    assert len(res.durations) == 5 and len(res.realized) == 6 and len(res.cause_event) == 6
    assert list(res.cause_event[:3]) == [-1, 0, 1]


def test_unsorted_precedence_same_result(cuda):
    """test/test_simulator.py:64-82."""
    results = []
    for reverse in (False, True):
        gen = GenericDelayGenerator()
        gen.add_constant(activity_type=1, factor=1.0)
        results.append(Simulator(_six_event_context(reverse), gen).run(seed=7))
    a, b = results
    np.testing.assert_allclose(a.realized, b.realized)
    np.testing.assert_allclose(a.durations, b.durations)
    np.testing.assert_array_equal(a.cause_event, b.cause_event)


def test_exponential_via_generic(cuda):
    """test/test_simulator.py:84-105."""
    gen = GenericDelayGenerator()
    gen.add_exponential(1, 1000.0, max_scale=1.0)
    sim = Simulator(_six_event_context(), gen)
    for res in sim.run_many(tuple(range(3))):
        r = list(res.realized)
        assert r[0] == pytest.approx(0.0, abs=1e-6)
        assert r[1] >= 5.0
        assert r[2] >= r[1]
        assert r[2] <= r[1] + 5.0 * 10.0 + 1e-6
        assert len(list(res.durations)) == 5


def test_propagation(cuda):
    """test/test_simulator.py:107-137."""
    gen = GenericDelayGenerator()
    gen.add_constant(activity_type=1, factor=1.0)
    gen.add_constant(activity_type=3, factor=3.0)
    res = Simulator(_six_event_context(), gen).run_many(tuple(range(5)))[3]
    assert list(res.durations) == [6.0, 10.0, 10.0, 15.0, 40.0]
    assert list(res.realized) == [0.0, 6.0, 16.0, 22.0, 62.0, 100.0]
    assert list(res.cause_event) == [-1, 0, 1, -1, 3, -1]


def _event3_support(table, relative):
    """Every realized time event 3 can take when links 0 and 2 (type 1) draw from
    `table`: event 1 = max(5, 0 + d0), event 3 = max(22, event 1 + d2), each
    duration the reference's base + value or base + factor * base."""
    out = set()
    for a in table:
        d0 = 3.0 + a * 3.0 if relative else 3.0 + a
        r1 = max(5.0, 0.0 + d0)
        for b in table:
            d2 = 5.0 + b * 5.0 if relative else 5.0 + b
            out.add(max(22.0, r1 + d2))
    return out


def test_empirical_absolute(cuda):
    """test/test_simulator.py:139-146 (exact stream of seed 7: oracle only)."""
    values = [10, 20, 40, 50]
    gen = GenericDelayGenerator()
    gen.add_empirical_absolute(activity_type=1, values=values, weights=[0.1, 0.2, 0.3, 0.4])
    sim = Simulator(_six_event_context(), gen)
    support = _event3_support([float(v) for v in values], relative=False)
    res = sim.run(seed=7)
    assert res.realized[3] in support and res.realized[5] == 100.0
    seen = {r.realized[3] for r in sim.run_many(list(range(2000)))}
    assert seen <= support and len(seen) > 4


def test_empirical_relative(cuda):
    """test/test_simulator.py:148-155 (exact stream of seed 7: oracle only)."""
    factors = [1.2, 1.3, 1.35, 4.5]
    gen = GenericDelayGenerator()
    gen.add_empirical_relative(activity_type=1, factors=factors, weights=[0.1, 0.2, 0.3, 0.4])
    sim = Simulator(_six_event_context(), gen)
    support = _event3_support(factors, relative=True)
    res = sim.run(seed=7)
    assert res.realized[3] in support and res.realized[5] == 100.0
    seen = {r.realized[3] for r in sim.run_many(list(range(2000)))}
    assert seen <= support and len(seen) > 4


def test_empirical_relative_with_exponential(cuda):
    """test/test_simulator.py:157-172: a 1,000-bin relative table from a truncated
    exponential sample (exact stream of seed 7: oracle only)."""
    values = []
    rs = np.random.RandomState(7)
    while len(values) < 1_000_000:  # the reference's rejection loop, vectorised
        draws = rs.exponential(3.0, size=200_000)
        values.extend(draws[draws <= 5.0].tolist())
    values = values[:1_000_000]
    hist, edges = np.histogram(values, bins=1000, density=True)
    centers = 0.5 * (edges[:-1] + edges[1:])
    gen = GenericDelayGenerator()
    gen.add_empirical_relative(activity_type=1, factors=centers, weights=hist)
    res = Simulator(_six_event_context(), gen).run(seed=7)
    lo, hi = float(centers.min()), float(centers.max())
    r1 = res.realized[1]
    assert max(5.0, 3.0 + lo * 3.0) <= r1 <= max(5.0, 3.0 + hi * 3.0)
    assert max(22.0, r1 + 5.0 + lo * 5.0) <= res.realized[3] <= max(22.0, r1 + 5.0 + hi * 5.0)
    assert res.realized[5] == 100.0


def _chain_context(n: int = 10_000) -> DagContext:
    """The fixture of test/test_simulator.py:175-183."""
    events = [Event(str(i), EventTimestamp(float(i), 100.0 + i, 0.0)) for i in range(n)]
    links = {(i, i + 1): Activity(idx=i, minimal_duration=3.0, activity_type=1) for i in range(n - 1)}
    prec = [(i, [(i - 1, i)]) for i in range(1, n)]
    return DagContext(events=events, activities=links, precedence_list=prec, max_delay=1e6)


def test_large_scale_simulation(cuda):
    """test/test_simulator.py:185-199."""
    gen = GenericDelayGenerator()
    gen.add_constant(activity_type=1, factor=1.0)
    res = Simulator(_chain_context(), gen).run(seed=7)
    assert len(res.realized) == 10_000 and len(res.durations) == 9999 and len(res.cause_event) == 10_000
    assert res.realized[0] == pytest.approx(0.0, abs=1e-6)
    assert res.realized[9999] == pytest.approx(59988.0, abs=1e-6)


def test_multithreading(cuda):
    """test/test_simulator.py:201-215: one simulator per thread, run_many in parallel."""
    gen = GenericDelayGenerator()
    gen.add_constant(activity_type=1, factor=1.0)
    ctx = _chain_context()
    sims = [Simulator(ctx, gen) for _ in range(4)]
    seeds = [[i + j for i in range(1000)] for j in range(4)]
    with ThreadPoolExecutor(max_workers=4) as pool:
        results = list(chain.from_iterable(pool.map(lambda a: a[0].run_many(a[1]), zip(sims, seeds))))
    assert len(results) == 4000
    for r in results:
        assert len(r.realized) == 10_000 and len(r.durations) == 9999 and len(r.cause_event) == 10_000
    # constant links: every sample is the same chain
    assert all(r.realized[9999] == results[0].realized[9999] for r in results)


# ---------------------------------------------------------------- test/test_monte_carlo_extra.py

def _three_event_context(max_delay: float = 1e6) -> DagContext:
    """The fixture of test/test_monte_carlo_extra.py:9-21."""
    events = [Event(str(i), EventTimestamp(0.0, 100.0, 0.0)) for i in range(3)]
    acts = {(0, 1): Activity(idx=0, minimal_duration=1.0, activity_type=1),
            (1, 2): Activity(idx=1, minimal_duration=2.0, activity_type=1)}
    return DagContext(events=events, activities=acts, precedence_list=[(1, [(0, 0)]), (2, [(1, 1)])],
                      max_delay=max_delay)


def test_constant_distribution(cuda):
    """test/test_monte_carlo_extra.py:28-35."""
    gen = GenericDelayGenerator()
    gen.add_constant(activity_type=1, factor=1.0)
    res = Simulator(_three_event_context(), gen).run(seed=42)
    np.testing.assert_allclose(res.durations, [2.0, 4.0])
    np.testing.assert_allclose(res.realized, [0.0, 2.0, 6.0])


@pytest.mark.parametrize("seed,add", [
    (0, lambda g: g.add_exponential(activity_type=1, lambda_=2.0, max_scale=0.5)),  # :37-46
    (1, lambda g: g.add_gamma(activity_type=1, shape=2.0, scale=1.0, max_scale=0.5)),  # :48-57
])
def test_truncated_distribution_bounds(cuda, seed, add):
    """test/test_monte_carlo_extra.py:37-57 (and the same bounds over 500 more seeds)."""
    gen = GenericDelayGenerator()
    add(gen)
    sim = Simulator(_three_event_context(), gen)
    for res in [sim.run(seed=seed)] + sim.run_many(list(range(500))):
        assert 1.0 <= res.durations[0] <= 1.5
        assert 2.0 <= res.durations[1] <= 3.0
        assert res.realized[2] >= res.realized[1]


def test_cycle_detection(cuda):
    """test/test_monte_carlo_extra.py:61-72."""
    events = [Event("0", EventTimestamp(0.0, 100.0, 0.0)), Event("1", EventTimestamp(0.0, 100.0, 0.0))]
    acts = {(0, 1): Activity(idx=0, minimal_duration=1.0, activity_type=1),
            (1, 0): Activity(idx=1, minimal_duration=1.0, activity_type=1)}
    ctx = DagContext(events=events, activities=acts, precedence_list=[(1, [(0, 0)]), (0, [(1, 1)])], max_delay=1e6)
    gen = GenericDelayGenerator()
    gen.add_constant(1, 0.0)
    with pytest.raises(RuntimeError):
        Simulator(ctx, gen)


def test_reserved_activity_type(cuda):
    """test/test_monte_carlo_extra.py:74-79."""
    gen = GenericDelayGenerator()
    gen.add_constant(-1, 0.0)
    with pytest.raises(RuntimeError):
        Simulator(_three_event_context(), gen)


def test_negative_max_delay_rejected(cuda):
    """test/test_monte_carlo_extra.py:81-92."""
    ctx = _three_event_context()
    bad = DagContext(events=ctx.events, activities=ctx.activities, precedence_list=ctx.precedence_list,
                     max_delay=-1.0)
    gen = GenericDelayGenerator()
    gen.add_constant(1, 0.0)
    with pytest.raises(RuntimeError):
        Simulator(bad, gen)


def test_run_many_matches_individual_runs(cuda):
    """test/test_monte_carlo_extra.py:95-109."""
    gen = GenericDelayGenerator()
    gen.add_exponential(activity_type=1, lambda_=1.0, max_scale=0.5)
    sim = Simulator(_three_event_context(), gen)
    seeds = list(range(5))
    batch = sim.run_many(seeds)
    solo = [sim.run(s) for s in seeds]
    assert len(batch) == len(solo)
    for b, s in zip(batch, solo):
        np.testing.assert_allclose(b.realized, s.realized)
        np.testing.assert_allclose(b.durations, s.durations)
        np.testing.assert_array_equal(b.cause_event, s.cause_event)


# ---------------------------------------------------------------- test/test_naming_conventions.py

def test_monte_carlo_class_name_is_primary():
    """test/test_naming_conventions.py:6-8."""
    assert MonteCarloPropagator.__name__ == "MonteCarloPropagator"
    assert Simulator is MonteCarloPropagator and MCSimulator is MonteCarloPropagator


def test_public_surface_and_types(cuda):
    """The reference's public surface (src/mc_dagprop/__init__.py:33-49, types.py)."""
    for name in mc_dagprop.__all__:
        assert hasattr(mc_dagprop, name), name
    assert isinstance(mc_dagprop.__version__, str) and mc_dagprop.__version__.startswith("0.9.0")
    ts = EventTimestamp(Second(1.0), Second(2.0), Second(3.0))
    ev = Event(EventId("a"), ts)
    act = Activity(ActivityIndex(0), 1.5, 2)
    assert (ev.event_id, ev.timestamp.earliest, act.idx) == ("a", 1.0, 0)
