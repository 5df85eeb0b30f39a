"""The reference's analytic-engine tests (test/test_discrete_simulator.py),
restated against ``import mc_dagprop``: the same contexts and the same
assertions, through the GPU engine.  (Its validation-error cases run on the host
in tests/test_analytic_cpu.py.  test_clipping_tolerates_rounding_errors calls the
reference propagator's private _convert_to_simulated_event; the GPU engine clips
inside its fold kernel and has no such method, so that case is covered by the
mass checks of the rule tables below.)"""
from __future__ import annotations

from dataclasses import replace

import numpy as np
import pytest

from mc_dagprop import (
    Activity,
    AnalyticContext,
    DagContext,
    DiscretePMF,
    Event,
    EventTimestamp,
    GenericDelayGenerator,
    Simulator,
    create_analytic_propagator,
)
from mc_dagprop.analytic import OverflowRule, UnderflowRule
from mc_dagprop.analytic._context import AnalyticActivity, SimulatedEvent

pytestmark = pytest.mark.gpu

T, RM, RD = UnderflowRule.TRUNCATE, UnderflowRule.REMOVE, UnderflowRule.REDISTRIBUTE
OT, ORM, ORD = OverflowRule.TRUNCATE, OverflowRule.REMOVE, OverflowRule.REDISTRIBUTE


def _pmf(values, probs, step=1):
    return DiscretePMF(np.array(values, dtype=float), np.array(probs, dtype=float), step=step)


def _three_event_setup():
    """The fixture of test/test_discrete_simulator.py:47-84: a two-edge chain in
    both engines."""
    events = tuple(Event(str(i), EventTimestamp(0.0, 100.0, 0.0)) for i in range(3))
    prec = ((1, ((0, 0),)), (2, ((1, 1),)))
    acts = {(0, 1): (0, AnalyticActivity(0, _pmf([1.0, 2.0], [0.5, 0.5]))),
            (1, 2): (1, AnalyticActivity(1, _pmf([0.0, 1.0], [0.5, 0.5])))}
    a_ctx = AnalyticContext(events=events, activities=acts, precedence_list=prec, step=1, underflow_rule=T,
                            overflow_rule=OT)
    mc_ctx = DagContext(events=events,
                        activities={(0, 1): Activity(idx=0, minimal_duration=0.0, activity_type=1),
                                    (1, 2): Activity(idx=1, minimal_duration=0.0, activity_type=2)},
                        precedence_list=prec, max_delay=1e6)
    gen = GenericDelayGenerator()
    gen.add_empirical_absolute(1, [1.0, 2.0], [0.5, 0.5])
    gen.add_empirical_absolute(2, [0.0, 1.0], [0.5, 0.5])
    return events, a_ctx, Simulator(mc_ctx, gen)


def test_compare_to_monte_carlo(cuda):
    """test/test_discrete_simulator.py:86-96."""
    _, a_ctx, sim = _three_event_setup()
    res = create_analytic_propagator(a_ctx).run()
    assert all(isinstance(ev, SimulatedEvent) for ev in res)
    final = res[2].pmf
    samples = [sim.run(seed=i).realized[2] for i in range(2000)]
    counts = np.bincount(np.array(samples, dtype=int))[1:4]
    mc = counts / counts.sum()
    assert np.allclose(final.values, [1.0, 2.0, 3.0])
    assert np.allclose(final.probabilities, [0.25, 0.5, 0.25], atol=0.05)
    assert np.allclose(mc, final.probabilities, atol=0.05)


def test_event_without_predecessor(cuda):
    """test/test_discrete_simulator.py:98-106."""
    events, a_ctx, sim = _three_event_setup()
    first = create_analytic_propagator(a_ctx).run()[0].pmf
    assert np.allclose(first.values, [events[0].timestamp.earliest])
    assert np.allclose(first.probabilities, [1.0])
    assert sim.run(seed=0).cause_event[0] == -1


def test_skip_validation(cuda):
    """test/test_discrete_simulator.py:147-161: a context step the activity PMF
    does not share runs when validation is off."""
    events, _, _ = _three_event_setup()
    ctx = AnalyticContext(events=events, activities={(0, 1): (0, AnalyticActivity(0, _pmf([1.0, 2.0], [0.5, 0.5])))},
                          precedence_list=((1, ((0, 0),)),), step=2, underflow_rule=T, overflow_rule=OT)
    assert len(create_analytic_propagator(ctx, validate=False).run()) == 3


def test_bounds_and_overflow(cuda):
    """test/test_discrete_simulator.py:176-201."""
    events = (Event("0", EventTimestamp(0.0, 0.0, 0.0)), Event("1", EventTimestamp(0.0, 2.0, 0.0)),
              Event("2", EventTimestamp(0.0, 1.0, 0.0)))
    ctx = AnalyticContext(events=events,
                          activities={(0, 1): (0, AnalyticActivity(0, _pmf([1.0, 2.0], [0.5, 0.5]))),
                                      (1, 2): (1, AnalyticActivity(1, _pmf([0.0, 1.0], [0.5, 0.5])))},
                          precedence_list=((1, ((0, 0),)), (2, ((1, 1),))), step=1, underflow_rule=T,
                          overflow_rule=OT)
    res = create_analytic_propagator(ctx).run()
    assert all(isinstance(ev, SimulatedEvent) for ev in res)
    assert abs(res[1].overflow) < 5e-7 and abs(res[2].overflow) < 5e-7
    assert np.allclose(res[1].pmf.values, [1.0, 2.0])
    assert np.all(res[1].pmf.values <= 2) and np.all(res[2].pmf.values <= 1)
    assert abs(res[2].pmf.probabilities.sum() - 1.0) < 5e-7


def test_rule_combinations(cuda):
    """test/test_discrete_simulator.py:203-245: half the mass below, half above
    the window [0, 1]."""
    events = (Event("0", EventTimestamp(0.0, 10.0, 0.0)), Event("1", EventTimestamp(0.0, 1.0, 0.0)))
    edge = AnalyticActivity(0, _pmf([-1.0, 0.0, 1.0, 2.0], [0.5, 0.0, 0.0, 0.5]))
    ctx = AnalyticContext(events=events, activities={(0, 1): (0, edge)}, precedence_list=((1, ((0, 0),)),), step=1,
                          underflow_rule=T, overflow_rule=OT)
    r = create_analytic_propagator(ctx).run()[1]
    assert abs(r.underflow) < 5e-7 and abs(r.overflow) < 5e-7
    assert np.allclose(r.pmf.values, [0.0, 1.0])
    create_analytic_propagator(replace(ctx, underflow_rule=RM, overflow_rule=ORM)).run()
    r1 = create_analytic_propagator(replace(ctx, underflow_rule=RM)).run()[1]
    assert abs(r1.underflow - 0.5) < 5e-7 and abs(r1.overflow) < 5e-7
    assert np.allclose(r1.pmf.values, [0.0, 1.0])
    r2 = create_analytic_propagator(replace(ctx, overflow_rule=ORM)).run()[1]
    assert abs(r2.underflow) < 5e-7 and abs(r2.overflow - 0.5) < 5e-7
    assert np.allclose(r2.pmf.values, [0.0, 1.0])


def test_large_uniform_network(cuda):
    """test/test_discrete_simulator.py:247-274: 1,981-bin uniform delays on a
    five-event network."""
    values = np.arange(-180.0, 1800.1, 1.0)
    probs = np.ones_like(values) / len(values)
    events = tuple(Event(str(i), EventTimestamp(0.0, 2000.0, 0.0)) for i in range(5))
    prec = ((1, ((0, 0),)), (2, ((0, 1),)), (3, ((1, 2), (2, 3))), (4, ((2, 4), (3, 5))))
    arcs = [(0, 1), (0, 2), (1, 3), (2, 3), (2, 4), (3, 4)]
    acts = {arc: (k, AnalyticActivity(k, DiscretePMF(values, probs, step=1))) for k, arc in enumerate(arcs)}
    ctx = AnalyticContext(events=events, activities=acts, precedence_list=prec, step=1, underflow_rule=T,
                          overflow_rule=OT)
    res = create_analytic_propagator(ctx).run()
    assert len(res) == 5
    for e in res[1:]:
        assert abs(e.pmf.step - 1.0) < 5e-7
    assert all(e.underflow >= 0.0 for e in res) and all(e.overflow >= 0.0 for e in res)


def test_run_returns_simulated_event_objects(cuda):
    """test/test_discrete_simulator.py:304-320."""
    events = (Event("0", EventTimestamp(0.0, 10.0, 0.0)), Event("1", EventTimestamp(0.0, 10.0, 0.0)))
    edge = AnalyticActivity(0, _pmf([-1.0, 0.0, 1.0, 2.0], [0.25] * 4))
    ctx = AnalyticContext(events=events, activities={(0, 1): (0, edge)}, precedence_list=((1, ((0, 0),)),), step=1,
                          underflow_rule=T, overflow_rule=OT)
    assert all(isinstance(ev, SimulatedEvent) for ev in create_analytic_propagator(ctx).run())


def _rule_case(u, o):
    """The one-edge case of test/test_discrete_simulator.py:27-44."""
    events = (Event("source", EventTimestamp(0.0, 0.0, 0.0)), Event("bounded_target", EventTimestamp(0.0, 2.0, 0.0)))
    edge = AnalyticActivity(0, _pmf([-2.0, -1.0, 0.0, 1.0, 2.0, 3.0], [0.10, 0.15, 0.20, 0.25, 0.10, 0.20]))
    ctx = AnalyticContext(events=events, activities={(0, 1): (0, edge)}, precedence_list=((1, ((0, 0),)),), step=1,
                          underflow_rule=u, overflow_rule=o)
    return create_analytic_propagator(ctx).run()[1]


RULE_TABLE = [  # test/test_discrete_simulator.py:341-416
    (T, OT, [0.45, 0.25, 0.30], 0.0, 0.0),
    (T, ORM, [0.45, 0.25, 0.10], 0.0, 0.20),
    (T, ORD, [0.5625, 0.3125, 0.1250], 0.0, 0.0),
    (RM, OT, [0.20, 0.25, 0.30], 0.25, 0.0),
    (RM, ORM, [0.20, 0.25, 0.10], 0.25, 0.20),
    (RM, ORD, [0.2727272727272727, 0.3409090909090909, 0.13636363636363635], 0.25, 0.0),
    (RD, OT, [0.26666666666666666, 0.3333333333333333, 0.4000000000000001], 0.0, 0.0),
    (RD, ORM, [0.2909090909090909, 0.36363636363636365, 0.14545454545454545], 0.0, 0.20),
    (RD, ORD, [0.36363636363636365, 0.4545454545454546, 0.18181818181818182], 0.0, 0.0),
]


@pytest.mark.parametrize("u,o,probs,under,over", RULE_TABLE)
def test_all_underflow_and_overflow_rule_combinations(cuda, u, o, probs, under, over):
    """test/test_discrete_simulator.py:419-433."""
    r = _rule_case(u, o)
    np.testing.assert_allclose(r.pmf.values, [0.0, 1.0, 2.0])
    np.testing.assert_allclose(r.pmf.probabilities, probs, rtol=0.0, atol=1e-12)
    assert float(r.underflow) == pytest.approx(under)
    assert float(r.overflow) == pytest.approx(over)


@pytest.mark.parametrize("u", list(UnderflowRule))
@pytest.mark.parametrize("o", list(OverflowRule))
def test_rule_combinations_preserve_total_mass_and_non_negative_probabilities(cuda, u, o):
    """test/test_discrete_simulator.py:436-451."""
    r = _rule_case(u, o)
    assert np.all(r.pmf.probabilities >= 0.0)
    assert np.isclose(float(r.pmf.total_mass + r.underflow + r.overflow), 1.0, rtol=1e-12, atol=1e-15)
