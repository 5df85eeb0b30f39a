"""The ``mc_dagprop`` drop-in package imports without a GPU and exposes the
reference's module layout and names (src/mc_dagprop/__init__.py:5-49,
monte_carlo/__init__.py, types.py, core.py, analytic/__init__.py)."""
from __future__ import annotations

import importlib


def test_reference_module_layout():
    for mod in ("mc_dagprop", "mc_dagprop.monte_carlo", "mc_dagprop.monte_carlo._core", "mc_dagprop.types",
                "mc_dagprop.core", "mc_dagprop.analytic"):
        importlib.import_module(mod)
    import mc_dagprop
    import mc_dagprop_gb300

    expected = {"GenericDelayGenerator", "DagContext", "SimResult", "Event", "Activity", "Simulator",
                "MonteCarloPropagator", "EventTimestamp", "DiscretePMF", "SimulatedEvent", "UnderflowRule",
                "OverflowRule", "AnalyticContext", "AnalyticPropagator", "create_analytic_propagator", "__version__"}
    assert expected <= set(mc_dagprop.__all__)
    for name in expected - {"__version__"}:
        assert getattr(mc_dagprop, name) is getattr(mc_dagprop_gb300, name), name
    assert mc_dagprop.Simulator is mc_dagprop.MonteCarloPropagator
    assert mc_dagprop.MonteCarloPropagator.__name__ == "MonteCarloPropagator"
    assert mc_dagprop.__version__.startswith("0.9.0")


def test_types_and_core_names():
    import mc_dagprop.core as core
    import mc_dagprop.types as T

    assert set(T.__all__) == {"Second", "ProbabilityMass", "ActivityIndex", "EventIndex", "ActivityType", "EventId"}
    assert T.Second(1.5) == 1.5 and T.EventId("x") == "x"
    assert set(core.__all__) == {"EventTimestamp", "Event", "Activity", "DagContext"}
    ts = core.EventTimestamp(0.0, 1.0, 0.5)
    assert repr(ts).startswith("EventTimestamp(")


def test_reference_loader_coexists_with_dropin():
    """Loading the reference's own module for the oracle pin tests leaves this
    package's `mc_dagprop` names in place."""
    import ref_loader

    import mc_dagprop
    import mc_dagprop.types

    before = (mc_dagprop, mc_dagprop.types)
    if ref_loader.available():
        ref = ref_loader.load()
        assert ref.MonteCarloPropagator is not mc_dagprop.MonteCarloPropagator
    import sys

    assert (sys.modules["mc_dagprop"], sys.modules["mc_dagprop.types"]) == before
