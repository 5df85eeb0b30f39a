"""GB300-native Monte Carlo DAG propagation, a drop-in for ``mc_dagprop``'s
Monte Carlo path (``MonteCarloPropagator.run`` / ``run_many``), with its analytic
PMF propagator (``create_analytic_propagator``) on the GPU as well.

The compiled extension (``_core`` over ``_lib/libmcdagprop_gb300.so``) is
required; there is no CPU fallback.  Build it with
``python mc_dagprop_gb300/_build.py``.
"""
from __future__ import annotations

__version__ = "0.9.0+gb300"

try:
    from .monte_carlo import (
        Activity,
        Batch,
        Server,
        DagContext,
        Event,
        EventTimestamp,
        GenericDelayGenerator,
        MonteCarloPropagator,
        SimResult,
        Simulator,
    )
except ImportError as exc:  # the compiled module is missing: fail loudly
    raise ImportError(
        "mc_dagprop_gb300 requires its compiled extension 'mc_dagprop_gb300._core' "
        "(CUDA, sm_103a). Build it with `python mc_dagprop_gb300/_build.py`."
    ) from exc

from .analytic import (  # noqa: E402
    AnalyticContext,
    AnalyticPropagator,
    DiscretePMF,
    OverflowRule,
    SimulatedEvent,
    UnderflowRule,
    create_analytic_propagator,
)

__all__ = [
    "DiscretePMF",
    "SimulatedEvent",
    "UnderflowRule",
    "OverflowRule",
    "AnalyticContext",
    "AnalyticPropagator",
    "create_analytic_propagator",
    "Batch",
    "Server",
    "GenericDelayGenerator",
    "DagContext",
    "SimResult",
    "Event",
    "Activity",
    "Simulator",
    "MonteCarloPropagator",
    "EventTimestamp",
    "__version__",
]
