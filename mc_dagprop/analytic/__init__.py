"""``mc_dagprop.analytic``: the analytic PMF engine (GPU) under the reference's
package name (reference ``src/mc_dagprop/analytic/__init__.py``)."""
from __future__ import annotations

from mc_dagprop_gb300.analytic import *  # noqa: F401,F403
from mc_dagprop_gb300.analytic import __all__  # noqa: F401
