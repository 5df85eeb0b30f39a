"""``mc_dagprop.analytic``: the analytic PMF engine (GPU) under the reference's
package name (reference ``src/mc_dagprop/analytic/__init__.py``).  The
reference's submodules (``_context``, ``_pmf``, ``_propagator``,
``distributions``) resolve to this package's modules of the same names, so
imports such as ``from mc_dagprop.analytic._pmf import DiscretePMF`` work too."""
from __future__ import annotations

import sys

from mc_dagprop_gb300.analytic import *  # noqa: F401,F403
from mc_dagprop_gb300.analytic import __all__  # noqa: F401
from mc_dagprop_gb300.analytic import _context, _pmf, _propagator, distributions

for _m in (_context, _pmf, _propagator, distributions):
    sys.modules.setdefault(__name__ + "." + _m.__name__.rsplit(".", 1)[1], _m)
del _m
