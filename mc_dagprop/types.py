"""``mc_dagprop.types``: the public type aliases (the same objects as
``mc_dagprop_gb300.types``)."""
from __future__ import annotations

from mc_dagprop_gb300.types import *  # noqa: F401,F403
from mc_dagprop_gb300.types import __all__  # noqa: F401
