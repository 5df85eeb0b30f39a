"""Loads the reference's own compiled Monte Carlo module (test infrastructure only).

``oracle/build_ref.sh`` compiles ``src/mc_dagprop/monte_carlo/_core.cpp`` of the
reference into ``oracle/_ref/``.  The compiled module imports ``mc_dagprop.types``
at initialisation (``_core.cpp:453``), so this loader registers a minimal
``mc_dagprop`` package whose ``types`` submodule is the reference's own file,
then loads the extension under its real name ``mc_dagprop.monte_carlo._core``.
No reference source is copied.

Only tests, the golden-fixture script and the CPU baseline may use this module.
"""
from __future__ import annotations

import glob
import importlib.machinery
import importlib.util
import os
import sys
import types

HERE = os.path.dirname(os.path.abspath(__file__))
REF_ROOT = os.environ.get("MCD_REFERENCE_ROOT", "/root/reference")


def ref_so_path() -> str | None:
    hits = sorted(glob.glob(os.path.join(HERE, "_ref", "_core*.so")))
    return hits[0] if hits else None


def available() -> bool:
    return ref_so_path() is not None and os.path.isfile(
        os.path.join(REF_ROOT, "src", "mc_dagprop", "types.py"))


def load():
    """Return the reference's ``_core`` module (MonteCarloPropagator, DagContext, ...)."""
    name = "mc_dagprop.monte_carlo._core"
    if name in sys.modules:
        return sys.modules[name]
    so = ref_so_path()
    if so is None:
        raise ImportError("oracle/_ref is not built (run oracle/build_ref.sh)")
    pkg_dir = os.path.join(REF_ROOT, "src", "mc_dagprop")
    if "mc_dagprop" not in sys.modules:
        pkg = types.ModuleType("mc_dagprop")
        pkg.__path__ = []  # namespace-like: submodules registered by hand below
        sys.modules["mc_dagprop"] = pkg
    spec = importlib.util.spec_from_file_location("mc_dagprop.types", os.path.join(pkg_dir, "types.py"))
    tmod = importlib.util.module_from_spec(spec)
    sys.modules["mc_dagprop.types"] = tmod
    spec.loader.exec_module(tmod)
    mc = types.ModuleType("mc_dagprop.monte_carlo")
    mc.__path__ = []
    sys.modules["mc_dagprop.monte_carlo"] = mc
    loader = importlib.machinery.ExtensionFileLoader(name, so)
    spec = importlib.util.spec_from_file_location(name, so, loader=loader)
    core = importlib.util.module_from_spec(spec)
    sys.modules[name] = core
    loader.exec_module(core)
    mc._core = core
    return core


def load_analytic():
    """Return the reference's pure-Python analytic package ``mc_dagprop.analytic``
    (loaded from its sources; it imports ``Event`` from the package root, which is
    the compiled module's class)."""
    name = "mc_dagprop.analytic"
    if name in sys.modules:
        return sys.modules[name]
    core = load()
    root = sys.modules["mc_dagprop"]
    for attr in ("Event", "EventTimestamp", "Activity", "DagContext", "GenericDelayGenerator", "SimResult"):
        if hasattr(core, attr):
            setattr(root, attr, getattr(core, attr))
    pkg_dir = os.path.join(REF_ROOT, "src", "mc_dagprop", "analytic")
    spec = importlib.util.spec_from_file_location(name, os.path.join(pkg_dir, "__init__.py"),
                                                  submodule_search_locations=[pkg_dir])
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    root.analytic = mod
    return mod
