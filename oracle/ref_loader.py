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


def _ref_root() -> str:
    """Where the reference's sources are: $MCD_REFERENCE_ROOT, else the place
    oracle/build_ref.sh compiled them from (recorded next to the module)."""
    env = os.environ.get("MCD_REFERENCE_ROOT")
    if env:
        return env
    rec = os.path.join(HERE, "_ref", "REFERENCE_ROOT")
    if os.path.isfile(rec):
        with open(rec) as f:
            return f.read().strip()
    return ""


REF_ROOT = _ref_root()


def ref_so_path() -> str | None:
    hits = sorted(glob.glob(os.path.join(HERE, "_ref", "_core*.so")))
    return hits[0] if hits else None


def available() -> bool:
    return ref_so_path() is not None and os.path.isfile(
        os.path.join(REF_ROOT, "src", "mc_dagprop", "types.py"))


_LOADED: dict = {}


class _ReferenceNamespace:
    """Installs the reference's package names (`mc_dagprop`, `mc_dagprop.types`,
    ...) in sys.modules while its modules initialise, then puts back whatever held
    those names before -- e.g. this repository's own `mc_dagprop` drop-in package
    -- so both can live in one process.  The reference's modules keep the objects
    they imported while loading."""

    def __enter__(self):
        self.saved = {k: v for k, v in sys.modules.items() if k == "mc_dagprop" or k.startswith("mc_dagprop.")}
        for k in self.saved:
            del sys.modules[k]
        for k, v in _LOADED.items():
            sys.modules[k] = v
        if "mc_dagprop" not in sys.modules:
            pkg = types.ModuleType("mc_dagprop")
            pkg.__path__ = []  # namespace-like: submodules registered by hand
            sys.modules["mc_dagprop"] = pkg
        return sys.modules["mc_dagprop"]

    def __exit__(self, *exc):
        for k in [k for k in sys.modules if k == "mc_dagprop" or k.startswith("mc_dagprop.")]:
            if exc[0] is None:
                _LOADED[k] = sys.modules[k]
            del sys.modules[k]
        sys.modules.update(self.saved)
        return False


def load():
    """Return the reference's ``_core`` module (MonteCarloPropagator, DagContext, ...)."""
    name = "mc_dagprop.monte_carlo._core"
    if name in _LOADED:
        return _LOADED[name]
    so = ref_so_path()
    if so is None:
        raise ImportError("oracle/_ref is not built (run oracle/build_ref.sh)")
    pkg_dir = os.path.join(REF_ROOT, "src", "mc_dagprop")
    with _ReferenceNamespace():
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
    if name in _LOADED:
        return _LOADED[name]
    core = load()
    with _ReferenceNamespace() as root:
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
