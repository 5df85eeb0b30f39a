"""pytest set-up: import paths, the `gpu` marker, and an up-to-date build.

The compiled extension and the C oracle are (re)built on collection when their
sources are newer than the binaries; the build is a no-op otherwise.
"""
from __future__ import annotations

import importlib.util
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def _ensure_built():
    spec = importlib.util.spec_from_file_location("_mcd_build", os.path.join(ROOT, "mc_dagprop_gb300", "_build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.build()
    import oracle  # noqa: E402

    oracle.build()


_ensure_built()


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300)")


def gpu_available() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def cuda():
    if not gpu_available():
        pytest.fail("a gpu-marked test ran without a CUDA device")
    import torch

    return torch.device("cuda:0")
