"""Builds the compiled parts of mc_dagprop_gb300 in-tree (no cmake, no setuptools).

  _lib/libmcdagprop_gb300.so   CUDA kernels + C++ host runtime behind the C ABI
                               (include/mc_dagprop_gb300.h), sm_103a only
  _core<EXT_SUFFIX>            pybind11 module mirroring the reference's Python API;
                               it calls only the C ABI

Translation units compile in parallel; the whole build takes well under a minute.
pybind11 headers come from the pybind11 package when installed, else from the
copy shipped inside PyTorch's include directory.

    python mc_dagprop_gb300/_build.py [--force]     (a plain script: it must run before the package imports)
"""
from __future__ import annotations

import sys

# Run as a script, this file's directory leads sys.path, and the package's own
# modules (types.py) would shadow the standard library's.
if sys.path and sys.path[0] and __name__ == "__main__":
    sys.path.pop(0)

import os
import shutil
import subprocess
import sysconfig
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(ROOT, "_build", "mc_dagprop_gb300")
LIBDIR = os.path.join(PKG, "_lib")
LIB = os.path.join(LIBDIR, "libmcdagprop_gb300.so")
EXT = os.path.join(PKG, "_core" + sysconfig.get_config_var("EXT_SUFFIX"))
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc") if os.path.exists(os.path.join(CUDA_HOME, "bin", "nvcc")) else "nvcc"

HOST_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function"]

SOURCES_CU = ["mcd_kernels.cu", "mcd_prop_sample.cu", "mcd_prop_sample_gt.cu", "mcd_prop_given.cu", "mcd_adjoint.cu",
              "mcd_analytic.cu", "mcd_inspect.cu"]
SOURCES_CPP = ["mcd_compile.cpp", "mcd_capi.cpp", "mcd_batch.cpp", "mcd_grad.cpp", "mcd_server.cpp"]
HEADERS = ["mcd_internal.hpp", "mcd_host.hpp", "mcd_device.cuh", "mcd_handle.hpp"]


def _pybind_include() -> str:
    try:
        import pybind11  # type: ignore

        return pybind11.get_include()
    except ImportError:
        import torch  # type: ignore

        return os.path.join(os.path.dirname(torch.__file__), "include")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> None:
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    inc = ["-I" + os.path.join(ROOT, "include"), "-I" + CSRC]
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(ROOT, "include", "mc_dagprop_gb300.h")]
    cuda_inc = "-I" + os.path.join(CUDA_HOME, "include")
    jobs = []
    objs = []
    for src in SOURCES_CU:
        obj = os.path.join(BUILD, src + ".o")
        objs.append(obj)
        if force or _newer(obj, [os.path.join(CSRC, src)] + hdrs):
            jobs.append([NVCC, *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                         "-Xptxas", "-v" if verbose else "-O3", *inc, "-c", os.path.join(CSRC, src), "-o", obj])
    for src in SOURCES_CPP:
        obj = os.path.join(BUILD, src + ".o")
        objs.append(obj)
        if force or _newer(obj, [os.path.join(CSRC, src)] + hdrs):
            jobs.append(["g++", *HOST_FLAGS, cuda_inc, *inc, "-c", os.path.join(CSRC, src), "-o", obj])
    py_src = os.path.join(CSRC, "mcd_core_pybind.cpp")
    py_obj = os.path.join(BUILD, "mcd_core_pybind.o")
    if force or _newer(py_obj, [py_src] + hdrs):
        jobs.append(["g++", *HOST_FLAGS, "-fvisibility=hidden", "-I" + sysconfig.get_paths()["include"],
                     "-I" + _pybind_include(), *inc, "-c", py_src, "-o", py_obj])
    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        results = list(ex.map(_run, jobs))
    if verbose:
        for r in results:
            sys.stderr.write(r.stderr)
    if force or _newer(LIB, objs):
        _run([NVCC, *ARCH, "-shared", "-Xcompiler", "-fPIC", *objs, "-o", LIB])
    if force or _newer(EXT, [py_obj, LIB]):
        _run(["g++", "-shared", "-fPIC", py_obj, "-L" + LIBDIR, "-lmcdagprop_gb300",
              "-Wl,-rpath,$ORIGIN/_lib", "-o", EXT])


def clean() -> None:
    for p in (LIB, EXT):
        if os.path.exists(p):
            os.remove(p)
    shutil.rmtree(BUILD, ignore_errors=True)


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print("built", LIB, EXT)
