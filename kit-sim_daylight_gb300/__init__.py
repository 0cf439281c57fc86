"""GB300 (sm_103a) ray-cast-and-accumulate engine for kit-sim_daylight's hot path.

The engine is a CUDA library with a C ABI (include/kitsim_gb300.h) that replaces the reference's GPU contract
(src/internal.h:125-220: gpu.cu over OptiX + trace_dev.cu). This package builds it (`build()`), loads it (`load()`)
and binds it for Python (`kgb.Engine`). The reference's own host code links it through the C++ shim in
shim/daylight_gpu.cpp. There is no CPU fallback: `load()` raises when the library is missing or no GPU is present.
"""
import os
import subprocess

from . import kgb, shard, workloads  # noqa: F401
from .kgb import Engine, KgbError, Lib, Slot  # noqa: F401

ROOT = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(ROOT, "_build", "libkitsim_gb300.so")


def build(jobs=None):
    """Compiles the engine for sm_103a (make, parallel): _build/libkitsim_gb300.so."""
    jobs = jobs or max(2, min(16, os.cpu_count() or 2))
    subprocess.check_call(["make", "-s", "-j", str(jobs)], cwd=ROOT)
    return LIB_PATH


_LIB = None


def load(path=None):
    """The engine library (kgb.Lib). Raises when it was not built: the engine never falls back to the CPU."""
    global _LIB
    path = path or LIB_PATH
    if _LIB is not None and _LIB.path == path:
        return _LIB
    if not os.path.exists(path):
        raise RuntimeError("kit-sim GB300 engine library missing (%s): run build() first" % path)
    _LIB = Lib(path)
    return _LIB


def engine():
    """A new engine on the current CUDA device."""
    return Engine(load())
