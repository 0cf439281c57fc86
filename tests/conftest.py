"""Shared fixtures. `gpu` marks tests that need a CUDA device (the engine); the rest run on the CPU."""
import importlib.util
import os
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def package():
    """The engine package (its directory name has a hyphen, so it is loaded by path)."""
    if "kitsim_gb300" in sys.modules:
        return sys.modules["kitsim_gb300"]
    d = os.path.join(REPO, "kit-sim_daylight_gb300")
    spec = importlib.util.spec_from_file_location("kitsim_gb300", os.path.join(d, "__init__.py"), submodule_search_locations=[d])
    m = importlib.util.module_from_spec(spec)
    sys.modules["kitsim_gb300"] = m
    spec.loader.exec_module(m)
    return m


ORACLE_SO = os.path.join(REPO, "oracle", "_build", "liboracle.so")


def oracle_lib():
    """The oracle (the checker), built from oracle/ on first use."""
    subprocess.check_call(["make", "-s", "-C", os.path.join(REPO, "oracle"), "all"])
    return package().kgb.Lib(ORACLE_SO)


@pytest.fixture(scope="session")
def pkg():
    return package()


@pytest.fixture(scope="session")
def kgb(pkg):
    return pkg.kgb


@pytest.fixture(scope="session")
def oracle():
    return oracle_lib()


@pytest.fixture(scope="session")
def engine_lib(pkg):
    """The CUDA engine: built if needed; on a machine without a GPU the gpu tests are not collected to run here."""
    if not os.path.exists(pkg.LIB_PATH):
        pkg.build()
    return pkg.load()
