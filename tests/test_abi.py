"""The C ABI (CPU): the engine library builds for sm_103a and exports every entry point include/kitsim_gb300.h
declares (nothing is called: no GPU here); the oracle exports the same ABI; flag values equal the reference's."""
import ctypes
import os
import re

import pytest

from conftest import REPO


def declared():
    txt = open(os.path.join(REPO, "include", "kitsim_gb300.h")).read()
    return sorted(set(re.findall(r"KGB_API\s+[\w\s\*]+?\b(kgb_\w+)\s*\(", txt)))


def test_header_declares_the_contract():
    names = declared()
    # one entry point per function of the reference's GPU contract (src/internal.h:125-220), plus version/error/dims
    for n in ["kgb_init", "kgb_destroy", "kgb_build", "kgb_build_bytes", "kgb_trim", "kgb_set_slots", "kgb_detach", "kgb_attach",
              "kgb_free_scene", "kgb_free_bytes", "kgb_set_scene", "kgb_trace", "kgb_reduce", "kgb_series", "kgb_bounce",
              "kgb_reduce_dc", "kgb_download_dc", "kgb_download_bits", "kgb_download_bytes", "kgb_set_labels", "kgb_view",
              "kgb_reduce_view", "kgb_download_view", "kgb_get_stats", "kgb_ray_flags", "kgb_bounce_flags"]:
        assert n in names


def test_engine_library_exports_every_symbol(engine_lib, kgb):
    for n in declared():
        assert hasattr(engine_lib.dll, n), n
    assert {s[0] for s in kgb.SIGNATURES} <= set(declared())
    assert engine_lib.dll.kgb_version() == 1


def test_oracle_exports_every_symbol(oracle):
    for n in declared():
        assert hasattr(oracle.dll, n), n


@pytest.mark.parametrize("which", ["engine", "oracle"])
def test_flag_values_are_the_references(which, engine_lib, oracle):
    lib = engine_lib if which == "engine" else oracle
    # tests/check_gpu.cpp:98-101 and its bounce block: 5 / 21 / 4 / 20 and 1 / 17 (pure host functions: no GPU needed)
    assert [lib.ray_flags(False, False), lib.ray_flags(True, False), lib.ray_flags(False, True), lib.ray_flags(True, True)] == [5, 21, 4, 20]
    assert [lib.bounce_flags(False), lib.bounce_flags(True)] == [1, 17]
