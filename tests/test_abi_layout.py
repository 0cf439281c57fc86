"""The ctypes mirrors of the C ABI's structs (kit-sim_daylight_gb300/kgb.py) against include/kitsim_gb300.h (CPU):
a C program compiled with gcc prints each struct's size and each field's offset, and the Python binding's layout must
match field for field, so that a field added to the header (kgb_stats grows at its end) cannot leave the binding
reading the wrong bytes."""
import ctypes
import os
import subprocess

import pytest

from conftest import REPO, package

STRUCTS = {   # C struct -> the binding's class
    "kgb_slot": "Slot", "kgb_scene": "SceneHandle", "kgb_stats": "Stats", "kgb_series_in": "SeriesIn",
    "kgb_sky_step": "SkyStep", "kgb_bounce_in": "BounceIn", "kgb_view_in": "ViewIn",
    "kgb_daylight_request": "DaylightRequest", "kgb_views_request": "ViewsRequest", "kgb_series_request": "SeriesRequest",
    "kgb_mesh_info": "MeshInfo",
}


@pytest.fixture(scope="module")
def c_layout(tmp_path_factory):
    kgb = package().kgb
    d = tmp_path_factory.mktemp("abi")
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "kitsim_gb300.h"', "int main(void) {"]
    for cname, pyname in STRUCTS.items():
        cls = getattr(kgb, pyname)
        lines.append('  printf("%s size %%zu\\n", sizeof(%s));' % (cname, cname))
        for f, _ in cls._fields_:
            lines.append('  printf("%s %s %%zu\\n", offsetof(%s, %s));' % (cname, f, cname, f))
    lines += ["  return 0;", "}"]
    src = d / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = d / "layout"
    subprocess.check_call(["gcc", "-std=c11", "-I" + os.path.join(REPO, "include"), "-o", str(exe), str(src)])
    out = {}
    for line in subprocess.check_output([str(exe)], text=True).splitlines():
        a, b, v = line.split()
        out[(a, b)] = int(v)
    return out


@pytest.mark.parametrize("cname", sorted(STRUCTS))
def test_binding_matches_header(c_layout, cname):
    cls = getattr(package().kgb, STRUCTS[cname])
    assert ctypes.sizeof(cls) == c_layout[(cname, "size")], "%s: size" % cname
    for f, _ in cls._fields_:
        assert getattr(cls, f).offset == c_layout[(cname, f)], "%s.%s: offset" % (cname, f)
