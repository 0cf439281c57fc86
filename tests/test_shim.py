"""The drop-in boundary (CPU, where the reference tree is present): the engine's C++ shim compiles against the
reference's src/internal.h, links with its host code (run.cpp, views.cpp, sky.cpp, solar.cpp, mesh.cpp, cli.cpp,
c_api.cpp) and, on the oracle behind the engine ABI, passes the reference's own tests/check_gpu.cpp, check_views.cpp
and check_sky.cpp unchanged."""
import os
import subprocess

import pytest

from conftest import REPO

REF = os.environ.get("KITSIM_REFERENCE") or os.path.join(os.path.dirname(REPO), "reference")
pytestmark = pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "src")), reason="reference tree not present (GPU box)")


def test_reference_checks_pass_through_the_shim():
    subprocess.check_call(["make", "-s", "-j8", "-C", os.path.join(REPO, "oracle"), "ref", "REF=" + REF])
    r = subprocess.run([os.path.join(REPO, "oracle", "_ref", "check_ref"), os.path.join(REF, "tests")], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0 and r.stdout.strip().endswith("OK: 0 failure(s)"), r.stdout[-3000:]
