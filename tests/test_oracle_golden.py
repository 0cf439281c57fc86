"""The oracle against the golden fixtures (CPU): recordings of the reference's host code at the engine boundary
replay on the oracle bit for bit (on any host: x86 here, Arm on the GPU machine), and the recorded runs equal the
reference's published outputs for tests/box.obj."""
import json
import os

import numpy as np
import pytest

import replay

GOLDEN = replay.GOLDEN


@pytest.mark.parametrize("case", replay.cases())
def test_oracle_replays_recording(oracle, kgb, case):
    e = kgb.Engine(oracle)
    try:
        assert replay.replay(e, kgb, case) == []
    finally:
        e.close()


def test_recorded_runs_match_published_outputs():
    pub = json.load(open(os.path.join(GOLDEN, "published.json")))
    assert set(pub) == {"box_clearsky", "box_sunhours_day", "box_views"}
    for case, p in pub.items():
        got = np.load(os.path.join(GOLDEN, case, "result.npy"))
        cols = json.load(open(os.path.join(GOLDEN, case, "manifest.json")))["columns"]
        want = np.array(p["values"])
        assert got.shape[0] == want.shape[0] == 16
        for k, c in enumerate(p["columns"]):
            g, w = got[:, cols.index(c)], want[:, k]
            if c.startswith("sunhours"):
                np.testing.assert_allclose(g, w, rtol=1e-8, atol=1e-7)   # printed to 10 digits: the counts exactly
            else:
                np.testing.assert_allclose(g, w, rtol=2e-7, atol=1e-9)   # the docs print 10 significant digits


def test_box_clearsky_sunhours_are_integer_counts():
    got = np.load(os.path.join(GOLDEN, "box_clearsky", "result.npy"))
    cols = json.load(open(os.path.join(GOLDEN, "box_clearsky", "manifest.json")))["columns"]
    sh = got[:, cols.index("sunhours_front")]
    assert np.array_equal(sh, np.round(sh)) and sh.max() == 4456
