"""The GPU FP64 sky (kgb_sky: the Perez all-weather sky + AddDirect per step and patch; kgb_sun_noaa) against the
reference's own src/sky.cpp gendaymtx_step and src/solar.cpp sun_noaa on the same inputs (tests/golden/sky, written by
the reference code compiled in oracle/). FP64 elementary functions differ between CUDA and the host C library in the
last ulp; the float outputs are compared to a few float ulps and the bit-identical share is reported."""
import json
import os

import numpy as np
import pytest

from replay import GOLDEN

pytestmark = pytest.mark.gpu
SKY = os.path.join(GOLDEN, "sky")


@pytest.fixture(scope="module")
def eng(engine_lib, kgb):
    e = kgb.Engine(engine_lib)
    yield e
    e.close()


def test_sun_positions(eng):
    idx = json.load(open(os.path.join(SKY, "index.json")))["sun"]
    rows = np.fromfile(os.path.join(SKY, idx["in"]), np.float64).reshape(-1, 7)
    want = np.fromfile(os.path.join(SKY, idx["out"]), np.float64).reshape(-1, 6)
    got = eng.sun_noaa(rows)
    np.testing.assert_allclose(got[:, 0], want[:, 0], rtol=0, atol=1e-9)           # altitude, degrees
    daz = np.abs(got[:, 1] - want[:, 1])
    assert np.max(np.minimum(daz, 360 - daz)) < 1e-8                                 # azimuth, degrees
    assert np.array_equal(got[:, 2], want[:, 2])                                      # up
    np.testing.assert_allclose(got[:, 3:], want[:, 3:], rtol=0, atol=2e-7)          # float direction
    print("\nsun: %d positions, max |d alt| %.2e deg, identical directions %.4f" %
          (len(rows), np.abs(got[:, 0] - want[:, 0]).max(), np.mean(np.all(got[:, 3:] == want[:, 3:], axis=1))))


@pytest.mark.parametrize("case", json.load(open(os.path.join(SKY, "index.json")))["sky"], ids=lambda c: c["out"])
def test_sky_matrix(eng, case):
    steps = np.fromfile(os.path.join(SKY, case["in"]), np.float64).reshape(-1, 5)
    P = 144 * case["mf"] ** 2 + 1
    want = np.fromfile(os.path.join(SKY, case["out"]), np.float32).reshape(-1, P + 1, 3)
    got = eng.sky(case["mf"], steps, grefl=case["grefl"], sun=bool(case["sun"]), sky=bool(case["sky"]), visible=bool(case["visible"]))
    scale = np.maximum(np.abs(want).max(axis=(1, 2), keepdims=True), 1e-30)   # per step
    err = np.abs(got - want) / scale
    same = np.mean(got == want)
    print("\n%s: max error %.2e of the step's maximum, %.4f of the values bit-identical" % (case["out"], err.max(), same))
    assert err.max() <= 2e-6
    assert same > 0.9
