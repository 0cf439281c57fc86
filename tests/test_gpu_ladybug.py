"""Ladybug mode's sky on the GPU (kgb_sky_ladybug) against the reference's own code on the urban weather year
(tests/golden/ladybug, from oracle/ref_sky_golden.cpp; pinned to the reference's run() by tests/test_ladybug_golden.py).

The steps' sun (Radiance sun.c) and Perez skies run in FP64 on the GPU, whose elementary functions differ from the host
C library's in the last ulp; the float sums over the year then agree to about 1e-7, and the weights printed to three
significant digits agree exactly unless a sum lies within that of a printing boundary. The stated bounds: every sum
within SUM_TOL relative, every weight equal or one printed step off (a %.3g rounding flip), and the radiation an open
horizontal sensor sums from the weights within RAD_TOL relative (the criterion: ladybug radiation within 1e-6 relative)."""
import os

import numpy as np
import pytest

from replay import GOLDEN

pytestmark = pytest.mark.gpu

SUM_TOL = 1e-6
RAD_TOL = 1e-6
SERIES_TOL = 2e-6   # the series columns, per step's maximum (as the physical sky's test)


@pytest.mark.parametrize("mf", [1, 2])
def test_ladybug_sky_against_the_reference(engine_lib, kgb, mf):
    g = np.load(os.path.join(GOLDEN, "ladybug", "mf%d.npz" % mf))
    T, P, Tup, hours, lat, lon, tz = g["head"]
    T, P, Tup = int(T), int(P), int(Tup)
    e = kgb.Engine(engine_lib)
    try:
        lb, acc, S, gs = e.sky_ladybug(mf, g["steps"], lat, lon, tz, float(g["grefl"]), hours, series=True)
    finally:
        e.close()
    assert lb.shape == (3 * P + 1,) and S.shape == (P, Tup)
    ref_acc = g["acc"]
    live = ref_acc != 0
    assert np.array_equal(acc[~live], ref_acc[~live])
    sum_err = np.abs(acc[live].astype(np.float64) - ref_acc[live]) / np.abs(ref_acc[live].astype(np.float64))
    ref_lb = g["lb"]
    diff = lb != ref_lb
    flips = int(diff[:3 * P].sum())
    rad = np.abs(lb[2 * P:3 * P].sum() - ref_lb[2 * P:3 * P].sum()) / ref_lb[2 * P:3 * P].sum()
    cols = g["S"].shape[1]
    s_err = np.abs(S[:, :cols] - g["S"]).max(axis=0) / np.maximum(np.abs(g["S"]).max(axis=0), 1e-30)
    print("\nladybug mf %d: sums within %.2e (%.4f bit-identical), %d of %d weights differ, open-sensor radiation within %.2e, "
          "series within %.2e of each step's maximum (%.4f bit-identical), ground %s" %
          (mf, sum_err.max(), np.mean(acc == ref_acc), flips, 3 * P, rad, s_err.max(), np.mean(S[:, :cols] == g["S"]),
           "equal" if lb[3 * P] == ref_lb[3 * P] else "%.2e" % (abs(lb[3 * P] - ref_lb[3 * P]) / ref_lb[3 * P])))
    assert sum_err.max() <= SUM_TOL
    assert rad <= RAD_TOL
    assert flips <= max(3, 3 * P // 500)
    assert s_err.max() <= SERIES_TOL
    assert np.abs(gs[:cols] - g["g"]).max() <= SERIES_TOL * max(np.abs(g["g"]).max(), 1e-30)
