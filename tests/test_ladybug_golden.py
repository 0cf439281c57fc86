"""Ladybug mode's sky goldens (CPU): the weights that tests/golden/ladybug/mf2.npz holds (the reference's own functions
driven by oracle/ref_sky_golden.cpp in ladybug mode) are the ones the reference's run() puts into its gpu_reduce calls
in ladybug mode on the same weather year (tests/golden/urban_ladybug, recorded at the engine boundary): radiation =
skyRad per sky direction and gndLB per ground direction, direct = skyDirLB and no ground, diffuse = skyDifLB and gndLB
(src/run.cpp:491-505), every value the float of the golden double, bit for bit."""
import os

import numpy as np

import replay

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_ladybug_goldens_are_the_references_weights():
    g = np.load(os.path.join(GOLDEN, "ladybug", "mf2.npz"))
    P = int(g["head"][1])
    lb = g["lb"]
    calls, arr = replay.load_calls("urban_ladybug")
    last = max(i for i, c in enumerate(calls) if c["call"] == "gpu_set_scene")
    D = arr(calls[last], "D").reshape(-1, 3)
    Ws = [arr(c, "W") for c in calls[last:] if c["call"] == "gpu_reduce"]
    assert P == 577 and len(Ws) == 3 and len(D) >= 2 * P
    rad, direct, diffuse = Ws
    f = lambda x: np.asarray(x, np.float64).astype(np.float32)
    assert np.array_equal(rad[:P], f(lb[2 * P:3 * P])) and np.all(rad[P:2 * P] == f(lb[3 * P]))
    assert np.array_equal(direct[:P], f(lb[:P])) and np.all(direct[P:2 * P] == 0)
    assert np.array_equal(diffuse[:P], f(lb[P:2 * P])) and np.all(diffuse[P:2 * P] == f(lb[3 * P]))
    for W in Ws:
        assert np.all(W[2 * P:] == 0)   # ladybug mode bins the sun into the sky patches: no sun directions weighted
    # the accumulators behind them: direct light on some patches, diffuse on all; the ground row is lit by the sky
    # pass only (gendaymtx -d leaves it dark)
    acc = g["acc"]
    assert acc[:P].max() > 0 and np.all(acc[P:4 * P] > 0) and np.all(acc[4 * P:4 * P + 3] == 0) and np.all(acc[4 * P + 3:] > 0)
