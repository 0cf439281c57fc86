"""Parity at the measured configurations' full scale (GPU): the engine runs the whole scene, the oracle a seeded sample
of it at the same global sensor indices (so the same jitter and path seeds), and every result must agree.

 - views city (the views configuration: 50k facade sensors, 2 M triangles, 3 target groups): fov 120 and fov 360 at
   2 degree cells, jitter on, isovist volume and reach 6 / 20 / 50 at fov 360; classes and distances bit for bit on
   512 sensors, and every double of gpu_reduce_view, both on those chunks and as rows of one whole-city launch;
 - precision configuration (the urban block at 2305 patches + ground, 20 % glass in byte mode, one bounce of 1024 paths
   per sensor, the hourly series of the non-night hours with reflected light): transmittance bytes, reflected-light
   rows and the ground reduce bit for bit on a 1024-sensor chunk, and the split-BF16 series against the oracle's FP64
   contraction, per output (elementwise) and per column;
 - urban block (the headline configuration) with the reference's own direction table and weights: bits and the four
   reduces of 256 sampled sensors bit for bit."""
import os

import numpy as np
import pytest

import replay

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
# the series against FP64 (the criterion: within 1e-6 relative, stated per output column)
COLUMN_TOL = 1e-6          # per column: max_i |E - E64| / max_i |E64|
ELEMENT_TOL = 1e-6         # per output: |E - E64| / E64 over outputs above ELEMENT_FLOOR x their column's maximum
ELEMENT_P99_TOL = 5e-7
ELEMENT_FLOOR = 1e-6


@pytest.fixture(scope="module")
def city(pkg):
    return pkg.workloads.views_city()


def test_views_city_full_scale(engine_lib, oracle, kgb, pkg, city):
    nc_all = len(city["P"])
    assert nc_all >= 50_000 and len(city["tri"]) >= 1_900_000
    e, o = kgb.Engine(engine_lib), kgb.Engine(oracle)
    starts = np.sort(np.random.default_rng(17).choice(nc_all // 64, 8, replace=False)) * 64
    try:
        for x in (e, o):
            x.build(city["v"], city["tri"])
            x.set_labels(city["label"])
            x.set_scene(city["P"], city["N"], np.zeros((0, 3), np.float32))
        flags = engine_lib.bounce_flags(False)
        for fov, world, reach, iso in ((120.0, False, [], 0), (360.0, True, [6.0, 20.0, 50.0], 3)):
            nAz, nEl, dAz, rowSin, wRow = pkg.workloads.views_grid(fov, 2.0)
            kw = dict(world=world, cull=world, jitter=True, vground=True, groundZ=city["groundZ"])
            az0 = 0.0 if world else -fov / 2
            # the whole city in one call on the engine: its sums, kept for the sampled rows
            e.view(0, nc_all, flags, nAz, nEl, az0, dAz, rowSin, **kw)
            whole = e.reduce_view(nc_all, wRow, 6, 1000.0, reach=reach, isoDim=iso)
            for i0 in starts:
                got = []
                for x in (e, o):
                    x.view(int(i0), 64, flags, nAz, nEl, az0, dAz, rowSin, **kw)
                    cls, dist = x.download_view(64)
                    got.append((cls, dist, x.reduce_view(64, wRow, 6, 1000.0, reach=reach, isoDim=iso)))
                (c0, d0, r0), (c1, d1, r1) = got
                assert np.array_equal(c0, c1), "fov %g sensors %d+: %d of %d classes differ" % (fov, i0, np.sum(c0 != c1), c0.size)
                assert np.array_equal(d0.view(np.uint32), d1.view(np.uint32)), "fov %g sensors %d+: distances differ" % (fov, i0)
                assert np.array_equal(r0.view(np.uint64), r1.view(np.uint64)), "fov %g sensors %d+: view sums differ" % (fov, i0)
                assert np.array_equal(whole[i0:i0 + 64].view(np.uint64), r1.view(np.uint64)), "fov %g: the whole-city launch differs" % fov
            classes = np.unique(c0 & 0x7F)
            assert {0, 1, 2} <= set(classes.tolist())   # sky, ground and obstructions all occur
    finally:
        e.close()
        o.close()


@pytest.fixture(scope="module")
def precision_inputs(engine_lib, kgb, pkg):
    """The precision configuration's scene, directions and series inputs (sky built on the GPU, as the bench does)."""
    e = kgb.Engine(engine_lib)
    try:
        mf = 4
        Dsky, omega = pkg.workloads.patch_dirs(mf)
        yr = pkg.workloads.urban_year_sky(e, mf, np.load(os.path.join(GOLDEN, "urban_sky", "weather.npy")))
    finally:
        e.close()
    P = len(Dsky)
    D = np.concatenate([Dsky, -Dsky, yr["sunVec"]]).astype(np.float32)
    scene = pkg.workloads.urban_block(glass_share=0.2)
    slots = [(0.2, 0, 0, 0), (0.0, 0.64, kgb.tn_from_Tn(0.64), kgb.SLOT_GLASS), (0.2, 0, 0, 0)]
    Wg = np.zeros(len(D), np.float32)
    Wg[P:2 * P] = omega
    sargs = dict(nSky=P, row=np.arange(P), wsky=omega, S=yr["S"], g=yr["g"], sun0=2 * P, sunStep=yr["sunStep"], sunVec=yr["sunVec"],
                 sunW=yr["sunW"], Sdc=yr["Sdc"])
    return dict(scene=scene, slots=slots, D=D, Wg=Wg, sargs=sargs, P=P, T=yr["T"])


def series_errors(E, E64):
    """Per-column normwise error and per-output relative error of E against E64 (outputs at or above ELEMENT_FLOOR x
    their column's maximum; every term of the contraction is non-negative, so no output is a cancellation)."""
    E, E64 = E.astype(np.float64), E64.astype(np.float64)
    cmax = np.abs(E64).max(axis=0)
    live = cmax > 0
    col = (np.abs(E - E64).max(axis=0)[live] / cmax[live])
    mask = (E64 > 0) & (E64 >= ELEMENT_FLOOR * cmax[None, :])
    rel = np.abs(E - E64)[mask] / E64[mask]
    return dict(column_max=float(col.max()), element_max=float(rel.max()), element_p99=float(np.percentile(rel, 99)),
                element_median=float(np.median(rel)), outputs=int(mask.sum()), columns=int(live.sum()))


def test_precision_config_chunk(engine_lib, oracle, kgb, precision_inputs):
    pi = precision_inputs
    s, D = pi["scene"], pi["D"]
    assert len(s["P"]) > 190_000 and len(D) > 9000
    nc = 1024
    i0 = int(np.random.default_rng(23).integers(0, len(s["P"]) - nc))
    res = []
    for lib in (engine_lib, oracle):
        x = kgb.Engine(lib)
        try:
            x.build(s["v"], s["tri"], s["slot"], pi["slots"], per_slot=True)
            x.set_slots(pi["slots"])
            x.set_scene(s["P"], s["N"], D)
            x.trace(i0, nc, lib.ray_flags(False, True))
            byt = x.download_bytes(nc)
            x.bounce(i0, nc, lib.bounce_flags(False), N=1, M=1024, mf=4, north=0.0)
            dc = x.download_dc(nc)
            G = x.reduce(nc, pi["Wg"], True)
            E = x.series(nc, G=G.astype(np.float32), **pi["sargs"])
            res.append((byt, dc, G, E))
        finally:
            x.close()
    (b0, dc0, G0, E0), (b1, dc1, G1, E1) = res
    assert np.array_equal(b0, b1), "%d of %d transmittance bytes differ" % (np.sum(b0 != b1), b0.size)
    assert np.count_nonzero((b0 > 0) & (b0 < 255)) > 0   # glass crossings happened
    assert np.array_equal(dc0, dc1), "%d of %d reflected-light coefficients differ" % (np.sum(dc0 != dc1), dc0.size)
    assert np.array_equal(G0.view(np.uint64), G1.view(np.uint64))
    err = series_errors(E0, E1)
    print("precision chunk: split-BF16 series against FP64:", err)
    assert err["outputs"] > 0.5 * E0.size
    assert err["column_max"] <= COLUMN_TOL, err
    assert err["element_max"] <= ELEMENT_TOL, err
    assert err["element_p99"] <= ELEMENT_P99_TOL, err


def test_urban_block_recorded_directions(engine_lib, oracle, kgb, pkg):
    """The full urban block on the engine with the reference's own direction table and its four quantities' weights
    (tests/golden/urban_sky); 256 seeded sensors on the oracle: bits and every reduce double equal."""
    s = pkg.workloads.urban_block()
    D, Ws = replay.urban_sky()
    assert len(D) == 5610 and len(Ws) == 4
    e, o = kgb.Engine(engine_lib), kgb.Engine(oracle)
    try:
        e.build(s["v"], s["tri"])
        e.set_scene(s["P"], s["N"], D)
        nc = len(s["P"])
        flags = engine_lib.ray_flags(False, False)
        e.trace(0, nc, flags)
        bits = e.download_bits(nc)
        sums = [e.reduce(nc, W, c) for W, c in Ws]
        pick = np.sort(np.random.default_rng(5).choice(nc, 256, replace=False))
        o.build(s["v"], s["tri"])
        o.set_scene(s["P"][pick], s["N"][pick], D)
        o.trace(0, len(pick), flags)
        assert np.array_equal(bits[:, pick], o.download_bits(len(pick)))
        for (W, c), full in zip(Ws, sums):
            assert np.array_equal(full[pick].view(np.uint64), o.reduce(len(pick), W, c).view(np.uint64))
        sunhours = sums[3]
        assert np.array_equal(sunhours, np.round(sunhours))   # hourly sun hours are integer counts
    finally:
        e.close()
        o.close()
