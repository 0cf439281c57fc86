"""Parity of the CUDA engine with the oracle (GPU). Bit-exact for visibility bits / bytes, ray classes and distances,
reflected-light rows and every double of the reductions; the FP32 time series within 1e-5 relative of the oracle's
FP64 contraction. Inputs: the golden recordings of the reference's host code (tests/golden) and seeded scenes."""
import numpy as np
import pytest

import replay

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pair(engine_lib, oracle, kgb):
    e, o = kgb.Engine(engine_lib), kgb.Engine(oracle)
    yield e, o
    e.close()
    o.close()


def both(pair, fn):
    return fn(pair[0]), fn(pair[1])


@pytest.mark.parametrize("case", replay.cases())
def test_engine_replays_golden(engine_lib, kgb, case):
    e = kgb.Engine(engine_lib)
    try:
        assert replay.replay(e, kgb, case) == []
    finally:
        e.close()


def _scene(pkg, seed, **kw):
    return pkg.workloads.random_city(seed, **kw)


SLOTS = None


def optics_slots(kgb):
    tn = kgb.tn_from_Tn(0.64)
    s = [(0.2, 0, 0, 0), (0.3, 0.5, 0, 0), (0.0, 0.64, tn, kgb.SLOT_GLASS), (0.25, 0, 0, 0), (0.2, 0, 0, 0), (0.2, 0, 0, 0), (0.2, 0, 0, 0),
         (0.1, 0.6, 0, kgb.SLOT_THIN)]
    return s


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_bits_and_reduce_random_city(pair, pkg, kgb, seed):
    s = _scene(pkg, seed)
    D = pkg.workloads.hemisphere_dirs(145, 400, seed)
    for eng in pair:
        eng.build(s["v"], s["tri"])
        eng.set_scene(s["P"], s["N"], D)
    nc = len(s["P"])
    for cull in (False, True):
        flags = pair[0].lib.ray_flags(cull, False)
        bits = [None, None]
        for k, eng in enumerate(pair):
            eng.trace(0, nc, flags)
            bits[k] = eng.download_bits(nc)
        assert np.array_equal(bits[0], bits[1]), "%d of %d words differ" % (np.sum(bits[0] != bits[1]), bits[0].size)
        W = np.random.default_rng(seed).uniform(0.001, 2.0, len(D)).astype(np.float32)
        for use_cos in (True, False):
            r = [eng.reduce(nc, W, use_cos) for eng in pair]
            assert np.array_equal(r[0], r[1])
    # a chunk gives the bits and sums its sensors have in the whole run
    e = pair[0]
    e.trace(0, nc, pair[0].lib.ray_flags(False, False))
    whole = e.download_bits(nc)
    i0, m = nc // 3, nc // 2
    e.trace(i0, m, pair[0].lib.ray_flags(False, False))
    assert np.array_equal(e.download_bits(m), whole[:, i0:i0 + m])


@pytest.mark.parametrize("seed", [4, 5])
def test_bytes_transmission_random_city(pair, pkg, kgb, seed):
    s = _scene(pkg, seed, porous=True, glass=True, thin=True)
    D = pkg.workloads.hemisphere_dirs(145, 300, seed)
    slots = optics_slots(kgb)
    for eng in pair:
        eng.build(s["v"], s["tri"], s["slot"], slots)
        eng.set_slots(slots)
        eng.set_scene(s["P"], s["N"], D)
    nc = len(s["P"])
    for cull in (False, True):
        flags = pair[0].lib.ray_flags(cull, True)
        got = []
        for eng in pair:
            eng.trace(0, nc, flags)
            got.append(eng.download_bytes(nc))
        assert np.array_equal(got[0], got[1]), "%d of %d bytes differ" % (np.sum(got[0] != got[1]), got[0].size)
        assert 0 < np.count_nonzero((got[0] > 0) & (got[0] < 255))   # translucent crossings happened
        W = np.random.default_rng(seed).uniform(0.001, 2.0, len(D)).astype(np.float32)
        r = [eng.reduce(nc, W, True) for eng in pair]
        assert np.array_equal(r[0], r[1])
    # opaque flags on the same scene: bits, translucent slots block
    got = []
    for eng in pair:
        eng.trace(0, nc, pair[0].lib.ray_flags(False, False))
        got.append(eng.download_bits(nc))
    assert np.array_equal(got[0], got[1])


@pytest.mark.parametrize("world,cell,jitter", [(False, 2.0, True), (True, 4.0, True), (False, 3.0, False)])
def test_views_random_city(pair, pkg, kgb, world, cell, jitter):
    s = _scene(pkg, 7, glass=True)
    nt = len(s["tri"])
    rng = np.random.default_rng(11)
    label = rng.integers(2, 6, nt).astype(np.uint8)
    label[s["slot"] == 2] = kgb.LABEL_PASS   # glass passed
    fovH, lo, hi = (360.0, -70.0, 50.0) if world else (120.0, -70.0, 50.0)
    nAz, nEl = int(round(fovH / cell)), int(round((hi - lo) / cell))
    dEl = (hi - lo) / nEl
    rowSin = np.array([[np.sin(np.radians(hi - (k + 1) * dEl)), np.sin(np.radians(hi - k * dEl))] for k in range(nEl)], np.float32)
    wRow = np.array([np.radians(fovH / nAz) * (r[1] - r[0]) for r in rowSin.astype(np.float64)])
    wRow /= wRow.sum() * nAz
    nc = 700
    P, N = s["P"][:nc], s["N"][:nc]
    for eng in pair:
        eng.build(s["v"], s["tri"])
        eng.set_scene(P, N, np.zeros((0, 3), np.float32))
        eng.set_labels(label)
    flags = pair[0].lib.bounce_flags(False)
    res = []
    for eng in pair:
        eng.view(0, nc, flags, nAz, nEl, 0.0 if world else -fovH / 2, fovH / nAz, rowSin, world=world, cull=world, jitter=jitter,
                 vground=True, groundZ=float(s["v"][:, 2].min()), north=15.0)
        cls, dist = eng.download_view(nc)
        out = eng.reduce_view(nc, wRow, 6, 300.0, reach=[6.0, 20.0, 50.0], glazing=True, isoDim=3 if world else 0)
        res.append((cls, dist, out))
    (c0, d0, o0), (c1, d1, o1) = res
    assert np.array_equal(c0, c1), "%d of %d classes differ" % (np.sum(c0 != c1), c0.size)
    assert np.array_equal(d0.view(np.uint32), d1.view(np.uint32))
    assert np.any(c0 & kgb.VIEW_GLAZED)
    assert np.array_equal(o0.view(np.uint64), o1.view(np.uint64))


def test_bounce_random_city(pair, pkg, kgb):
    s = _scene(pkg, 9, porous=True, glass=True, thin=True)
    slots = optics_slots(kgb)
    D = pkg.workloads.hemisphere_dirs(10, 10, 9)
    nc = 500
    for eng in pair:
        eng.build(s["v"], s["tri"], s["slot"], slots, per_slot=True)
        eng.set_slots(slots)
        eng.set_scene(s["P"][:nc], s["N"][:nc], D)
    for mf, N in [(1, 1), (2, 3)]:
        rows = []
        for eng in pair:
            eng.bounce(0, nc, pair[0].lib.bounce_flags(False), N=N, M=128, mf=mf, north=20.0)
            rows.append(eng.download_dc(nc))
        assert np.array_equal(rows[0], rows[1]), "%d of %d coefficients differ" % (np.sum(rows[0] != rows[1]), rows[0].size)
        assert rows[0].sum() > 0
        W = np.random.default_rng(mf).uniform(0, 3, rows[0].shape[0]).astype(np.float32)
        r = [eng.reduce_dc(nc, W) for eng in pair]
        assert np.array_equal(r[0], r[1])


def test_series_fp32_within_tolerance_of_fp64(pair, pkg):
    s = _scene(pkg, 12)
    rng = np.random.default_rng(3)
    nSky, nSun, T = 145, 200, 300
    D = pkg.workloads.hemisphere_dirs(nSky, nSun, 3)
    nc = 1000
    for eng in pair:
        eng.build(s["v"], s["tri"])
        eng.set_scene(s["P"][:nc], s["N"][:nc], D)
        eng.trace(0, nc, eng.lib.ray_flags(False, False))
    args = dict(nSky=nSky, row=np.arange(nSky), wsky=rng.uniform(0.01, 0.05, nSky), S=rng.uniform(0, 300, (nSky, T)), g=rng.uniform(0, 50, T),
                G=rng.uniform(0, 1, nc), sun0=2 * nSky, sunStep=np.sort(rng.integers(0, T, nSun)), sunVec=D[2 * nSky:], sunW=rng.uniform(0, 900, nSun))
    E = [eng.series(nc, **args) for eng in pair]
    np.testing.assert_allclose(E[0], E[1], rtol=1e-5, atol=1e-3)


def test_urban_block_sampled_against_oracle(engine_lib, oracle, kgb, pkg):
    """The full urban block (~200k sensors, ~400k triangles) on the engine; a seeded sample of its sensors on the oracle."""
    s = pkg.workloads.urban_block()
    D = pkg.workloads.hemisphere_dirs(577, 600, 42)
    e, o = kgb.Engine(engine_lib), kgb.Engine(oracle)
    try:
        e.build(s["v"], s["tri"])
        e.set_scene(s["P"], s["N"], D)
        nc = len(s["P"])
        e.trace(0, nc, e.lib.ray_flags(False, False))
        bits = e.download_bits(nc)
        pick = np.sort(np.random.default_rng(5).choice(nc, 192, replace=False))
        o.build(s["v"], s["tri"])
        o.set_scene(s["P"][pick], s["N"][pick], D)
        o.trace(0, len(pick), o.lib.ray_flags(False, False))
        assert np.array_equal(bits[:, pick], o.download_bits(len(pick)))
        # sun-hours-like counts are integers, bit-exact
        W = np.zeros(len(D), np.float32)
        W[2 * 577:] = 1.0
        r = e.reduce(nc, W, False)
        assert np.array_equal(r, np.round(r))
    finally:
        e.close()
        o.close()


def test_errors_are_the_references(engine_lib, kgb, pkg):
    s = _scene(pkg, 1)
    e = kgb.Engine(engine_lib)
    try:
        e.build(s["v"], s["tri"])
        e.set_scene(s["P"][:10], s["N"][:10], pkg.workloads.hemisphere_dirs(8, 8, 1))
        with pytest.raises(kgb.KgbError, match="gpu_trace: sensor range exceeds the scene"):
            e.trace(5, 10, e.lib.ray_flags(False, False))
        e.trace(0, 10, e.lib.ray_flags(False, True))
        with pytest.raises(kgb.KgbError, match="the last trace wrote bytes"):
            e.download_bits(10)
        with pytest.raises(kgb.KgbError, match="slot"):
            e.build(s["v"], s["tri"], np.full(len(s["tri"]), 3, np.uint32), [(0.2, 0.5, 0, 0)] * 2)
        # an empty scene: every hemisphere direction is visible
        e.build(np.zeros((0, 3)), np.zeros((0, 3)))
        e.trace(0, 10, e.lib.ray_flags(False, False))
        N = s["N"][:10]
        D = pkg.workloads.hemisphere_dirs(8, 8, 1)
        W = np.ones(len(D), np.float32)   # one weight per direction (sky, ground, sun)
        up = ((N[:, 0:1] * D[None, :, 0] + N[:, 1:2] * D[None, :, 1]) + N[:, 2:3] * D[None, :, 2]) > 0
        assert np.array_equal(e.reduce(10, W, False), up.sum(axis=1).astype(np.float64))
    finally:
        e.close()
