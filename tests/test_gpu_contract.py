"""The stateful parts of the GPU contract on the CUDA engine (GPU), restating the reference's own checks of them at the
engine's C ABI: the adaptive sub-launch policy and its stats (tests/check_gpu.cpp:230-246: 5000 sensors, exactly two
launches), the build-memory estimate (check_gpu.cpp:124-127), resident scenes parked and attached without a rebuild
(check_gpu.cpp:692-728, run()'s sceneKey and residentScenes on top of gpu_detach / gpu_attach / gpu_free), cancel
between sub-launches of gpu_bounce and gpu_view (gpu.cu:554, 594; check_gpu.cpp:730-734), the per-run stats
(check_gpu.cpp:790-797), and the engine's bounded-execution limits driven to their error returns."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def box_scene():
    """check_gpu.cpp:103-119: ground [-2, 2]^2 at z = 0 and the box [0.5, 1.5]^3, every face outward, quads as two
    triangles (0-1-2, 0-2-3, the reference's triangulation)."""
    lo, hi = 0.5, 1.5
    quads = [[(-2, -2, 0), (2, -2, 0), (2, 2, 0), (-2, 2, 0)],
             [(lo, lo, lo), (lo, hi, lo), (hi, hi, lo), (hi, lo, lo)], [(lo, lo, hi), (hi, lo, hi), (hi, hi, hi), (lo, hi, hi)],
             [(lo, lo, lo), (lo, lo, hi), (lo, hi, hi), (lo, hi, lo)], [(hi, lo, lo), (hi, hi, lo), (hi, hi, hi), (hi, lo, hi)],
             [(lo, lo, lo), (hi, lo, lo), (hi, lo, hi), (lo, lo, hi)], [(lo, hi, lo), (lo, hi, hi), (hi, hi, hi), (hi, hi, lo)]]
    v, tri = [], []
    for q in quads:
        b = len(v)
        v += q
        tri += [(b, b + 1, b + 2), (b, b + 2, b + 3)]
    return np.array(v, np.float32), np.array(tri, np.uint32)


def box_dirs():
    """check_gpu.cpp:134-143: 145 'patches' (7 rows of uniform azimuth + zenith), then zenith, near-horizontal, nadir."""
    D = []
    for r, n in enumerate([30, 30, 24, 24, 18, 12, 6]):
        alt = np.radians(6 + 12 * r)
        for j in range(n):
            az = 2 * np.pi * j / n
            D.append((np.cos(alt) * np.sin(az), np.cos(alt) * np.cos(az), np.sin(alt)))
    D.append((0, 0, 1))
    D.append((0, 0, 1))
    h = np.array([0.999, 0, 0.0447])
    D.append(tuple(h / np.linalg.norm(h)))
    D.append((0, 0, -1))
    return np.array(D, np.float32)


SENS_P = np.array([(1, 1, 0), (-1, -1, 0), (-1, -1, 0), (1, 1, 2), (1, 1, 1)], np.float32)
SENS_N = np.array([(0, 0, 1), (0, 0, 1), (0, 0, -1), (0, 0, -1), (0, 0, 1)], np.float32)


def hits_box(o, d, lo=0.5, hi=1.5):
    """check_gpu.cpp:82-90: the slab test of a ray from o along d against [lo, hi]^3, t > 0, in double."""
    t0, t1 = 0.0, 1e30
    with np.errstate(divide="ignore", invalid="ignore"):
        for a in range(3):
            ta, tb = (lo - float(o[a])) / float(d[a]) if d[a] else np.copysign(np.inf, lo - float(o[a])), \
                (hi - float(o[a])) / float(d[a]) if d[a] else np.copysign(np.inf, hi - float(o[a]))
            ta, tb = min(ta, tb), max(ta, tb)
            t0, t1 = max(t0, ta), min(t1, tb)
    return t0 <= t1


def dotf(n, d):
    """The reference's dotf (gpu.cu:69-72): per-operation float rounding, no fused multiply-add."""
    n, d = np.float32(n), np.float32(d)
    return np.float32(np.float32(np.float32(n[0] * d[0]) + np.float32(n[1] * d[1])) + np.float32(n[2] * d[2]))


@pytest.fixture
def eng(engine_lib, kgb):
    e = kgb.Engine(engine_lib)
    yield e
    e.close()


def test_box_bits_launch_policy_and_stats(eng, engine_lib):
    v, tri = box_scene()
    D = box_dirs()
    nDir, nWords = len(D), (len(D) + 31) // 32
    assert (len(tri), nDir, nWords) == (14, 148, 5)
    eng.build(v, tri)
    st = eng.stats()
    assert st["gasBytes"] > 0
    # the build estimate covers what the build made (the reference's VRAM admission rests on it)
    est = eng.build_bytes(len(v), len(tri))
    assert est >= st["gasBytes"] and est >= st["buildOutputBytes"]
    assert eng.build_bytes(0, 0) == 0
    eng.set_scene(SENS_P, SENS_N, D)
    flags = engine_lib.ray_flags(False, False)
    eng.trace(0, 5, flags)
    bits = eng.download_bits(5)
    bit = lambda i, d: (int(bits[d // 32, i]) >> (d % 32)) & 1
    Z, H, NA = 145, 146, 147
    assert (bit(0, Z), bit(0, H), bit(1, Z), bit(1, NA), bit(2, NA), bit(2, Z), bit(3, NA), bit(4, Z)) == (0, 1, 1, 0, 1, 0, 0, 0)
    for d in range(nDir):   # every bit of s0 and s1 against the slab test (s1 never sees the box)
        for i in (0, 1):
            want = 1 if dotf(SENS_N[i], D[d]) > 0 and not hits_box(SENS_P[i], D[d]) else 0
            assert bit(i, d) == want, (i, d)
    # 5000 copies of s1: the adaptive sub-launch path (4096 + 904 sensors), exactly two launches, every word s1's
    ref = bits[:, 1].copy()
    eng.set_scene(np.repeat(SENS_P[1:2], 5000, 0), np.repeat(SENS_N[1:2], 5000, 0), D)
    before = eng.stats()
    eng.trace(0, 5000, flags)
    after = eng.stats()
    assert after["launches"] - before["launches"] == 2
    assert after["rays"] - before["rays"] == 5000 * nDir
    assert after["traceMs"] > before["traceMs"]
    many = eng.download_bits(5000)
    assert np.array_equal(many, np.repeat(ref[:, None], 5000, 1))


def test_resident_scenes_park_attach_free(eng, engine_lib, pkg):
    """Scene A traced, parked; scene B built and traced; A attached again gives A's bits with no rebuild (build time
    and gas bytes unchanged); B freed returns its memory; an empty handle attaches as an empty scene."""
    a, b = pkg.workloads.random_city(21, n_boxes=200), pkg.workloads.random_city(22, n_boxes=300)
    D = pkg.workloads.hemisphere_dirs(145, 200, 21)
    P, N = a["P"][:2000], a["N"][:2000]
    flags = engine_lib.ray_flags(False, False)
    eng.build(a["v"], a["tri"])
    gas_a = eng.stats()["gasBytes"]
    eng.set_scene(P, N, D)
    eng.trace(0, len(P), flags)
    bits_a = eng.download_bits(len(P))
    sa = eng.detach()
    assert sa.bytes == gas_a and eng.stats()["gasBytes"] == 0
    eng.build(b["v"], b["tri"])
    gas_b = eng.stats()["gasBytes"]
    eng.trace(0, len(P), flags)
    bits_b = eng.download_bits(len(P))
    assert not np.array_equal(bits_a, bits_b)
    sb = eng.detach()
    built = eng.stats()["buildMs"]
    eng.attach(sa)
    assert eng.stats()["gasBytes"] == gas_a and eng.stats()["buildMs"] == built   # attached, not rebuilt
    eng.trace(0, len(P), flags)
    assert np.array_equal(eng.download_bits(len(P)), bits_a)
    free0 = engine_lib.dll.kgb_free_bytes()
    eng.free_scene(sb)
    assert sb.handle is None and sb.bytes == 0
    assert engine_lib.dll.kgb_free_bytes() >= free0 + gas_b // 2   # its device memory went back
    eng.free_scene(sb)   # freeing an empty handle is a no-op
    # an engine whose scene was detached traces an empty scene: every culled-in direction visible
    sa2 = eng.detach()
    eng.trace(0, len(P), flags)
    up = ((N[:, None, 0] * D[None, :, 0] + N[:, None, 1] * D[None, :, 1]) + N[:, None, 2] * D[None, :, 2]) > 0   # float32, in order
    got = eng.download_bits(len(P))
    vis = np.array([[(int(got[d // 32, i]) >> (d % 32)) & 1 for d in range(len(D))] for i in range(0, len(P), 97)])
    assert np.array_equal(vis, up[::97].astype(int))
    eng.attach(sa2)
    eng.trace(0, len(P), flags)
    assert np.array_equal(eng.download_bits(len(P)), bits_a)


def test_build_estimate_covers_the_build(eng, pkg):
    """gpu_build_bytes (internal.h:136) covers a build's peak: the device builder's temporaries plus its output, for
    scenes from a few hundred to a few hundred thousand triangles, opaque and slotted."""
    for seed, boxes in ((31, 20), (32, 400), (33, 3000)):
        s = pkg.workloads.random_city(seed, n_boxes=boxes, porous=True)
        for slotted in (False, True):
            if slotted:
                eng.build(s["v"], s["tri"], s["slot"], [(0.2, 0, 0, 0), (0.3, 0.5, 0, 0)] + [(0.2, 0, 0, 0)] * 8, per_slot=True)
            else:
                eng.build(s["v"], s["tri"])
            st = eng.stats()
            est = eng.build_bytes(len(s["v"]), len(s["tri"]), slotted)
            assert est >= st["buildTempBytes"] + st["buildOutputBytes"], (seed, slotted, est, st)


class Countdown:
    """A cancel hook that fires at its k-th check (the reference's atomic flag, set while the call runs)."""

    def __init__(self, k):
        self.k, self.checks = k, 0

    def __call__(self):
        self.checks += 1
        return self.checks >= self.k


def test_cancel_between_bounce_launches(eng, engine_lib, pkg, kgb):
    s = pkg.workloads.random_city(41, n_boxes=300)
    nc = 20000
    eng.build(s["v"], s["tri"], np.zeros(len(s["tri"]), np.uint32), [(0.3, 0, 0, 0)], per_slot=True)
    eng.set_scene(s["P"][:nc], s["N"][:nc], pkg.workloads.hemisphere_dirs(10, 0, 41))
    flags = engine_lib.bounce_flags(False)
    eng.bounce(0, nc, flags, N=1, M=256, mf=1)
    whole = eng.download_dc(nc)
    launches = eng.stats()["bounceLaunches"]
    assert launches >= 2   # more than one launch: there is a check between launches to cancel at
    for k in (1, 2):
        hook = Countdown(k)
        before = eng.stats()
        with pytest.raises(kgb.KgbError, match="^cancelled$"):
            eng.bounce(0, nc, flags, N=1, M=256, mf=1, cancel=hook)
        after = eng.stats()
        assert hook.checks == k
        assert after["bounceLaunches"] - before["bounceLaunches"] == k - 1   # the launches before the cancel, no more
        assert (after["paths"] - before["paths"]) % nc == 0
    eng.bounce(0, nc, flags, N=1, M=256, mf=1, cancel=Countdown(10 ** 9))   # a hook that never fires changes nothing
    assert np.array_equal(eng.download_dc(nc), whole)


def test_cancel_between_view_launches(eng, engine_lib, pkg, kgb):
    s = pkg.workloads.random_city(42, n_boxes=400)
    nc = min(len(s["P"]), 12000)
    nAz, nEl, dAz, rowSin, wRow = pkg.workloads.views_grid(120.0, 2.0)
    eng.build(s["v"], s["tri"])
    eng.set_scene(s["P"][:nc], s["N"][:nc], np.zeros((0, 3), np.float32))
    flags = engine_lib.bounce_flags(False)
    kw = dict(world=False, cull=False, jitter=True, vground=True, groundZ=float(s["v"][:, 2].min()))
    before = eng.stats()
    eng.view(0, nc, flags, nAz, nEl, -60.0, dAz, rowSin, **kw)
    assert eng.stats()["launches"] - before["launches"] >= 2
    cls, dist = eng.download_view(nc)
    for k in (1, 2):
        hook = Countdown(k)
        before = eng.stats()
        with pytest.raises(kgb.KgbError, match="^cancelled$"):
            eng.view(0, nc, flags, nAz, nEl, -60.0, dAz, rowSin, cancel=hook, **kw)
        assert hook.checks == k and eng.stats()["launches"] - before["launches"] == k - 1
    eng.view(0, nc, flags, nAz, nEl, -60.0, dAz, rowSin, cancel=Countdown(10 ** 9), **kw)
    c2, d2 = eng.download_view(nc)
    assert np.array_equal(c2, cls) and np.array_equal(d2.view(np.uint32), dist.view(np.uint32))


def test_view_launch_carry_and_chunks(eng, engine_lib, pkg):
    """gpu_view's sub-launch size carries from chunk to chunk (gpu.cu:586-607, ViewLaunch::launch) and no chunk or
    launch boundary changes a class or a distance (check_views.cpp:851-867)."""
    s = pkg.workloads.random_city(43, n_boxes=300)
    nc = min(len(s["P"]), 9000)
    nAz, nEl, dAz, rowSin, wRow = pkg.workloads.views_grid(360.0, 4.0)
    eng.build(s["v"], s["tri"])
    eng.set_scene(s["P"][:nc], s["N"][:nc], np.zeros((0, 3), np.float32))
    flags = engine_lib.bounce_flags(False)
    kw = dict(world=True, cull=True, jitter=True, vground=True, groundZ=float(s["v"][:, 2].min()))
    carry = eng.view(0, nc, flags, nAz, nEl, 0.0, dAz, rowSin, **kw)
    assert carry > 0
    whole = eng.download_view(nc)
    iso = eng.reduce_view(nc, wRow, 3, 500.0, reach=[6.0, 20.0], isoDim=3)
    parts, isos, launch = [], [], 0
    for i0 in range(0, nc, 2500):
        m = min(2500, nc - i0)
        launch = eng.view(i0, m, flags, nAz, nEl, 0.0, dAz, rowSin, launch=launch, **kw)
        parts.append(eng.download_view(m))
        isos.append(eng.reduce_view(m, wRow, 3, 500.0, reach=[6.0, 20.0], isoDim=3))
    assert np.array_equal(np.concatenate([p[0] for p in parts]), whole[0])
    assert np.array_equal(np.concatenate([p[1] for p in parts]).view(np.uint32), whole[1].view(np.uint32))
    assert np.array_equal(np.concatenate(isos).view(np.uint64), iso.view(np.uint64))


def test_bounded_execution_limits(eng, engine_lib, pkg, kgb):
    """The traversal's node limit and the bounce step's time limit, lowered so that the calls reach them: each call
    fails with its message, and the next call, with the limits restored, gives the same results as before."""
    s = pkg.workloads.random_city(44, n_boxes=300)
    nc = 3000
    D = pkg.workloads.hemisphere_dirs(145, 100, 44)
    eng.build(s["v"], s["tri"], np.zeros(len(s["tri"]), np.uint32), [(0.3, 0, 0, 0)], per_slot=True)
    eng.set_scene(s["P"][:nc], s["N"][:nc], D)
    bits_flags, bflags = engine_lib.ray_flags(False, False), engine_lib.bounce_flags(False)
    nAz, nEl, dAz, rowSin, wRow = pkg.workloads.views_grid(120.0, 4.0)
    kw = dict(world=False, cull=False, jitter=True, vground=True, groundZ=float(s["v"][:, 2].min()))
    eng.trace(0, nc, bits_flags)
    bits = eng.download_bits(nc)
    eng.view(0, nc, bflags, nAz, nEl, -60.0, dAz, rowSin, **kw)
    view = eng.download_view(nc)
    eng.bounce(0, nc, bflags, N=3, M=64, mf=1)
    dc = eng.download_dc(nc)
    eng.set_limits(node_limit=3)
    with pytest.raises(kgb.KgbError, match="traversal gave up"):
        eng.trace(0, nc, bits_flags)
    with pytest.raises(kgb.KgbError, match="traversal gave up"):
        eng.view(0, nc, bflags, nAz, nEl, -60.0, dAz, rowSin, **kw)
    with pytest.raises(kgb.KgbError, match="gpu_bounce: traversal gave up .*first walk that gave up: sensor"):
        eng.bounce(0, nc, bflags, N=3, M=64, mf=1)
    eng.set_limits(0, bounce_limit_ns=1)
    with pytest.raises(kgb.KgbError, match=r"gpu_bounce: a launch of \d+ samples x 3000 sensors passed its 1e-09 s limit"):
        eng.bounce(0, nc, bflags, N=3, M=64, mf=1)
    eng.set_limits(0, 0)
    eng.trace(0, nc, bits_flags)
    assert np.array_equal(eng.download_bits(nc), bits)
    eng.view(0, nc, bflags, nAz, nEl, -60.0, dAz, rowSin, **kw)
    v2 = eng.download_view(nc)
    assert np.array_equal(v2[0], view[0]) and np.array_equal(v2[1].view(np.uint32), view[1].view(np.uint32))
    eng.bounce(0, nc, bflags, N=3, M=64, mf=1)
    assert np.array_equal(eng.download_dc(nc), dc)


def test_per_run_stats(eng, engine_lib, pkg):
    """check_gpu.cpp:790-797 at the engine: trace, bounce and build times positive, rays = sensors x directions of
    the calls made, paths = sensors x samples."""
    s = pkg.workloads.random_city(45, n_boxes=100)
    nc = len(s["P"])
    D = pkg.workloads.hemisphere_dirs(145, 50, 45)
    eng.build(s["v"], s["tri"], np.zeros(len(s["tri"]), np.uint32), [(0.3, 0, 0, 0)], per_slot=True)
    eng.set_scene(s["P"], s["N"], D)
    st0 = eng.stats()
    for i0 in range(0, nc, 700):   # tiny chunks: many calls
        m = min(700, nc - i0)
        eng.trace(i0, m, engine_lib.ray_flags(False, False))
        eng.bounce(i0, m, engine_lib.bounce_flags(False), N=1, M=32, mf=1)
    st1 = eng.stats()
    assert st1["buildMs"] > 0 and st1["gasBytes"] > 0
    assert st1["traceMs"] > st0["traceMs"] and st1["bounceMs"] > st0["bounceMs"]
    assert st1["rays"] - st0["rays"] == nc * len(D)
    assert st1["paths"] - st0["paths"] == nc * 32
    assert st1["launches"] > st0["launches"] and st1["bounceLaunches"] > st0["bounceLaunches"]


def test_series_pipeline_wait_limit(eng, engine_lib, pkg, kgb):
    """The tensor-core series pipeline's bounded waits: with the producer withholding its fills (a barrier nothing
    completes) and a 1 ms wait limit, the MMA issuer's and the epilogue's waits run out; the kernel finishes what it
    issued, frees its TMEM and ends, and kgb_series fails with the timeout message. With the limits restored the same
    engine gives the series it gave before, bit for bit."""
    s = pkg.workloads.random_city(45, n_boxes=40)
    nc, P, T, nSun = 1024, 145, 200, 60
    D = pkg.workloads.hemisphere_dirs(P, nSun, 45)
    eng.build(s["v"], s["tri"])
    eng.set_scene(s["P"][:nc], s["N"][:nc], D)
    eng.trace(0, nc, engine_lib.ray_flags(False, False))
    rng = np.random.default_rng(45)
    args = dict(nSky=P, row=np.arange(P), wsky=np.full(P, 2 * np.pi / P, np.float32), S=rng.uniform(0, 300, (P, T)).astype(np.float32),
                g=rng.uniform(0, 50, T).astype(np.float32), G=rng.uniform(0.1, 1.0, nc).astype(np.float32), sun0=2 * P,
                sunStep=np.sort(rng.choice(T, nSun, replace=False)), sunVec=D[2 * P:2 * P + nSun], sunW=rng.uniform(100, 900, nSun).astype(np.float32))
    E0 = eng.series(nc, **args)
    eng.set_limits(series_wait_ns=1_000_000, withhold_fills=True)
    t0 = time.perf_counter()
    with pytest.raises(kgb.KgbError, match="timed out waiting"):
        eng.series(nc, **args)
    assert time.perf_counter() - t0 < 3.0   # the waits gave up at their 1 ms limit, not the default 4 s
    eng.set_limits()
    E1 = eng.series(nc, **args)
    assert np.array_equal(E0.view(np.uint32), E1.view(np.uint32))
    eng.trace(0, nc, engine_lib.ray_flags(False, False))   # the engine's other kernels still run

