"""The visibility kernels' tracing order (GPU): the engine traces a call's sensors grouped by the orientation of their
normals, a permutation that must leave every sensor's result where the caller put it. Checked on a random box city
(every face a sensor, so the six orientation classes interleave along the sensor array): a call over any sub-range
gives the full call's columns of that range, bit for bit, in bits and in byte mode; and the same engine, given the
sensors again in another order (same count, other classes at each index: the order is rebuilt) or the same sensors
again (the order kept), gives each sensor the bits it had."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def city(pkg):
    s = pkg.workloads.random_city(11, n_boxes=30, extent=40.0, q=1.5, glass=True)
    D = pkg.workloads.hemisphere_dirs(145, 200, 5)
    return s, D


def engine_for(kgb, engine_lib, s, D, P=None, N=None):
    e = kgb.Engine(engine_lib)
    e.build(s["v"], s["tri"])
    e.set_scene(s["P"] if P is None else P, s["N"] if N is None else N, D)
    return e


def test_the_city_mixes_the_classes(city):
    s, _ = city
    N = s["N"]
    ax = np.argmax(np.abs(N), axis=1)
    cls = 2 * ax + (N[np.arange(len(N)), ax] > 0)
    assert len(np.unique(cls)) >= 5
    assert np.count_nonzero(np.diff(cls)) > 100   # classes change along the array many times


def test_sub_ranges_give_the_full_calls_columns(kgb, engine_lib, city):
    s, D = city
    nc = len(s["P"])
    e = engine_for(kgb, engine_lib, s, D)
    try:
        flags = engine_lib.ray_flags(False, False)
        e.trace(0, nc, flags)
        full = e.download_bits(nc)
        rng = np.random.default_rng(2)
        ranges = [(0, 1), (nc - 1, 1), (1, nc - 1), (37, 4100), (nc // 3, nc // 3)]
        ranges += [(int(a), int(rng.integers(1, nc - a))) for a in rng.integers(0, nc - 1, 4)]
        for i0, n in ranges:
            e.trace(i0, n, flags)
            assert np.array_equal(e.download_bits(n), full[:, i0:i0 + n]), (i0, n)
    finally:
        e.close()


def test_sub_ranges_in_byte_mode(kgb, engine_lib, city):
    s, D = city
    nc = len(s["P"])
    slots = [(0.2, 0, 0, 0), (0.3, 0.5, 0, 0), (0.0, 0.64, kgb.tn_from_Tn(0.64), kgb.SLOT_GLASS), (0.25, 0, 0, 0)]   # the city's slots
    e = kgb.Engine(engine_lib)
    try:
        e.build(s["v"], s["tri"], s["slot"], slots)
        e.set_slots(slots)
        e.set_scene(s["P"], s["N"], D)
        flags = engine_lib.ray_flags(False, True)
        e.trace(0, nc, flags)
        full = e.download_bytes(nc).reshape(-1, nc)
        for i0, n in [(5, 3000), (nc // 2, nc - nc // 2), (1, 1)]:
            e.trace(i0, n, flags)
            assert np.array_equal(e.download_bytes(n).reshape(-1, n), full[:, i0:i0 + n]), (i0, n)
    finally:
        e.close()


def test_new_sensors_of_the_same_count_rebuild_the_order(kgb, engine_lib, city):
    s, D = city
    nc = len(s["P"])
    perm = np.random.default_rng(4).permutation(nc)
    flags = engine_lib.ray_flags(False, False)
    e = engine_for(kgb, engine_lib, s, D)
    try:
        e.trace(0, nc, flags)
        ref = e.download_bits(nc)
        e.set_scene(np.ascontiguousarray(s["P"][perm]), np.ascontiguousarray(s["N"][perm]), D)   # other classes at each index
        e.trace(0, nc, flags)
        assert np.array_equal(e.download_bits(nc), ref[:, perm])
        e.set_scene(s["P"], s["N"], D)   # back: rebuilt again
        e.trace(0, nc, flags)
        assert np.array_equal(e.download_bits(nc), ref)
        e.set_scene(s["P"], s["N"], D)   # the same sensors: the order kept
        e.trace(0, nc, flags)
        assert np.array_equal(e.download_bits(nc), ref)
    finally:
        e.close()
    fresh = engine_for(kgb, engine_lib, s, D, P=np.ascontiguousarray(s["P"][perm]), N=np.ascontiguousarray(s["N"][perm]))
    try:
        fresh.trace(0, nc, flags)
        assert np.array_equal(fresh.download_bits(nc), ref[:, perm])
    finally:
        fresh.close()
