"""How far the shared float decision lies from exact geometry (CPU, on the oracle; the engine's decisions equal the
oracle's bit for bit, which the GPU parity tests check on the same scenes).

The oracle's kgbo_recheck_bits / kgbo_recheck_view decide each ray of a sample twice: as the kernels do (the watertight
float test and the reference's per-hit rules in float) and with every test and rule in double from the same float
inputs. A ray decided differently is attributed to a triangle edge within EDGE_REL x (|o|max + t) of the ray, a grazing
hit (|cos| < 0.05, the reference's own exclusion, validate/README.md:189), a sign or threshold test of the rules (the
reference excludes rays within 1e-6 of a sign test and hits within 1 mm of the downward ray's end), or, in views, a tie
of two hits within 1e-5 of each other's distance, or a float distance off by more than the reference's distance check
(1e-5 t + 1e-4 m). The tests require no ray outside these classes, and view distances within DIST_REL of the double
walk's (the criterion: within 1e-5 relative)."""
import ctypes

import numpy as np
import pytest

EDGE_REL = 2.0 ** -16      # the stated edge band, relative to |o|max + t (the float test's rounding scales with them)
DIST_REL = 1e-5            # view distances against the double walk
KEYS = ["rays", "differ", "edge", "grazing", "threshold", "tie", "rounding", "other"]


def recheck(lib):
    f = lib.dll.kgbo_recheck_bits
    f.restype, f.argtypes = ctypes.c_int, [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_uint32, ctypes.c_double, ctypes.c_void_p]
    g = lib.dll.kgbo_recheck_view
    g.restype, g.argtypes = ctypes.c_int, [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_double,
                                           ctypes.c_void_p]
    return f, g


def summary(outs):
    """Sums the oracle's out[24] arrays of several chunks into a dict (maxima where the entry is a maximum)."""
    t = np.zeros(24)
    for o in outs:
        t[:17] += o[:17]
        t[19:21] += o[19:21]
        t[[17, 18, 21]] = np.maximum(t[[17, 18, 21]], o[[17, 18, 21]])
    d = {k: int(x) for k, x in zip(KEYS, t[:8])}
    d.update(edge_dist_bins=[int(x) for x in t[8:14]], cos_bins=[int(x) for x in t[14:17]], max_edge_dist=float(t[17]),
             max_edge_rel=float(t[18]), class_differences=int(t[19]), distance_differences=int(t[20]), max_dist_rel=float(t[21]))
    others = [o for o in outs if o[22] >= 0]
    d["first_other"] = (int(others[0][22]), int(others[0][23])) if others else None
    return d


def bits_sample(lib, o, i0s, nc, flags):
    f, _ = recheck(lib)
    outs = []
    for i0 in i0s:
        out = np.zeros(24)
        assert f(o.h, int(i0), nc, flags, EDGE_REL, out.ctypes.data_as(ctypes.c_void_p)), lib.err()
        outs.append(out)
    return summary(outs)


def view_sample(lib, kgb, o, i0s, nc, grid, fov, world, groundZ):
    _, g = recheck(lib)
    nAz, nEl, dAz, rowSin, wRow = grid
    rs = np.ascontiguousarray(rowSin, np.float32)
    v = kgb.ViewIn(nAz, nEl, 0.0 if world else -fov / 2, dAz, rs.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), int(world), int(world), 1, 0, 1,
                   1, groundZ, 0.0, kgb.CANCEL_FN(), None)
    outs = []
    for i0 in i0s:
        out = np.zeros(24)
        assert g(o.h, int(i0), nc, lib.bounce_flags(False), ctypes.byref(v), EDGE_REL, out.ctypes.data_as(ctypes.c_void_p)), lib.err()
        outs.append(out)
    return summary(outs)


def check(s):
    assert s["differ"] == s["edge"] + s["grazing"] + s["threshold"] + s["tie"] + s["rounding"] + s["other"], s
    assert s["other"] == 0, s
    assert s["max_edge_rel"] <= EDGE_REL, s
    assert s["max_dist_rel"] <= DIST_REL, s


def test_urban_block_bits_against_double(oracle, kgb, pkg):
    """The urban block with the reference's direction table (577 patches, ground, 4456 sun hours)."""
    import replay
    s = pkg.workloads.urban_block()
    D, _ = replay.urban_sky()
    o = kgb.Engine(oracle)
    try:
        o.build(s["v"], s["tri"])
        o.set_scene(s["P"], s["N"], D)
        i0s = np.random.default_rng(5).choice(len(s["P"]) - 128, 6, replace=False)
        r = bits_sample(oracle, o, i0s, 128, oracle.ray_flags(False, False))
    finally:
        o.close()
    print("urban block bits:", r)
    assert r["rays"] > 300_000
    check(r)


@pytest.fixture(scope="module")
def views_city(pkg):
    return pkg.workloads.views_city()


def test_views_city_against_double(oracle, kgb, pkg, views_city):
    """The 2 M-triangle views city (rotated boxes, gable roofs, km-long ground quads), fov 120 and fov 360 at
    2 degree cells with jitter, and the visibility bits of a hemisphere of directions on its facades."""
    c = views_city
    o = kgb.Engine(oracle)
    try:
        o.build(c["v"], c["tri"])
        o.set_labels(c["label"])
        o.set_scene(c["P"], c["N"], np.zeros((0, 3), np.float32))
        i0s = np.random.default_rng(3).choice(len(c["P"]) - 32, 6, replace=False)
        res = {}
        for fov, world in ((120.0, False), (360.0, True)):
            res[fov] = view_sample(oracle, kgb, o, i0s, 32, pkg.workloads.views_grid(fov, 2.0), fov, world, c["groundZ"])
        o.set_scene(c["P"], c["N"], pkg.workloads.hemisphere_dirs(577, 600, 9))
        res["bits"] = bits_sample(oracle, o, i0s, 32, oracle.ray_flags(False, False))
    finally:
        o.close()
    for k, r in res.items():
        print("views city", k, r)
        assert r["rays"] > 100_000
        check(r)


def test_a_planted_rounding_error_is_caught(oracle, kgb, pkg):
    """The check catches distances off exact geometry: a strip 6 km long and 50 m wide (the views city's water and park
    strips are such triangles) seen from 21 m above it, 2.3 km from the strip's ends. With the refinement of far hits
    (the kernels' rule) its distances stay within 2e-7 of the double walk's; with the refinement switched off in the
    oracle (the mistake planted, on the CPU) the float test's own rounding shows (1.6e-4 relative), and the check
    fails."""
    v = np.array([[-3000, -3000, 0], [3000, -3000, 0], [3000, -2950, 0], [-3000, -2950, 0]], np.float32)
    tri = np.array([[0, 1, 2], [0, 2, 3]], np.uint32)
    P = np.array([[-2327.85, -2987.36, 20.8]], np.float32)
    N = np.array([[0.0, 0.0, -1.0]], np.float32)
    plant = oracle.dll.kgbo_set_refine
    plant.restype, plant.argtypes = None, [ctypes.c_int]
    o = kgb.Engine(oracle)
    try:
        o.build(v, tri)
        o.set_labels(np.full(2, 3, np.uint8))
        o.set_scene(P, N, np.zeros((0, 3), np.float32))
        grid = pkg.workloads.views_grid(120.0, 1.0, lo=-85.0, hi=-5.0)
        good = view_sample(oracle, kgb, o, [0], 1, grid, 120.0, False, -1e4)
        plant(0)
        try:
            bad = view_sample(oracle, kgb, o, [0], 1, grid, 120.0, False, -1e4)
        finally:
            plant(1)
    finally:
        o.close()
    print("km quad, refined:", good)
    print("km quad, planted:", bad)
    check(good)
    assert good["max_dist_rel"] < 2e-7
    assert bad["max_dist_rel"] > DIST_REL and bad["rounding"] > 0
    with pytest.raises(AssertionError):
        check(bad)
