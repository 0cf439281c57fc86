"""Both BVH builders (kgb_set_builder: 1 the device LBVH with treelet restructuring, the default; 0 the host binned
SAH tree), collapsed to the same 8-wide records. Every result must equal the oracle's bit for bit with either: the
tree only changes which boxes are visited, never the hit set. Covered: visibility bits and transmittance bytes on seeded
cities, closest-hit view classes and distances, reflected-light rows (slot records), scenes of 0 to 4 triangles and
triangles sharing one centroid (equal Morton codes, the tie rule of the radix tree)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


BUILDERS = [1, 0]


def engines(engine_lib, oracle, kgb, builder):
    e, o = kgb.Engine(engine_lib), kgb.Engine(oracle)
    e.set_builder(builder)
    return e, o


def bits_of(eng, nc, flags):
    eng.trace(0, nc, flags)
    return eng.download_bits(nc)


@pytest.mark.parametrize("builder", BUILDERS)
@pytest.mark.parametrize("seed", [1, 2, 3])
def test_tree_bits(engine_lib, oracle, kgb, pkg, seed, builder):
    s = pkg.workloads.random_city(seed)
    D = pkg.workloads.hemisphere_dirs(145, 300, seed)
    e, o = engines(engine_lib, oracle, kgb, builder)
    try:
        for x in (e, o):
            x.build(s["v"], s["tri"])
            x.set_scene(s["P"], s["N"], D)
        nc = len(s["P"])
        for cull in (False, True):
            f = engine_lib.ray_flags(cull, False)
            a, b = bits_of(e, nc, f), bits_of(o, nc, f)
            assert np.array_equal(a, b), "%d of %d words differ" % (np.sum(a != b), a.size)
        assert e.stats()["gasBytes"] > 0
    finally:
        e.close(); o.close()


@pytest.mark.parametrize("builder", BUILDERS)
def test_tree_bytes_and_bounce(engine_lib, oracle, kgb, pkg, builder):
    s = pkg.workloads.random_city(9, porous=True, glass=True, thin=True)
    tn = kgb.tn_from_Tn(0.64)
    slots = [(0.2, 0, 0, 0), (0.3, 0.5, 0, 0), (0.0, 0.64, tn, kgb.SLOT_GLASS), (0.25, 0, 0, 0), (0.2, 0, 0, 0), (0.2, 0, 0, 0),
             (0.2, 0, 0, 0), (0.1, 0.6, 0, kgb.SLOT_THIN)]
    D = pkg.workloads.hemisphere_dirs(145, 300, 9)
    e, o = engines(engine_lib, oracle, kgb, builder)
    try:
        for x in (e, o):
            x.build(s["v"], s["tri"], s["slot"], slots, per_slot=True)
            x.set_slots(slots)
            x.set_scene(s["P"], s["N"], D)
        nc = len(s["P"])
        got = []
        for x in (e, o):
            x.trace(0, nc, engine_lib.ray_flags(False, True))
            got.append(x.download_bytes(nc))
        assert np.array_equal(got[0], got[1]), "%d of %d bytes differ" % (np.sum(got[0] != got[1]), got[0].size)
        rows = []
        for x in (e, o):
            x.bounce(0, 400, engine_lib.bounce_flags(False), N=2, M=64, mf=1, north=10.0)
            rows.append(x.download_dc(400))
        assert np.array_equal(rows[0], rows[1])
    finally:
        e.close(); o.close()


@pytest.mark.parametrize("builder", BUILDERS)
def test_tree_views(engine_lib, oracle, kgb, pkg, builder):
    s = pkg.workloads.random_city(7, glass=True)
    label = np.random.default_rng(2).integers(2, 6, len(s["tri"])).astype(np.uint8)
    nAz, nEl, dAz, rowSin, wRow = pkg.workloads.views_grid(120.0, 4.0)
    e, o = engines(engine_lib, oracle, kgb, builder)
    try:
        out = []
        for x in (e, o):
            x.build(s["v"], s["tri"])
            x.set_labels(label)
            x.set_scene(s["P"][:600], s["N"][:600], np.zeros((0, 3), np.float32))
            x.view(0, 600, engine_lib.bounce_flags(False), nAz, nEl, -60.0, dAz, rowSin, jitter=True)
            out.append(x.download_view(600))
        for a, b in zip(out[0], out[1]):
            assert np.array_equal(a.view(np.uint8), b.view(np.uint8))
    finally:
        e.close(); o.close()


@pytest.mark.parametrize("builder", BUILDERS)
@pytest.mark.parametrize("nt", [0, 1, 2, 3, 4, 97])
def test_tree_small_and_tied(engine_lib, oracle, kgb, nt, builder):
    rng = np.random.default_rng(nt)
    if nt == 97:   # every triangle with the same centroid: equal Morton codes throughout
        c = np.array([0.5, 0.5, 2.0], np.float32)
        d = rng.normal(size=(nt, 3, 3)).astype(np.float32)
        d -= d.mean(axis=1, keepdims=True)
        v = (c + d).reshape(-1, 3)
    else:
        v = rng.uniform(-3, 3, (3 * nt, 3)).astype(np.float32) + np.array([0, 0, 2], np.float32)
    tri = np.arange(3 * nt, dtype=np.uint32).reshape(-1, 3)
    P = np.stack([rng.uniform(-2, 2, 64), rng.uniform(-2, 2, 64), np.zeros(64)], axis=1).astype(np.float32)
    N = np.tile(np.array([0, 0, 1], np.float32), (64, 1))
    z = rng.uniform(0.05, 1, 256)
    a = rng.uniform(0, 2 * np.pi, 256)
    D = np.stack([np.sqrt(1 - z * z) * np.cos(a), np.sqrt(1 - z * z) * np.sin(a), z], axis=1).astype(np.float32)
    e, o = engines(engine_lib, oracle, kgb, builder)
    try:
        got = []
        for x in (e, o):
            x.build(v.reshape(-1, 3), tri)
            x.set_scene(P, N, D)
            got.append(bits_of(x, 64, engine_lib.ray_flags(False, False)))
        assert np.array_equal(got[0], got[1])
        if nt == 0:
            assert np.all(got[0] == 0xffffffff)
    finally:
        e.close(); o.close()
