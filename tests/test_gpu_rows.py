"""Sensor-major downloads (GPU): per-ray results transposed on the device, in slices of at most 64 MiB of rows, equal
the direction-major buffers transposed on the host, bit for bit, also when a download spans several slices."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _slots(kgb):
    tn = kgb.tn_from_Tn(0.64)
    return [(0.2, 0, 0, 0), (0.3, 0.5, 0, 0), (0.0, 0.64, tn, kgb.SLOT_GLASS), (0.25, 0, 0, 0), (0.2, 0, 0, 0), (0.2, 0, 0, 0),
            (0.2, 0, 0, 0), (0.1, 0.6, 0, kgb.SLOT_THIN)]


@pytest.mark.parametrize("n_sky, n_sun", [(145, 300), (60_000, 80_000)])   # one slice; 6250 words a sensor: several
def test_bits_rows(engine_lib, kgb, pkg, n_sky, n_sun):
    s = pkg.workloads.random_city(5, n_boxes=40)
    D = pkg.workloads.hemisphere_dirs(n_sky, n_sun, 5)
    nc = min(len(s["P"]), 6000)
    e = kgb.Engine(engine_lib)
    try:
        e.build(s["v"], s["tri"])
        e.set_scene(s["P"][:nc], s["N"][:nc], D)
        e.trace(0, nc, engine_lib.ray_flags(False, False))
        raw = e.download_bits(nc)                       # [nWords x nc]
        rows = e.download_bits_rows(nc)                 # [nc x nWords]
        assert rows.shape == (nc, raw.shape[0])
        assert np.array_equal(rows, raw.T)
        assert raw.any()
    finally:
        e.close()


@pytest.mark.parametrize("n_sky, n_sun", [(145, 300), (20_000, 12_000)])    # one slice; 52,000 bytes a sensor: several
def test_bytes_rows(engine_lib, kgb, pkg, n_sky, n_sun):
    s = pkg.workloads.random_city(6, porous=True, glass=True, thin=True)
    D = pkg.workloads.hemisphere_dirs(n_sky, n_sun, 6)
    nc = min(len(s["P"]), 3000)
    slots = _slots(kgb)
    e = kgb.Engine(engine_lib)
    try:
        e.build(s["v"], s["tri"], s["slot"], slots)
        e.set_slots(slots)
        e.set_scene(s["P"][:nc], s["N"][:nc], D)
        e.trace(0, nc, engine_lib.ray_flags(False, True))
        raw = e.download_bytes(nc)                      # [nDir x nc]
        rows = e.download_bytes_rows(nc)                # [nc x nDir]
        assert np.array_equal(rows, raw.T)
        assert len(np.unique(raw)) > 2
    finally:
        e.close()


def test_view_rows_across_slices(engine_lib, kgb, pkg):
    """fov 360 at 2 degrees (10,800 rays, 43 kB of distances a sensor): 4000 sensors span three slices; the same
    sensors viewed and downloaded in chunks of 500 (one slice each) give the same rows."""
    city = pkg.workloads.views_city(seed=4, n_buildings=200, target_tris=40_000, n_sensors=5000)
    nc = min(4000, len(city["P"]))
    nAz, nEl, dAz, rowSin, wRow = pkg.workloads.views_grid(360.0, 2.0)
    kw = dict(world=True, cull=True, jitter=True, vground=True, groundZ=city["groundZ"])
    e = kgb.Engine(engine_lib)
    try:
        e.build(city["v"], city["tri"])
        e.set_labels(city["label"])
        e.set_scene(city["P"][:nc], city["N"][:nc], np.zeros((0, 3), np.float32))
        flags = engine_lib.bounce_flags(False)
        e.view(0, nc, flags, nAz, nEl, 0.0, dAz, rowSin, **kw)
        cls, dist = e.download_view(nc)
        assert cls.shape == (nc, nAz * nEl)
        parts = []
        for i0 in range(0, nc, 500):
            m = min(500, nc - i0)
            e.view(i0, m, flags, nAz, nEl, 0.0, dAz, rowSin, **kw)
            parts.append(e.download_view(m))
        assert np.array_equal(cls, np.concatenate([p[0] for p in parts]))
        assert np.array_equal(dist.view(np.uint32), np.concatenate([p[1] for p in parts]).view(np.uint32))
        assert len(np.unique(cls)) > 2
    finally:
        e.close()
