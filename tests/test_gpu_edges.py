"""Edge cases of the engine's entry points beyond the reference's (GPU): empty chunks for the sensor-major downloads and
the series file, a bounce with one sample and no diffuse reflection allowed (every path ends within the first steps
of the wavefront), and server requests with no sensors or no directions."""
import os

import numpy as np
import pytest

from test_gpu_parity import optics_slots
from test_gpu_series import _inputs

pytestmark = pytest.mark.gpu


def test_empty_chunks(engine_lib, kgb, pkg, tmp_path):
    s = pkg.workloads.random_city(2, n_boxes=10)
    D = pkg.workloads.hemisphere_dirs(40, 10, 2)
    e = kgb.Engine(engine_lib)
    try:
        e.build(s["v"], s["tri"])
        e.set_scene(s["P"], s["N"], D)
        e.trace(0, 0, engine_lib.ray_flags(False, False))
        assert e.download_bits_rows(0).shape == (0, (len(D) + 31) // 32)
        e.trace(0, 0, engine_lib.ray_flags(False, True))
        assert e.download_bytes_rows(0).shape == (0, len(D))
        fd = os.open(str(tmp_path / "empty.npy"), os.O_CREAT | os.O_RDWR | os.O_TRUNC, 0o644)
        try:
            e.series_file(0, fd, 128, **_inputs(145, 16, 0, D, 40, 10, 1))
        finally:
            os.close(fd)
        assert os.path.getsize(tmp_path / "empty.npy") == 0
    finally:
        e.close()


@pytest.mark.parametrize("N", [0, 1])
def test_bounce_one_sample(engine_lib, oracle, kgb, pkg, N):
    s = pkg.workloads.random_city(11, porous=True, glass=True, thin=True)
    slots = optics_slots(kgb)
    D = pkg.workloads.hemisphere_dirs(10, 10, 11)
    nc = 300
    rows = []
    for lib in (engine_lib, oracle):
        x = kgb.Engine(lib)
        try:
            x.build(s["v"], s["tri"], s["slot"], slots, per_slot=True)
            x.set_slots(slots)
            x.set_scene(s["P"][:nc], s["N"][:nc], D)
            x.bounce(0, nc, lib.bounce_flags(False), N=N, M=1, mf=1, north=0.0)
            rows.append(x.download_dc(nc))
        finally:
            x.close()
    assert np.array_equal(rows[0], rows[1])


def test_server_empty_requests(engine_lib, kgb, pkg):
    s = pkg.workloads.random_city(3, n_boxes=12)
    srv = kgb.Server(engine_lib, 1e9)
    try:
        sid = srv.add_scene(s["v"], s["tri"])
        D = pkg.workloads.hemisphere_dirs(40, 0, 3)
        none = srv.submit(sid, s["P"][:0], s["N"][:0], D, np.ones((1, len(D)), np.float32), [True])
        nodir = srv.submit(sid, s["P"][:5], s["N"][:5], np.zeros((0, 3), np.float32), np.zeros((2, 0), np.float32), [True, False])
        nAz, nEl = 10, 4
        rowSin = np.array([[np.sin(np.radians(-10 + 10 * k)), np.sin(np.radians(10 * k))] for k in range(nEl)], np.float32)
        wRow = np.full(nEl, 1.0 / (nAz * nEl))
        noview = srv.submit_views(sid, s["P"][:0], s["N"][:0], nAz, nEl, -60.0, 12.0, rowSin, wRow, 3, 100.0)
        assert srv.wait(none).shape == (1, 0)
        assert np.array_equal(srv.wait(nodir), np.zeros((2, 5)))
        assert srv.wait(noview).shape == (0, 10)
        st, tm = srv.stats(), srv.timing()
        assert st["completed"] == 3 and st["items"] == 0 and tm["day_rays"] == 0 and tm["views_rays"] == 0
    finally:
        srv.close()
