"""The time series on the tensor cores (split-BF16 tcgen05 contraction, GPU) against the oracle's FP64 contraction of the
same FP32 per-direction weights: the error of every output column is measured and bounded.

Error of column t: max over sensors |E - E64| / max over sensors |E64| (normwise per column); the elementwise relative
error is reported over the entries of at least 1 % of their column's maximum."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

COLUMN_TOL = 1e-6   # normwise per-column bound of the tensor-core form against FP64 (measured values are printed)


def _setup(pkg, kgb, lib, s, D, nc):
    e = kgb.Engine(lib)
    e.build(s["v"], s["tri"])
    e.set_scene(s["P"][:nc], s["N"][:nc], D)
    e.trace(0, nc, lib.ray_flags(False, False))
    return e


def _inputs(P, T, nc, D, nSky, nSun, seed):
    rng = np.random.default_rng(seed)
    omega = 2 * np.pi / P
    # Perez-like magnitudes: radiance 0..500 W/m2/sr with a smooth patch and hour structure, dark hours included
    base = rng.uniform(20, 400, P)[:, None] * np.clip(np.sin(np.linspace(0, 6 * np.pi, T)), 0, None)[None, :]
    S = (base * rng.uniform(0.8, 1.2, (P, T))).astype(np.float32)
    sunStep = np.sort(rng.choice(T, nSun, replace=False))
    return dict(nSky=nSky, row=np.arange(nSky) % P, wsky=np.full(nSky, omega, np.float32), S=S, g=(S.mean(axis=0) * 0.2).astype(np.float32),
                G=rng.uniform(0.1, 1.0, nc).astype(np.float32), sun0=2 * nSky, sunStep=sunStep, sunVec=D[2 * nSky:2 * nSky + nSun],
                sunW=rng.uniform(100, 900, nSun).astype(np.float32))


def _column_errors(E, E64):
    cmax = np.abs(E64).max(axis=0)
    live = cmax > 0
    col = np.abs(E - E64).max(axis=0)[live] / cmax[live]
    big = np.abs(E64) >= 0.01 * cmax[None, :]
    elem = (np.abs(E - E64) / np.maximum(np.abs(E64), 1e-30))[big & live[None, :]]
    return col, elem


@pytest.mark.parametrize("seed", [1, 2])
def test_series_tensor_cores_vs_fp64(engine_lib, oracle, kgb, pkg, seed):
    s = pkg.workloads.random_city(20 + seed, n_boxes=60)
    P, T, nSun, nc = 2305, 384, 200, 1500
    D = np.concatenate([pkg.workloads.hemisphere_dirs(P, nSun, seed)])
    e, o = _setup(pkg, kgb, engine_lib, s, D, nc), _setup(pkg, kgb, oracle, s, D, nc)
    try:
        args = _inputs(P, T, nc, D, P, nSun, seed)
        E = e.series(nc, **args)
        E64 = o.series(nc, **args)
        col, elem = _column_errors(E, E64)
        print("\nsplit-BF16 tensor cores, P %d, T %d, %d sensors: column error max %.3g median %.3g; elementwise max %.3g"
              % (P, T, nc, col.max(), np.median(col), elem.max()))
        assert col.max() <= COLUMN_TOL
        # the plain FP32 form on the same inputs
        e.set_series_form(1)
        E32 = e.series(nc, **args)
        e.set_series_form(0)
        col32, elem32 = _column_errors(E32, E64)
        print("plain FP32 form: column error max %.3g median %.3g; elementwise max %.3g" % (col32.max(), np.median(col32), elem32.max()))
        assert col32.max() <= 1e-5
    finally:
        e.close()
        o.close()


def test_series_tensor_cores_with_reflected_light(engine_lib, oracle, kgb, pkg):
    s = pkg.workloads.random_city(31, n_boxes=40)
    P, T, nSun, nc = 577, 200, 120, 700
    D = pkg.workloads.hemisphere_dirs(P, nSun, 5)
    slots = [(0.3, 0, 0, 0)]
    engs = []
    for lib in (engine_lib, oracle):
        x = kgb.Engine(lib)
        x.build(s["v"], s["tri"], np.zeros(len(s["tri"]), np.uint32), slots, per_slot=True)
        x.set_slots(slots)
        x.set_scene(s["P"][:nc], s["N"][:nc], D)
        x.trace(0, nc, lib.ray_flags(False, False))
        x.bounce(0, nc, lib.bounce_flags(False), N=1, M=64, mf=2)
        engs.append(x)
    try:
        args = _inputs(P, T, nc, D, P, nSun, 9)
        nBins = engs[0].dims()["nBins"]
        args["Sdc"] = np.random.default_rng(4).uniform(0, 300, (nBins, T)).astype(np.float32)
        E, E64 = engs[0].series(nc, **args), engs[1].series(nc, **args)
        col, elem = _column_errors(E, E64)
        print("\nwith %d reflected-light bins: column error max %.3g, elementwise max %.3g" % (nBins, col.max(), elem.max()))
        assert col.max() <= COLUMN_TOL
    finally:
        for x in engs:
            x.close()


def test_series_chunks_equal_whole(engine_lib, kgb, pkg):
    """A chunk's rows equal the whole run's rows: the contraction of a sensor does not depend on its chunk."""
    s = pkg.workloads.random_city(7, n_boxes=30)
    P, T, nSun, nc = 145, 150, 60, 600
    D = pkg.workloads.hemisphere_dirs(P, nSun, 7)
    e = _setup(pkg, kgb, engine_lib, s, D, nc)
    try:
        args = _inputs(P, T, nc, D, P, nSun, 3)
        whole = e.series(nc, **args)
        e.trace(200, 300, engine_lib.ray_flags(False, False))
        a2 = dict(args, G=args["G"][200:500])
        part = e.series(300, **a2)
        assert np.array_equal(part, whole[200:500])
    finally:
        e.close()


def test_series_bands_equal_chunks(engine_lib, kgb, pkg):
    """A chunk of at least 32 rows of 128-sensor tiles runs in four bands whose downloads overlap the next band's
    kernel; its rows equal the same sensors' rows from chunks below that size (one band each), bit for bit."""
    s = pkg.workloads.random_city(8, n_boxes=40)
    P, T, nSun, nc = 145, 150, 60, 5000
    assert len(s["P"]) >= nc
    D = pkg.workloads.hemisphere_dirs(P, nSun, 8)
    e = _setup(pkg, kgb, engine_lib, s, D, nc)
    try:
        args = _inputs(P, T, nc, D, P, nSun, 4)
        whole = e.series(nc, **args)
        st = e.stats()   # the tensor-core kernels' event time and outputs (the bench's roofline reads them)
        assert st["seriesMs"] > 0 and st["seriesOutputs"] == nc * T
        parts = []
        for i0, m in ((0, 3000), (3000, 2000)):
            e.trace(i0, m, engine_lib.ray_flags(False, False))
            parts.append(e.series(m, **dict(args, G=args["G"][i0:i0 + m])))
        assert np.array_equal(whole, np.concatenate(parts))
        assert np.abs(whole).max() > 0
    finally:
        e.close()


def test_series_file_matches_series(engine_lib, kgb, pkg, tmp_path):
    """kgb_series_file writes the rows kgb_series returns, bit for bit, at the caller's offsets: chunks of 5000 sensors
    (four bands, each more than a staging slice of rows) appended after a header, as the reference's --timeseries
    file."""
    import os
    s = pkg.workloads.random_city(8, n_boxes=40)
    P, T, nSun, nc = 145, 4000, 600, 5000
    D = pkg.workloads.hemisphere_dirs(P, nSun, 8)
    e = _setup(pkg, kgb, engine_lib, s, D, nc)
    try:
        args = _inputs(P, T, nc, D, P, nSun, 6)
        want = e.series(nc, **args)
        header = 128
        path = str(tmp_path / "series.npy")
        fd = os.open(path, os.O_CREAT | os.O_RDWR | os.O_TRUNC, 0o644)
        try:
            os.pwrite(fd, b"H" * header, 0)
            e.series_file(nc, fd, header, **args)
        finally:
            os.close(fd)
        got = np.fromfile(path, np.float32, offset=header).reshape(nc, T)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    finally:
        e.close()


def test_series_two_engines_share_inputs(engine_lib, kgb, pkg):
    """Two engines on two threads compute series from the same host arrays at once. The inputs (S of 20 MB) and the
    outputs (E of 18 MB) are page-locked for each call; the two calls share the registration of S, which ends with
    the later of them. Each engine's rows equal the rows it computes alone, bit for bit."""
    import threading
    s = pkg.workloads.random_city(8, n_boxes=40)
    P, T, nSun, nc = 2305, 2200, 300, 2000
    D = pkg.workloads.hemisphere_dirs(P, nSun, 8)
    engs = [_setup(pkg, kgb, engine_lib, s, D, nc) for _ in range(2)]
    try:
        args = _inputs(P, T, nc, D, P, nSun, 6)
        assert args["S"].nbytes >= 16 << 20 and nc * T * 4 >= 16 << 20
        alone = [x.series(nc, **args) for x in engs]
        assert np.array_equal(alone[0], alone[1]) and np.abs(alone[0]).max() > 0
        out = [np.full((nc, T), np.nan, np.float32) for _ in engs]
        errs = []

        def work(k):
            try:
                for _ in range(3):
                    engs[k].series(nc, out=out[k], **args)
            except Exception as ex:   # reported below: an assertion in a thread would not fail the test
                errs.append(ex)
        th = [threading.Thread(target=work, args=(k,)) for k in range(2)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        assert not errs, errs
        for k in range(2):
            assert np.array_equal(out[k], alone[0])
    finally:
        for x in engs:
            x.close()


def test_series_into_caller_pinned_memory(engine_lib, kgb, pkg):
    """E written into memory the caller page-locked (torch's pinned allocator) is used as it is: the same rows as
    into pageable memory."""
    import torch
    s = pkg.workloads.random_city(8, n_boxes=40)
    P, T, nSun, nc = 2305, 2200, 300, 2000
    D = pkg.workloads.hemisphere_dirs(P, nSun, 8)
    e = _setup(pkg, kgb, engine_lib, s, D, nc)
    try:
        args = _inputs(P, T, nc, D, P, nSun, 6)
        ref = e.series(nc, **args)
        pinned = torch.empty((nc, T), dtype=torch.float32).pin_memory().numpy()
        got = e.series(nc, out=pinned, **args)
        assert np.array_equal(got, ref) and np.array_equal(pinned, ref)
    finally:
        e.close()
