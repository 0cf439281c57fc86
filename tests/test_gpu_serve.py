"""The serving loop (GPU): requests of uneven sizes on several resident scenes, submitted together, complete with the
results they get alone through the single-request entry points, bit for bit (daylight sums and views columns); a small
HBM budget only serialises admission."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _alone_daylight(kgb, lib, scene, P, N, D, W, use_cos):
    e = kgb.Engine(lib)
    try:
        e.build(scene["v"], scene["tri"])
        e.set_scene(P, N, D)
        e.trace(0, len(P), lib.ray_flags(False, False))
        return np.stack([e.reduce(len(P), W[q], c) for q, c in enumerate(use_cos)])
    finally:
        e.close()


def _views_grid(fov, cell, lo=-70.0, hi=50.0):
    nAz, nEl = int(round(fov / cell)), int(round((hi - lo) / cell))
    dEl = (hi - lo) / nEl
    rowSin = np.array([[np.sin(np.radians(hi - (k + 1) * dEl)), np.sin(np.radians(hi - k * dEl))] for k in range(nEl)], np.float32)
    wRow = np.array([np.radians(fov / nAz) * (r[1] - r[0]) for r in rowSin.astype(np.float64)])
    wRow /= wRow.sum() * nAz
    return nAz, nEl, rowSin, wRow


@pytest.mark.parametrize("budget_gb", [64, 0.05])
def test_mixed_requests_equal_alone(engine_lib, kgb, pkg, budget_gb):
    scenes = [pkg.workloads.random_city(s, n_boxes=30 + 10 * s) for s in (1, 2)]
    srv = kgb.Server(engine_lib, budget_gb * 1e9)
    try:
        ids = [srv.add_scene(s["v"], s["tri"]) for s in scenes]
        srv.autotune()
        rng = np.random.default_rng(3)
        reqs = []
        for k in range(14):
            sc = k % 2
            s = scenes[sc]
            n = int(rng.integers(5, min(len(s["P"]), 4000)))
            first = int(rng.integers(0, len(s["P"]) - n))
            P, N = s["P"][first:first + n], s["N"][first:first + n]
            D = pkg.workloads.hemisphere_dirs(int(rng.integers(10, 200)), int(rng.integers(0, 300)), k)
            nQ = int(rng.integers(1, 5))
            W = rng.uniform(0.0, 2.0, (nQ, len(D))).astype(np.float32)
            use_cos = [bool(x) for x in rng.integers(0, 2, nQ)]
            reqs.append((sc, P, N, D, W, use_cos, srv.submit(ids[sc], P, N, D, W, use_cos)))
        # a views request in the mix
        nAz, nEl, rowSin, wRow = _views_grid(120.0, 4.0)
        vs = scenes[0]
        vt = srv.submit_views(ids[0], vs["P"][:300], vs["N"][:300], nAz, nEl, -60.0, 120.0 / nAz, rowSin, wRow, 3, 500.0, reach=[6.0, 20.0],
                              groundZ=float(vs["v"][:, 2].min()))
        for sc, P, N, D, W, use_cos, t in reqs:
            got = srv.wait(t)
            want = _alone_daylight(kgb, engine_lib, scenes[sc], P, N, D, W, use_cos)
            assert np.array_equal(got, want)
        gotv = srv.wait(vt)
        e = kgb.Engine(engine_lib)
        try:
            e.build(vs["v"], vs["tri"])
            e.set_scene(vs["P"][:300], vs["N"][:300], np.zeros((0, 3), np.float32))
            e.view(0, 300, engine_lib.bounce_flags(False), nAz, nEl, -60.0, 120.0 / nAz, rowSin, groundZ=float(vs["v"][:, 2].min()))
            wantv = e.reduce_view(300, wRow, 3, 500.0, reach=[6.0, 20.0])
        finally:
            e.close()
        assert np.array_equal(gotv.view(np.uint64), wantv.view(np.uint64))
        st = srv.stats()
        assert st["completed"] == 15 and st["p99_s"] >= st["p50_s"] > 0
        print("\nserver (budget %.2f GB): %d requests, %d work items, p50 %.1f ms, p99 %.1f ms, chunk %d sensors" %
              (budget_gb, st["completed"], st["items"], 1e3 * st["p50_s"], 1e3 * st["p99_s"], st["chunk_sensors"]))
    finally:
        srv.close()


def _alone_views(kgb, lib, scene, P, N, fov, cell, label):
    nAz, nEl, rowSin, wRow = _views_grid(fov, cell)
    world = fov == 360.0
    e = kgb.Engine(lib)
    try:
        e.build(scene["v"], scene["tri"])
        e.set_labels(label)
        e.set_scene(P, N, np.zeros((0, 3), np.float32))
        e.view(0, len(P), lib.bounce_flags(False), nAz, nEl, 0.0 if world else -fov / 2, fov / nAz, rowSin, world=world, cull=world,
               groundZ=scene["groundZ"])
        return e.reduce_view(len(P), wRow, 6, 300.0, reach=[6.0, 20.0] if world else [], isoDim=3 if world else 0)
    finally:
        e.close()


def test_small_items_equal_alone(engine_lib, kgb, pkg):
    """Work items far smaller than the requests: every daylight request spans several batches and every views request
    several chunks, daylight and views items interleave on the work stream, and each result still equals its request
    run alone, bit for bit."""
    city = pkg.workloads.views_city(seed=3, n_buildings=60, target_tris=6000, n_sensors=1500)
    srv = kgb.Server(engine_lib, 64e9)
    try:
        sid = srv.add_scene(city["v"], city["tri"])
        srv.set_tuning(chunk_sensors=64, batch_rays=1 << 16, view_rays=1 << 16)
        rng = np.random.default_rng(11)
        day, views = [], []
        for k in range(6):
            n = int(rng.integers(300, len(city["P"])))
            first = int(rng.integers(0, len(city["P"]) - n))
            P, N = city["P"][first:first + n], city["N"][first:first + n]
            D = pkg.workloads.hemisphere_dirs(int(rng.integers(100, 400)), int(rng.integers(0, 200)), 20 + k)
            W = rng.uniform(0.0, 2.0, (2, len(D))).astype(np.float32)
            day.append((P, N, D, W, srv.submit(sid, P, N, D, W, [True, False])))
            fov = 120.0 if k % 2 else 360.0
            nAz, nEl, rowSin, wRow = _views_grid(fov, 4.0)
            world = fov == 360.0
            m = int(rng.integers(100, 400))
            Pv, Nv = city["P"][k * 200:k * 200 + m], city["N"][k * 200:k * 200 + m]
            views.append((Pv, Nv, fov, srv.submit_views(sid, Pv, Nv, nAz, nEl, 0.0 if world else -fov / 2, fov / nAz, rowSin, wRow, 6, 300.0,
                                                        reach=[6.0, 20.0] if world else [], isoDim=3 if world else 0, label=city["label"],
                                                        world=world, cull=world, groundZ=city["groundZ"])))
        for P, N, D, W, t in day:
            assert np.array_equal(srv.wait(t), _alone_daylight(kgb, engine_lib, city, P, N, D, W, [True, False]))
        for Pv, Nv, fov, t in views:
            got = srv.wait(t)
            want = _alone_views(kgb, engine_lib, city, Pv, Nv, fov, 4.0, city["label"])
            assert np.array_equal(got.view(np.uint64), want.view(np.uint64))
        st = srv.stats()
        assert st["completed"] == 12 and st["items"] > 40
        print("\nsmall items: %d requests, %d work items, p50 %.1f ms, p99 %.1f ms" % (st["completed"], st["items"], 1e3 * st["p50_s"], 1e3 * st["p99_s"]))
    finally:
        srv.close()


def test_set_tuning_rejects_out_of_range(engine_lib, kgb):
    srv = kgb.Server(engine_lib, 1e9)
    try:
        with pytest.raises(kgb.KgbError, match="chunk 32"):
            srv.set_tuning(chunk_sensors=8)
        with pytest.raises(kgb.KgbError, match="views chunk"):
            srv.set_tuning(view_rays=1 << 40)
    finally:
        srv.close()


def test_chunks_cut_to_the_batch(engine_lib, kgb, pkg):
    """A tuned chunk far larger than a batch's rays and bit pool: each batch takes the part of a chunk that fits, and
    the request's sums equal its run alone."""
    s = pkg.workloads.random_city(4, n_boxes=40)
    srv = kgb.Server(engine_lib, 64e9)
    try:
        sid = srv.add_scene(s["v"], s["tri"])
        srv.set_tuning(chunk_sensors=1 << 20, batch_rays=1 << 22)
        n = min(4000, len(s["P"]))
        P, N = s["P"][:n], s["N"][:n]
        D = pkg.workloads.hemisphere_dirs(5000, 2000, 9)     # 12000 directions: ~350 sensors a batch
        W = np.random.default_rng(2).uniform(0.0, 2.0, (1, len(D))).astype(np.float32)
        got = srv.wait(srv.submit(sid, P, N, D, W, [True]))
        assert np.array_equal(got, _alone_daylight(kgb, engine_lib, s, P, N, D, W, [True]))
        assert srv.stats()["items"] >= n * len(D) // (1 << 22)
    finally:
        srv.close()


def _series_inputs(rng, D_sky_n, P, T, nSun, sun0):
    """Series inputs of one request: nSky sky directions over P patches, T steps, nSun suns on distinct steps."""
    row = rng.integers(0, P, D_sky_n).astype(np.int32)
    wsky = rng.uniform(0.005, 0.05, D_sky_n).astype(np.float32)
    S = rng.uniform(0, 300, (P, T)).astype(np.float32)
    g = rng.uniform(0, 60, T).astype(np.float32)
    steps = np.sort(rng.choice(T, nSun, replace=False)).astype(np.int32)
    return dict(nSky=D_sky_n, row=row, wsky=wsky, S=S, g=g, sun0=sun0, sunStep=steps, sunW=rng.uniform(0, 900, nSun).astype(np.float32))


def _alone_series(kgb, lib, scene, P, N, D, W, use_cos, gQ, si):
    """The request alone through the single-request entry points: trace, the quantities' reduces, the series with G =
    quantity gQ's sums as float (the reference's run loop: gpu_reduce then gpu_series, src/run.cpp:672-687)."""
    e = kgb.Engine(lib)
    try:
        e.build(scene["v"], scene["tri"])
        e.set_scene(P, N, D)
        e.trace(0, len(P), lib.ray_flags(False, False))
        sums = np.stack([e.reduce(len(P), W[q], c) for q, c in enumerate(use_cos)])
        E = e.series(len(P), G=sums[gQ].astype(np.float32), sunVec=D[si["sun0"]:si["sun0"] + len(si["sunStep"])], **si)
        return sums, E
    finally:
        e.close()


@pytest.mark.parametrize("budget_gb", [64, 0.4])
def test_series_requests_equal_alone(engine_lib, kgb, pkg, budget_gb):
    """Daylight requests with time series (145, 577 and 2305 patches, uneven steps and sensor counts) in a stream with
    plain daylight and views requests: every request's sums and series rows equal the request run alone, bit for bit
    (each batch's series chunks run as one grouped tensor-core launch); a small budget serialises admission."""
    scenes = [pkg.workloads.random_city(s, n_boxes=40 + 10 * s) for s in (4, 5)]
    srv = kgb.Server(engine_lib, budget_gb * 1e9)
    try:
        ids = [srv.add_scene(s["v"], s["tri"]) for s in scenes]
        srv.set_tuning(chunk_sensors=1024, batch_rays=1 << 24)   # small chunks: a request's series spans several batches
        rng = np.random.default_rng(8)
        reqs = []
        for k, (patches, T) in enumerate([(145, 300), (577, 700), (2305, 97), (145, 2000), (577, 64), (2305, 400), (145, 7)]):
            sc = k % 2
            s = scenes[sc]
            n = int(rng.integers(100, min(len(s["P"]), 5000)))
            first = int(rng.integers(0, len(s["P"]) - n))
            P, N = s["P"][first:first + n], s["N"][first:first + n]
            nSky = patches + int(rng.integers(0, 100))
            nSun = int(rng.integers(0, min(T, 300) + 1))
            D = pkg.workloads.hemisphere_dirs(nSky, nSun, 100 + k)
            si = _series_inputs(rng, nSky, patches, T, nSun, 2 * nSky)
            W = np.stack([np.concatenate([np.zeros(nSky), rng.uniform(0.001, 0.01, nSky), np.zeros(nSun)]),
                          rng.uniform(0.0, 2.0, len(D))]).astype(np.float32)
            use_cos = [True, bool(k % 2)]
            t = srv.submit_series(ids[sc], P, N, D, W, use_cos, 0, sunVec=D[2 * nSky:], **si)
            reqs.append((sc, P, N, D, W, use_cos, si, t))
            if k == 2:   # plain requests and a views request in between
                Dp = pkg.workloads.hemisphere_dirs(80, 40, 7)
                plain = (sc, P[:700], N[:700], Dp, rng.uniform(0, 1, (2, len(Dp))).astype(np.float32), [True, False])
                tp = srv.submit(ids[plain[0]], *plain[1:])
                nAz, nEl, rowSin, wRow = _views_grid(120.0, 6.0)
                tv = srv.submit_views(ids[0], scenes[0]["P"][:200], scenes[0]["N"][:200], nAz, nEl, -60.0, 120.0 / nAz, rowSin, wRow, 3, 500.0,
                                      groundZ=float(scenes[0]["v"][:, 2].min()))
        for sc, P, N, D, W, use_cos, si, t in reqs:
            sums, E = srv.wait(t)
            want_sums, want_E = _alone_series(kgb, engine_lib, scenes[sc], P, N, D, W, use_cos, 0, si)
            assert np.array_equal(sums.view(np.uint64), want_sums.view(np.uint64))
            assert np.array_equal(E.view(np.uint32), want_E.view(np.uint32)), "%d of %d series values differ (P %d, T %d)" % (
                np.sum(E != want_E), E.size, si["S"].shape[0], si["S"].shape[1])
            assert E.max() > 0
        assert np.array_equal(srv.wait(tp), _alone_daylight(kgb, engine_lib, scenes[plain[0]], *plain[1:]))
        srv.wait(tv)
        assert srv.stats()["completed"] == len(reqs) + 2
    finally:
        srv.close()


def test_series_request_refusals(engine_lib, kgb, pkg):
    s = pkg.workloads.random_city(4, n_boxes=20)
    srv = kgb.Server(engine_lib, 1e9)
    try:
        sid = srv.add_scene(s["v"], s["tri"])
        rng = np.random.default_rng(1)
        D = pkg.workloads.hemisphere_dirs(145, 10, 1)
        si = _series_inputs(rng, 145, 145, 20, 10, 290)
        W = np.ones((1, len(D)), np.float32)
        with pytest.raises(kgb.KgbError, match="gQ is not one of the request's quantities"):
            srv.submit_series(sid, s["P"][:10], s["N"][:10], D, W, [True], 1, sunVec=D[290:], **si)
        bad = dict(si, sunStep=np.array([3, 3, 4, 5, 6, 7, 8, 9, 10, 11], np.int32))
        with pytest.raises(kgb.KgbError, match="two sun directions on one step"):
            srv.submit_series(sid, s["P"][:10], s["N"][:10], D, W, [True], 0, sunVec=D[290:], **bad)
        bad = dict(si, row=np.full(145, 145, np.int32))
        with pytest.raises(kgb.KgbError, match="row is not a patch"):
            srv.submit_series(sid, s["P"][:10], s["N"][:10], D, W, [True], 0, sunVec=D[290:], **bad)
        t = srv.submit_series(sid, s["P"][:0], s["N"][:0], D, W, [True], 0, sunVec=D[290:], **si)   # no sensors: empty results
        out, E = srv.wait(t)
        assert out.shape == (1, 0) and E.shape == (0, 20)
    finally:
        srv.close()
