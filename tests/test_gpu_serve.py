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
        print("\nserver (budget %.2f GB): %d requests, %d batches, p50 %.1f ms, p99 %.1f ms, chunk %d sensors" %
              (budget_gb, st["completed"], st["batches"], 1e3 * st["p50_s"], 1e3 * st["p99_s"], st["chunk_sensors"]))
    finally:
        srv.close()
