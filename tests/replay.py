"""Replays a recorded run of the reference's host code (tests/golden/<case>/calls.jsonl, written by the engine shim's
recorder) on a library that exports the engine's C ABI, and compares every result with the recording.

Bit-exact: visibility bits / bytes, reflected-light rows, view classes and distances, and the doubles of gpu_reduce,
gpu_reduce_dc and gpu_reduce_view (fixed summation orders). The FP32 time series (gpu_series) is compared with the
recording, the oracle's FP64 contraction, within SERIES_RTOL relative (+ SERIES_ATOL absolute).
"""
import ctypes
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
SERIES_RTOL, SERIES_ATOL = 1e-5, 1e-3


def cases():
    return sorted(d for d in os.listdir(GOLDEN) if os.path.exists(os.path.join(GOLDEN, d, "calls.jsonl")))


def load_calls(case):
    d = os.path.join(GOLDEN, case)
    calls = [json.loads(l) for l in open(os.path.join(d, "calls.jsonl"))]

    def arr(c, k, raw=False):
        dtype, shape, name = c[k]
        data = np.fromfile(os.path.join(d, name), dtype=np.uint8 if raw else np.dtype(dtype))
        return data if raw else data.reshape(shape)
    return calls, arr


def urban_sky():
    """The urban block's direction table D [nDir x 3] and its per-quantity weights [(W, useCos)] as the reference's host
    code made them (the last gpu_set_scene of the urban_sky recording and the gpu_reduce calls after it)."""
    calls, arr = load_calls("urban_sky")
    last = max(i for i, c in enumerate(calls) if c["call"] == "gpu_set_scene")
    D = arr(calls[last], "D").reshape(-1, 3)
    Ws = [(arr(c, "W"), bool(c["useCos"])) for c in calls[last:] if c["call"] == "gpu_reduce"]
    return D, Ws


def _slots(raw, kgb):
    n = raw.size // 16
    return (kgb.Slot * max(n, 1)).from_buffer_copy(raw.tobytes() if n else bytes(16))


def replay(engine, kgb, case, check=True):
    """Runs the recorded calls on `engine` (a kgb.Engine); returns a list of (seq, call, mismatch description)."""
    calls, arr = load_calls(case)
    bad = []
    nc_trace = 0
    for c in calls:
        name = c["call"]
        if not c["ok"]:
            continue
        if name == "gpu_build":
            v, tri = arr(c, "v"), arr(c, "tri")
            slot = arr(c, "slot")
            sl = _slots(arr(c, "slots", raw=True), kgb)
            engine._ok(engine.d.kgb_build(engine.h, v.ctypes.data_as(ctypes.c_void_p) if v.size else None, len(v),
                                          tri.ctypes.data_as(ctypes.c_void_p) if tri.size else None, len(tri),
                                          slot.ctypes.data_as(ctypes.c_void_p) if slot.size else None, ctypes.cast(sl, ctypes.c_void_p),
                                          len(sl) if arr(c, "slots", raw=True).size else 0, int(c["perSlot"])))
        elif name == "gpu_set_slots":
            raw = arr(c, "slots", raw=True)
            sl = _slots(raw, kgb)
            engine._ok(engine.d.kgb_set_slots(engine.h, ctypes.cast(sl, ctypes.c_void_p), raw.size // 16))
        elif name == "gpu_set_scene":
            engine.set_scene(arr(c, "P"), arr(c, "N"), arr(c, "D"))
        elif name == "gpu_set_labels":
            engine.set_labels(arr(c, "label"))
        elif name == "gpu_trace":
            nc = int(c["nc"])
            nc_trace = nc
            engine.trace(int(c["i0"]), nc, int(c["rayFlags"]))
            if check and nc:
                if "bits" in c:
                    got, want = engine.download_bits(nc), arr(c, "bits")
                else:
                    got, want = engine.download_bytes(nc), arr(c, "bytes")
                if not np.array_equal(got, want):
                    bad.append((c["seq"], name, "%d of %d visibility words/bytes differ" % (np.sum(got != want), want.size)))
        elif name == "gpu_reduce":
            out = engine.reduce(int(c["nc"]), arr(c, "W"), bool(c["useCos"]))
            want = arr(c, "out")
            if check and not np.array_equal(out, want):
                bad.append((c["seq"], name, "max abs diff %.3g" % np.max(np.abs(out - want))))
        elif name == "gpu_reduce_dc":
            out = engine.reduce_dc(int(c["nc"]), arr(c, "W"))
            want = arr(c, "out")
            if check and not np.array_equal(out, want):
                bad.append((c["seq"], name, "max abs diff %.3g" % np.max(np.abs(out - want))))
        elif name == "gpu_series":
            nc = int(c["nc"])
            E = engine.series(nc, int(c["nSky"]), arr(c, "row"), arr(c, "wsky"), arr(c, "S"), arr(c, "g"), arr(c, "G"), int(c["sun0"]),
                              arr(c, "sunStep"), arr(c, "sunVec"), arr(c, "sunW"), arr(c, "Sdc") if "Sdc" in c else None)
            want = arr(c, "E")
            if check and not np.allclose(E, want, rtol=SERIES_RTOL, atol=SERIES_ATOL):
                bad.append((c["seq"], name, "max rel diff %.3g" % np.max(np.abs(E - want) / np.maximum(np.abs(want), 1e-3))))
        elif name == "gpu_bounce":
            nc = int(c["nc"])
            engine.bounce(int(c["i0"]), nc, int(c["rayFlags"]), N=int(c["N"]), M=int(c["M"]), mf=int(c["mf"]), north=float(c["north"]))
            if check and nc:
                got, want = engine.download_dc(nc), arr(c, "dc")
                if not np.array_equal(got, want):
                    bad.append((c["seq"], name, "%d of %d reflected-light coefficients differ (max %.3g)" %
                                (np.sum(got != want), want.size, np.max(np.abs(got - want)))))
        elif name == "gpu_view":
            nc = int(c["nc"])
            engine.view(int(c["i0"]), nc, int(c["rayFlags"]), int(c["nAz"]), int(c["nEl"]), float(c["az0"]), float(c["dAz"]),
                        arr(c, "rowSin"), world=bool(c["world"]), cull=bool(c["cull"]), jitter=bool(c["jitter"]), back=bool(c["back"]),
                        vground=bool(c["vground"]), nS=int(c["nS"]), groundZ=float(c["groundZ"]), north=float(c["north"]),
                        launch=int(c["launch"]))
            if check and nc and "cls" in c:
                cls, dist = engine.download_view(nc)
                wc, wd = arr(c, "cls"), arr(c, "dist")
                if not np.array_equal(cls, wc):
                    bad.append((c["seq"], name, "%d of %d ray classes differ" % (np.sum(cls != wc), wc.size)))
                if not np.array_equal(dist.view(np.uint32), wd.view(np.uint32)):
                    bad.append((c["seq"], name, "%d of %d ray distances differ" % (np.sum(dist != wd), wd.size)))
        elif name == "gpu_reduce_view":
            out = engine.reduce_view(int(c["nc"]), arr(c, "wRow"), int(c["nClass"]), float(c["farDist"]), arr(c, "reach"),
                                     bool(c["glazing"]), int(c["isoDim"]))
            want = arr(c, "out")
            if check and not np.array_equal(out.view(np.uint64), want.view(np.uint64)):
                bad.append((c["seq"], name, "max abs diff %.3g" % np.nanmax(np.abs(out - want))))
        else:
            raise AssertionError("unknown recorded call " + name)
    return bad
