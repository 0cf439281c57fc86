"""kgb_reduce_noalloc (GPU): the reduce for callers that must not allocate device memory when they call it (a host that
reserved the GPU's memory for its own pool, a plugin loop that forbids allocation). It stages weights and sums in the
library's fixed 1 MiB device array instead of engine buffers, so its sums must equal kgb_reduce's bit for bit (the
reduce tests' tolerance), also on a second call right after the first, whose leftovers share that array.

Collected last, so it runs after every other GPU test as well as alone in a fresh process."""
import ctypes
from ctypes import c_int, c_size_t, c_void_p

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SCRATCH = 1 << 20


def noalloc(engine_lib, eng, nc, W, use_cos):
    f = engine_lib.dll.kgb_reduce_noalloc
    f.restype, f.argtypes = c_int, [c_void_p, c_size_t, c_void_p, c_int, c_void_p]
    W = np.ascontiguousarray(W, np.float32)
    out = np.full(nc, np.nan, np.float64)
    ok = f(eng.h, nc, W.ctypes.data_as(c_void_p), int(use_cos), out.ctypes.data_as(c_void_p))
    return out if ok else engine_lib.err()


def test_noalloc_reduce_equals_reduce_twice_in_a_row(engine_lib, kgb, pkg):
    s = pkg.workloads.random_city(3)
    D = pkg.workloads.hemisphere_dirs(145, 400, 3)
    e = kgb.Engine(engine_lib)
    try:
        e.build(s["v"], s["tri"])
        e.set_scene(s["P"], s["N"], D)
        nc = len(s["P"])
        e.trace(0, nc, engine_lib.ray_flags(False, False))
        rng = np.random.default_rng(7)
        W1, W2 = rng.uniform(0.001, 2.0, len(D)), rng.uniform(0.5, 900.0, len(D))
        first = noalloc(engine_lib, e, nc, W1, True)       # two calls in a row through the fixed array
        second = noalloc(engine_lib, e, nc, W2, False)
        assert not isinstance(first, str), first
        assert not isinstance(second, str), second
        assert np.array_equal(first, e.reduce(nc, W1, True))
        assert np.array_equal(second, e.reduce(nc, W2, False))
        assert first.sum() > 0 and not np.array_equal(first, second)
    finally:
        e.close()


def test_noalloc_reduce_refuses_a_call_beyond_its_array(engine_lib, kgb, pkg):
    s = pkg.workloads.random_city(3, n_boxes=40)   # 6251 sensors
    nDir = 250_000                     # 1,000,192 bytes of weights: room for 6048 sums
    D = np.tile(pkg.workloads.hemisphere_dirs(1000, 0, 1)[:1000], (nDir // 1000, 1))
    wBytes = (nDir * 4 + 255) // 256 * 256
    most = (SCRATCH - wBytes) // 8
    nc = most + 1
    assert len(s["P"]) >= nc
    e = kgb.Engine(engine_lib)
    try:
        e.build(s["v"], s["tri"])
        e.set_scene(s["P"][:nc], s["N"][:nc], D)
        e.trace(0, nc, engine_lib.ray_flags(False, False))
        msg = noalloc(engine_lib, e, nc, np.ones(nDir, np.float32), True)
        assert isinstance(msg, str) and "at most %d sensors" % most in msg, msg
        # one sensor fewer fits: the same sums as kgb_reduce on the traced chunk's first `most` sensors
        e.trace(0, most, engine_lib.ray_flags(False, False))
        W = np.ones(nDir, np.float32)
        got = noalloc(engine_lib, e, most, W, True)
        assert not isinstance(got, str), got
        assert np.array_equal(got, e.reduce(most, W, True))
    finally:
        e.close()
