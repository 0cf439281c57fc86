"""kgb_reduce_noalloc (GPU): the reduce for callers that must not allocate device memory when they call it (a host that
reserved the GPU's memory for its own pool, a plugin loop that forbids allocation). It stages weights and sums in the
library's fixed 1 MiB device array instead of engine buffers, so
 - its sums must equal kgb_reduce's bit for bit (the reduce tests' tolerance), also on a second call right after the
   first, whose leftovers share that array;
 - the device's free memory must not change across its calls, also right after kgb_trim has released the engine's
   buffers that kgb_reduce would grow again;
 - a call beyond the array's size is refused with the limit in the message.

Collected last (so that a run stopping at the first failure has run every other test before it); one test runs the
two calls in a fresh process as well, where they are the process's first use of the array."""
import json
import os
import subprocess
import sys
from ctypes import c_int, c_size_t, c_void_p

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SCRATCH = 1 << 20
HERE = os.path.dirname(os.path.abspath(__file__))


def noalloc(engine_lib, eng, nc, W, use_cos):
    f = engine_lib.dll.kgb_reduce_noalloc
    f.restype, f.argtypes = c_int, [c_void_p, c_size_t, c_void_p, c_int, c_void_p]
    W = np.ascontiguousarray(W, np.float32)
    out = np.full(nc, np.nan, np.float64)
    ok = f(eng.h, nc, W.ctypes.data_as(c_void_p), int(use_cos), out.ctypes.data_as(c_void_p))
    return out if ok else engine_lib.err()


def two_calls(engine_lib, kgb, pkg, warm=True):
    """Two no-alloc calls in a row on a traced random city, with the device's free bytes read around them (after
    kgb_trim released the engine's chunk buffers), then kgb_reduce on the same weights. Returns a dict of findings.
    warm: one call before the measured ones (with lazy module loading, the process's first call is where the driver
    loads the library's device image that holds the array)."""
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
        if warm:
            noalloc(engine_lib, e, nc, W2, True)
        e.trim(False)   # releases the weight / sum buffers kgb_reduce grows (the trace's visibility goes with them)
        e.trace(0, nc, engine_lib.ray_flags(False, False))
        free0 = engine_lib.dll.kgb_free_bytes()
        first = noalloc(engine_lib, e, nc, W1, True)       # two calls in a row through the fixed array
        second = noalloc(engine_lib, e, nc, W2, False)
        free1 = engine_lib.dll.kgb_free_bytes()
        if isinstance(first, str) or isinstance(second, str):
            return {"error": first if isinstance(first, str) else second}
        return {"free_before": int(free0), "free_after": int(free1),
                "first_equal": bool(np.array_equal(first, e.reduce(nc, W1, True))),
                "second_equal": bool(np.array_equal(second, e.reduce(nc, W2, False))),
                "nonzero_and_distinct": bool(first.sum() > 0 and not np.array_equal(first, second))}
    finally:
        e.close()


def check(r):
    assert "error" not in r, r
    assert r["first_equal"] and r["second_equal"] and r["nonzero_and_distinct"], r
    assert r["free_after"] == r["free_before"], "device free memory changed across the calls: %r" % r


def test_noalloc_reduce_equals_reduce_twice_in_a_row(engine_lib, kgb, pkg):
    check(two_calls(engine_lib, kgb, pkg))


def test_noalloc_reduce_in_a_fresh_process(engine_lib):
    """The same two calls as the first use of the array in a new process. Module loading is eager there, so that the
    library's device image (the array with it) is in place once the context exists, as a caller that must not allocate
    sets up before its loop."""
    code = ("import json, sys; sys.path.insert(0, %r); import conftest, test_zz_no_alloc as t; pkg = conftest.package(); "
            "print(json.dumps(t.two_calls(pkg.load(), pkg.kgb, pkg, warm=False)))" % HERE)
    env = dict(os.environ, CUDA_MODULE_LOADING="EAGER")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600, env=env, cwd=HERE)
    assert r.returncode == 0, r.stderr[-3000:]
    check(json.loads(r.stdout.strip().splitlines()[-1]))


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
        assert isinstance(msg, str) and msg.startswith("kgb_reduce_noalloc:") and "at most %d sensors" % most in msg, msg
        # one sensor fewer fits: the same sums as kgb_reduce on the traced chunk's first `most` sensors
        e.trace(0, most, engine_lib.ray_flags(False, False))
        W = np.ones(nDir, np.float32)
        got = noalloc(engine_lib, e, most, W, True)
        assert not isinstance(got, str), got
        assert np.array_equal(got, e.reduce(most, W, True))
        # a chunk that was not traced is refused with this entry point's own prefix
        msg = noalloc(engine_lib, e, most - 1, W, True)
        assert isinstance(msg, str) and msg.startswith("kgb_reduce_noalloc: no trace of this chunk"), msg
    finally:
        e.close()
