"""The 8-wide BVH layout the GPU kernels walk (CPU): built by the engine's host builder and checked by a CPU decoder of
the same records (tests/bvh_check.cpp): indices in range, every node and triangle referenced exactly once, child boxes
containing their triangles, depth within the traversal stacks. Run before any GPU launch reads the structure."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from conftest import REPO, package

SO = os.path.join(REPO, "tests", "_build", "bvh_check.so")


@pytest.fixture(scope="module")
def checker():
    os.makedirs(os.path.dirname(SO), exist_ok=True)
    src = [os.path.join(REPO, "tests", "bvh_check.cpp"), os.path.join(REPO, "kit-sim_daylight_gb300", "csrc", "bvh_build.cpp")]
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-I" + os.path.join(REPO, "include"), "-I/usr/local/cuda/include",
                           "-o", SO] + src)
    lib = ctypes.CDLL(SO)
    lib.bvh_check.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_char_p, ctypes.c_size_t,
                              ctypes.POINTER(ctypes.c_uint32)]
    return lib


def check(lib, v, tri):
    v = np.ascontiguousarray(v, np.float32)
    tri = np.ascontiguousarray(tri, np.uint32)
    msg = ctypes.create_string_buffer(256)
    depth = ctypes.c_uint32(0)
    r = lib.bvh_check(v.ctypes.data, len(v), tri.ctypes.data, len(tri), msg, 256, ctypes.byref(depth))
    return r, msg.value.decode(), depth.value


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_random_cities(checker, seed):
    s = package().workloads.random_city(seed, porous=True, glass=True, thin=True)
    r, msg, depth = check(checker, s["v"], s["tri"])
    assert r == 0, msg


def test_urban_block(checker):
    s = package().workloads.urban_block()
    r, msg, depth = check(checker, s["v"], s["tri"])
    assert r == 0, msg
    assert depth <= 26


@pytest.mark.parametrize("n", [1, 2, 3, 4, 9, 25, 64])
def test_tiny_and_degenerate(checker, n):
    rng = np.random.default_rng(n)
    v = rng.uniform(-5, 5, (3 * n, 3))
    tri = np.arange(3 * n).reshape(n, 3)
    assert check(checker, v, tri)[0] == 0
    # coincident triangles (identical centroids) and flat / zero-area ones
    v2 = np.repeat(v[:3], n, axis=0)
    assert check(checker, v2, tri)[0] == 0
    v3 = v.copy()
    v3[:, 2] = 0
    assert check(checker, v3, tri)[0] == 0
