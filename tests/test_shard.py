"""Sensor ranges across ranks (CPU, gloo, world size 2): each rank traces and reduces its own contiguous sensor range on
the oracle with the scene and directions replicated, and the concatenated row blocks equal the single-rank run bit for
bit; the step time reported is the maximum over ranks. This is the host logic of `bench.py --gpus N`; the kernels it
would run on each GPU are the ones the gpu tests check."""
import os
import socket

import numpy as np
import pytest

from conftest import ORACLE_SO, REPO, oracle_lib, package


def test_sensor_range_partitions():
    shard = package().shard
    for n in (0, 1, 7, 64, 1001):
        for world in (1, 2, 3, 8):
            got = [shard.sensor_range(n, r, world) for r in range(world)]
            assert sum(c for _, c in got) == n
            assert all(got[r][0] + got[r][1] == got[r + 1][0] for r in range(world - 1))
            assert got[0][0] == 0 and max(c for _, c in got) - min(c for _, c in got) <= 1
    with pytest.raises(ValueError):
        shard.sensor_range(10, 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out_dir):
    import sys
    sys.path.insert(0, os.path.join(REPO, "tests"))
    import torch.distributed as dist
    from conftest import package as pkg_of
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        pkg = pkg_of()
        s = pkg.workloads.random_city(3, n_boxes=12)
        D = pkg.workloads.hemisphere_dirs(145, 80, 3)
        W = np.random.default_rng(5).uniform(0.0, 2.0, len(D)).astype(np.float32)
        i0, nc = pkg.shard.sensor_range(len(s["P"]), rank, world)
        o = pkg.kgb.Engine(pkg.kgb.Lib(ORACLE_SO))
        o.build(s["v"], s["tri"])
        o.set_scene(s["P"], s["N"], D)   # every rank holds the whole scene and table; it traces its own range
        o.trace(i0, nc, o.lib.ray_flags(False, False))
        rows = o.reduce(nc, W, True)
        bits = o.download_bits(nc)
        o.close()
        step = pkg.shard.max_over_ranks([1.0 + rank, 5.0 - rank])
        np.save(os.path.join(out_dir, "rows%d.npy" % rank), rows)
        np.save(os.path.join(out_dir, "bits%d.npy" % rank), bits)
        np.save(os.path.join(out_dir, "step%d.npy" % rank), np.array(step))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_ranks_equal_one(tmp_path):
    import torch.multiprocessing as mp
    oracle_lib()   # built before the ranks start
    world, port = 2, _free_port()
    mp.start_processes(_rank, args=(world, port, str(tmp_path)), nprocs=world, start_method="spawn", join=True)
    pkg = package()
    s = pkg.workloads.random_city(3, n_boxes=12)
    D = pkg.workloads.hemisphere_dirs(145, 80, 3)
    W = np.random.default_rng(5).uniform(0.0, 2.0, len(D)).astype(np.float32)
    o = pkg.kgb.Engine(pkg.kgb.Lib(ORACLE_SO))
    try:
        o.build(s["v"], s["tri"])
        o.set_scene(s["P"], s["N"], D)
        n = len(s["P"])
        o.trace(0, n, o.lib.ray_flags(False, False))
        whole, whole_bits = o.reduce(n, W, True), o.download_bits(n)
    finally:
        o.close()
    rows = np.concatenate([np.load(tmp_path / ("rows%d.npy" % r)) for r in range(world)])
    assert np.array_equal(rows.view(np.uint64), whole.view(np.uint64))
    bits = np.concatenate([np.load(tmp_path / ("bits%d.npy" % r)) for r in range(world)], axis=1)   # word-major [nWords x nc]
    assert np.array_equal(bits, whole_bits)
    for r in range(world):
        assert list(np.load(tmp_path / ("step%d.npy" % r))) == [2.0, 5.0]
