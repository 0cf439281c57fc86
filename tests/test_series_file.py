"""kgb_series_file on the oracle (CPU): the rows a chunk's series writes to a file at an offset are the bytes
kgb_series returns, and chunks written one after another at their offsets (the reference's --timeseries .npy layout,
run.cpp:535-536, 683-686) give the whole run's rows."""
import os

import numpy as np

from conftest import oracle_lib, package
from test_gpu_series import _inputs


def test_oracle_series_file_matches_series(tmp_path):
    pkg = package()
    lib = oracle_lib()
    s = pkg.workloads.random_city(7, n_boxes=20)
    P, T, nSun, nc = 145, 40, 16, min(300, len(s["P"]))
    D = pkg.workloads.hemisphere_dirs(P, nSun, 7)
    args = _inputs(P, T, nc, D, P, nSun, 3)
    e = pkg.kgb.Engine(lib)
    try:
        e.build(s["v"], s["tri"])
        e.set_scene(s["P"][:nc], s["N"][:nc], D)
        header = 128
        path = str(tmp_path / "series.npy")
        fd = os.open(path, os.O_CREAT | os.O_RDWR | os.O_TRUNC, 0o644)
        try:
            os.pwrite(fd, b"H" * header, 0)
            rows = []
            for i0, m in ((0, 120), (120, nc - 120)):
                e.trace(i0, m, lib.ray_flags(False, False))
                a = dict(args, G=args["G"][i0:i0 + m])
                rows.append(e.series(m, **a))
                e.series_file(m, fd, header + i0 * T * 4, **a)
        finally:
            os.close(fd)
        data = open(path, "rb").read()
        assert data[:header] == b"H" * header and len(data) == header + nc * T * 4
        assert np.array_equal(np.frombuffer(data[header:], np.float32).reshape(nc, T), np.concatenate(rows))
    finally:
        e.close()
