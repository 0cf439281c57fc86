"""Meshes read straight to the device (GPU): kgb_mesh_read / kgb_mesh_file against the reference's read_dmesh
(tests/golden/dmesh, the same checks test_dmesh_golden.py runs on the oracle), and the scene built from kept meshes
(kgb_build_meshes: run.cpp's scene assembly and gpu_build with no array of the scene on the host) against the same scene
built from host arrays that kgb_triangulate produced (pinned to the reference's triangulate_into by
tests/golden/mesh): equal visibility bits on the engine and on the oracle."""
import os

import numpy as np
import pytest

from replay import GOLDEN
from test_dmesh_golden import check_reader
from test_dmesh_golden import expected_info

pytestmark = pytest.mark.gpu


def image(P, C, I, S=None):
    fl = 1 if S is not None else 0
    head = b"DLM1" + np.array([fl], np.uint32).tobytes() + np.array([len(P), len(C), len(I)], np.uint64).tobytes()
    return head + np.ascontiguousarray(P, np.float64).tobytes() + np.ascontiguousarray(C, np.int32).tobytes() + \
        np.ascontiguousarray(I, np.int32).tobytes() + (np.ascontiguousarray(S, np.uint16).tobytes() if S is not None else b"")


def readable(name):
    """A golden mesh of tests/golden/mesh as the .dmesh reader accepts it: faces of fewer than 3 corners (which the
    triangulation test keeps, as skipped faces) left out."""
    g = np.load(os.path.join(GOLDEN, "mesh", name + ".npz"))
    C, I, S = g["counts"], g["indices"], g["slots"]
    start = np.concatenate([[0], np.cumsum(C)[:-1]])
    keep = C >= 3
    I2 = np.concatenate([I[a:a + n] for a, n in zip(start[keep], C[keep])]) if keep.any() else np.zeros(0, np.int32)
    return g["points"], C[keep], I2.astype(np.int32), S[keep], g


def quad_grid(n, x0, y0, step, z=0.0, wave=0.0, seed=0):
    """An n x n grid of quads (the reference's ingest benchmark shape), a slot per face in 0..2."""
    xs, ys = np.meshgrid(np.arange(n + 1, dtype=np.float64), np.arange(n + 1, dtype=np.float64), indexing="ij")
    P = np.stack([x0 + xs.ravel() * step, y0 + ys.ravel() * step, z + wave * np.sin(xs.ravel() * 0.7) * np.cos(ys.ravel() * 0.3)], 1)
    q = np.arange(n * (n + 1)).reshape(n, n + 1)[:, :n].ravel()
    I = np.stack([q, q + n + 1, q + n + 2, q + 1], 1).astype(np.int32).ravel()
    S = np.random.default_rng(seed).integers(0, 3, n * n).astype(np.uint16)
    return P, np.full(n * n, 4, np.int32), I, S


def test_reader_matches_the_reference(engine_lib, kgb, tmp_path):
    check_reader(engine_lib, kgb, tmp_path)


def test_large_file_to_the_device(engine_lib, oracle, kgb, tmp_path):
    """A 1000 x 1000 quad grid with n-gons appended (46 MB with slots: two of the reader's 32 MiB slices) read from a
    file: arrays and info as the oracle's reader gives them."""
    P, C, I, S = quad_grid(1000, -500.0, -500.0, 1.0, wave=2.0, seed=3)
    gP, gC, gI, gS, _ = readable("ngons")
    P2 = np.concatenate([P, gP])
    C2 = np.concatenate([C, gC])
    I2 = np.concatenate([I, gI + len(P)])
    S2 = np.concatenate([S, gS])
    path = tmp_path / "grid.dmesh"
    path.write_bytes(image(P2, C2, I2, S2))
    assert os.path.getsize(path) > 40 << 20
    infos, arrays = [], []
    for lib in (engine_lib, oracle):
        e = kgb.Engine(lib)
        try:
            info = e.mesh_file(path)
            infos.append(info.as_dict())
            arrays.append(e.mesh_download(info))
        finally:
            e.close()
    assert infos[0] == infos[1]
    c = dict(points=P2.ravel(), counts=C2, indices=I2, slot=S2)
    for k, v in expected_info(c).items():
        assert infos[0][k] == v, k
    for a, b in zip(*arrays):
        assert np.array_equal(a.view(np.uint8), b.view(np.uint8))


def scene_meshes():
    """Four meshes in a run's order: a slotted ground grid, the n-gon golden mesh, a mesh that does not block, and the
    thin-solid golden mesh (slot bases count every mesh, points and triangles only the blocking ones)."""
    out = []
    P, C, I, S = quad_grid(40, -60.0, -60.0, 3.0, wave=0.5, seed=5)
    out.append((P, C, I, S, True))
    for name in ("ngons", "solids"):
        P, C, I, S, _ = readable(name)
        if name == "ngons":   # and a pentagon without area (collinear corners): a skipped face
            P = np.concatenate([P, np.stack([np.arange(5.0), np.zeros(5), np.zeros(5)], 1)])
            C, I, S = np.append(C, 5).astype(np.int32), np.append(I, np.arange(len(P) - 5, len(P))).astype(np.int32), np.append(S, 0).astype(np.uint16)
        out.append((P, C, I, S, True))
        if name == "ngons":
            Pn, Cn, In, Sn = quad_grid(6, -20.0, -20.0, 2.0, z=15.0)
            out.append((Pn, Cn, In, None, False))
    return out


def host_scene(e, meshes, c):
    """run.cpp:98-150's layout from kgb_triangulate's host outputs."""
    vs, ts, ss, made = [], [], [], []
    vBase = sBase = 0
    for P, C, I, S, blocks in meshes:
        nslots = int(S.max()) + 1 if S is not None else 1
        if blocks:
            v, tri, slot, _ = e.triangulate(P, C, I, None if S is None else S.astype(np.uint32), c, base=vBase, slot_base=sBase)
            vs.append(v); ts.append(tri); ss.append(slot); made.append(len(tri))
            vBase += len(P)
        else:
            made.append(0)
        sBase += nslots
    return np.concatenate(vs), np.concatenate(ts), np.concatenate(ss), np.array(made, np.uint64), sBase


@pytest.mark.parametrize("per_slot", [False, True])
def test_scene_from_kept_meshes(engine_lib, oracle, kgb, pkg, per_slot):
    meshes = scene_meshes()
    e = kgb.Engine(engine_lib)
    o = kgb.Engine(oracle)
    try:
        infos = [e.mesh_read(image(P, C, I, S), "m%d" % k) for k, (P, C, I, S, _) in enumerate(meshes)]
        lo = np.min([i.lo[:] for i in infos], axis=0)
        hi = np.max([i.hi[:] for i in infos], axis=0)
        c = np.where(lo <= hi, (lo + hi) / 2, 0.0)   # bbox_centre
        v, tri, slot, made_h, nSlots = host_scene(e, meshes, c)
        slots = [(0.2, 0.0, 0.0, 0)] * nSlots
        if per_slot:
            slots[5] = (0.0, 0.6, kgb.tn_from_Tn(0.6), kgb.SLOT_GLASS)   # a glass slot of the n-gon mesh
        made, skipped = e.build_meshes([i.id for i in infos], c, blocks=[m[4] for m in meshes], slots=slots, per_slot=per_slot)
        assert np.array_equal(made, made_h) and made[2] == 0
        rng = np.random.default_rng(9)
        Ps = np.concatenate([rng.uniform(-50, 50, (300, 2)), rng.uniform(0.5, 20, (300, 1))], 1).astype(np.float32) - c.astype(np.float32)
        Ns = np.tile(np.array([[0, 0, 1]], np.float32), (300, 1))
        D = pkg.workloads.hemisphere_dirs(145, 60, 4)
        flags = engine_lib.ray_flags(False, per_slot)
        e.set_slots(slots)
        e.set_scene(Ps, Ns, D)
        e.trace(0, 300, flags)
        got = e.download_bytes(300) if per_slot else e.download_bits(300)
        # the same scene from host arrays, on the engine and on the oracle
        for lib, x in ((engine_lib, e), (oracle, o)):
            x.build(v, tri, slot, slots, per_slot=per_slot)
            x.set_slots(slots)
            x.set_scene(Ps, Ns, D)
            x.trace(0, 300, flags)
            want = x.download_bytes(300) if per_slot else x.download_bits(300)
            assert np.array_equal(got, want), lib.path
        assert skipped > 0   # the n-gon mesh's faces without area
        # the thin-solid test on a kept mesh: the golden solids where the reference tested them
        g = np.load(os.path.join(GOLDEN, "mesh", "solids.npz"))
        solids = e.mesh_read(image(g["points"], g["counts"], g["indices"], g["slots"]), "solids")
        assert np.array_equal(e.mesh_thin_solids(solids, g["c"]), g["thin"])
    finally:
        e.close()
        o.close()


def test_scene_from_kept_meshes_refusals(engine_lib, kgb):
    """kgb_build_meshes refuses an unknown mesh and a slot beyond the table (gpu_build's own message), builds an empty
    scene from meshes that do not block (every ray misses), and kgb_mesh_thin_solids refuses an unknown mesh."""
    P, C, I, _ = quad_grid(4, 0.0, 0.0, 1.0, seed=1)
    S = (np.arange(16) % 3).astype(np.uint16)
    e = kgb.Engine(engine_lib)
    try:
        info = e.mesh_read(image(P, C, I, S), "grid")
        with pytest.raises(kgb.KgbError, match="no mesh 77"):
            e.build_meshes([info.id, 77], (2.0, 2.0, 0.0))
        with pytest.raises(kgb.KgbError, match="a triangle's slot has no Slot"):
            e.build_meshes([info.id], (2.0, 2.0, 0.0), slots=[(0.2, 0.0, 0.0, 0)], per_slot=True)   # slots 0..2 in the mesh
        made, skipped = e.build_meshes([info.id], (2.0, 2.0, 0.0), blocks=[0])
        assert made.tolist() == [0] and skipped == 0
        Ps = np.array([[0.5, 0.5, 5.0]], np.float32)
        e.set_scene(Ps, np.array([[0, 0, -1]], np.float32), np.array([[0, 0, -1]], np.float32))
        e.trace(0, 1, engine_lib.ray_flags(False, False))
        assert e.download_bits(1)[0, 0] & 1   # nothing blocks: the ray down to the grid sees through
        made, _ = e.build_meshes([info.id], (2.0, 2.0, 0.0), slots=[(0.2, 0.0, 0.0, 0)] * 3, per_slot=True)
        assert made.tolist() == [32]
        e.trace(0, 1, engine_lib.ray_flags(False, False))
        assert not e.download_bits(1)[0, 0] & 1   # the grid blocks it now
        with pytest.raises(kgb.KgbError, match="no mesh"):
            e.mesh_thin_solids(kgb.MeshInfo(id=999, slots=1))
        e.mesh_free(info.id)
        with pytest.raises(kgb.KgbError, match="no mesh"):
            e.build_meshes([info.id], (0.0, 0.0, 0.0))
    finally:
        e.close()

