"""The scene's preparation on the GPU (kgb_triangulate, kgb_thin_solids) against the reference's own triangulate_into
and thin_solid (src/mesh.cpp:137-168, 275-304) on seeded meshes (tests/golden/mesh, made by the reference's code; its
n-gons through the earcut restatement that the reference's own check_mesh.cpp cases pass on): recentred float
vertices, every triangle and slot, the skipped faces and every slot's thin-solid flags, bit for bit."""
import os

import numpy as np
import pytest

from replay import GOLDEN

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["ngons", "solids"])
def test_mesh_preparation_equals_the_references(engine_lib, kgb, name):
    g = np.load(os.path.join(GOLDEN, "mesh", name + ".npz"))
    e = kgb.Engine(engine_lib)
    try:
        v, tri, slot, skipped = e.triangulate(g["points"], g["counts"], g["indices"], g["slots"].astype(np.uint32), g["c"])
        flags = e.thin_solids(g["points"], g["counts"], g["indices"], g["slots"].astype(np.uint32), len(g["thin"]), g["c"])
        # the same faces offset into a scene: vertex and slot bases add to every index
        _, tri2, slot2, _ = e.triangulate(g["points"], g["counts"], g["indices"], g["slots"].astype(np.uint32), g["c"], base=1000, slot_base=7)
    finally:
        e.close()
    assert np.array_equal(v.view(np.uint32), g["v"].view(np.uint32))
    assert tri.shape == g["tri"].shape and np.array_equal(tri, g["tri"]), "%d of %d triangles differ" % (
        np.sum(np.any(tri != g["tri"], axis=1)) if tri.shape == g["tri"].shape else -1, len(g["tri"]))
    assert np.array_equal(slot, g["slot"]) and skipped == int(g["skipped"])
    assert np.array_equal(tri2, g["tri"] + 1000) and np.array_equal(slot2, g["slot"] + 7)
    assert np.array_equal(flags, g["thin"])
    if name == "ngons":
        assert len(tri) > 5000 and skipped > 0   # n-gons of 5..60 corners, degenerate faces among them


def test_mesh_preparation_refusals(engine_lib, kgb):
    e = kgb.Engine(engine_lib)
    try:
        with pytest.raises(kgb.KgbError, match="corner index exceeds the points"):
            e.triangulate(np.zeros((3, 3)), [3], [0, 1, 3])
        with pytest.raises(kgb.KgbError, match="slot is not below nSlots"):
            e.thin_solids(np.zeros((3, 3)), [3], [0, 1, 2], [2], n_slots=2)
        v, tri, slot, skipped = e.triangulate(np.zeros((0, 3)), np.zeros(0, np.int32), np.zeros(0, np.int32))
        assert len(v) == 0 and len(tri) == 0 and skipped == 0
    finally:
        e.close()
