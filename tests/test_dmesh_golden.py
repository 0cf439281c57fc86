"""The .dmesh reader against the reference's own (CPU, on the oracle's restatement; tests/test_gpu_dmesh.py runs the
same checks on the engine, whose arrays are read to and checked on the device).

tests/golden/dmesh/cases.npz holds seeded images and the reference's read_dmesh answer on each (oracle/ref_sky_golden.cpp,
mode dmesh, over src/mesh.cpp:450-478): valid meshes with and without the slot block, trailing bytes, an empty mesh, and
one image per rule of the header and of the arrays, two of them breaking two rules at once. Every answer must match:
success or the exact message, and on success the arrays read. The info the reader adds (slot_count, tri_cap, the
bounds bbox_centre takes, the largest face) is checked against the arrays. The file variant (read_dmesh of a path,
src/mesh.cpp:480-489) names the path in its messages."""
import os

import numpy as np
import pytest

from replay import GOLDEN

CASES = os.path.join(GOLDEN, "dmesh", "cases.npz")


def load_cases():
    g = np.load(CASES)
    names = bytes(g["names"]).decode().split("\n")
    out = []
    for n in names:
        ok, meshes = [int(x) for x in g[n + "/answer"]]
        c = dict(name=n, image=bytes(g[n + "/image"]), ok=bool(ok), meshes=meshes, message=bytes(g[n + "/message"]).decode())
        for k in ("points", "counts", "indices", "slot"):
            if n + "/" + k in g:
                c[k] = g[n + "/" + k]
        out.append(c)
    return out


def expected_info(c):
    P = c["points"].reshape(-1, 3)
    counts, slot = c["counts"], c["slot"]
    lo = [float(np.fmin.reduce(P[:, a])) if len(P) else np.inf for a in range(3)]
    hi = [float(np.fmax.reduce(P[:, a])) if len(P) else -np.inf for a in range(3)]
    return dict(nPoints=len(P), nFaces=len(counts), nIndices=len(c["indices"]), hasSlots=int(len(slot) > 0),
                slots=int(slot.max()) + 1 if len(slot) else 1, maxCorners=int(counts.max()), triCap=int((counts.astype(np.int64) - 2).sum()),
                lo=lo, hi=hi)


def check_reader(lib, kgb, tmp_path):
    """Every golden case through kgb_mesh_read (name "case") and kgb_mesh_file (the image as a file)."""
    cases = load_cases()
    assert len(cases) >= 20 and sum(c["ok"] for c in cases) >= 4
    e = kgb.Engine(lib)
    try:
        for c in cases:
            path = tmp_path / (c["name"] + ".dmesh")
            path.write_bytes(c["image"])
            for how in ("memory", "file"):
                try:
                    info = e.mesh_read(c["image"], "case") if how == "memory" else e.mesh_file(path)
                    got = None
                except kgb.KgbError as err:
                    info, got = None, str(err)
                want = c["message"] if how == "memory" else c["message"].replace("case:", str(path) + ":", 1)
                if not c["ok"]:
                    assert got == want, (c["name"], how, got, want)
                    continue
                assert got is None, (c["name"], how, got)
                if not c["meshes"]:
                    assert info.id == kgb.NO_MESH, c["name"]
                    continue
                assert info.id != kgb.NO_MESH
                P, C, I, S = e.mesh_download(info)
                assert np.array_equal(P.ravel().view(np.uint64), c["points"].view(np.uint64)), c["name"]
                assert np.array_equal(C, c["counts"]) and np.array_equal(I, c["indices"]), c["name"]
                assert np.array_equal(S if S is not None else np.zeros(0, np.uint16), c["slot"]), c["name"]
                d = info.as_dict()
                for k, v in expected_info(c).items():
                    assert d[k] == v, (c["name"], how, k, d[k], v)
                e.mesh_free(info.id)
        with pytest.raises(kgb.KgbError, match="^cannot open " + str(tmp_path / "absent.dmesh") + "$"):
            e.mesh_file(tmp_path / "absent.dmesh")
        with pytest.raises(kgb.KgbError, match="no mesh"):
            e.mesh_free(12345)
    finally:
        e.close()


def test_golden_answers_are_the_references():
    """The fixture's answers are the reference's own words (src/mesh.cpp:453-461, 436-445)."""
    msgs = {c["name"]: c["message"] for c in load_cases()}
    assert msgs["bad_magic"] == "case: not a .dmesh file (magic DLM1)"
    assert msgs["face_of_two_and_bad_index"] == "case: face with fewer than 3 vertices"
    assert msgs["sum_mismatch_and_bad_index"] == "case: sum(counts) != n_indices"
    assert msgs["truncated_slot_block"] == "case: truncated slot block"


def test_oracle_reader_matches_the_reference(oracle, kgb, tmp_path):
    check_reader(oracle, kgb, tmp_path)
