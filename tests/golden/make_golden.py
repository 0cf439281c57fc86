"""Generates the golden fixtures under tests/golden/ (run here, where the reference tree is present; the GPU machine only
reads the committed fixtures).

Each case runs the reference's own host code - its C ABI dl_run (kit-sim_daylight src/c_api.cpp) with the CLI's flags,
compiled from the reference tree by `make -C oracle ref` - on the oracle behind the engine's C++ shim, with the shim's
recorder on (KGB_RECORD): every call at the engine boundary (gpu_build, gpu_set_scene, gpu_trace, gpu_reduce, ...) is
written with its inputs and results to tests/golden/<case>/. The tests replay them on the engine and on the oracle.

It also extracts the reference's published outputs for tests/box.obj from its docs (docs/daylight.md, docs/views.md:
the example blocks) into published.json, and checks the recorded runs against them.

usage: python tests/golden/make_golden.py [--ref REFERENCE_CHECKOUT] [--only urban_ladybug,ladybug,mesh,...]
       (the reference: $KITSIM_REFERENCE, else ../reference beside the repo)
"""
import argparse
import ctypes
import json
import os
import shutil
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
DL_DAYLIGHT, DL_VIEWS = 0, 1

CASES = {
    # the box scene: box.obj, a clear-sky year in Berlin, Tregenza sky (docs/daylight.md:133-149 publishes radiation + sunhours)
    "box_clearsky": (DL_DAYLIGHT, ["--clear-sky", "--lat", "52.52", "--lon", "13.41", "--quantity", "radiation,direct,diffuse,sunhours"]),
    # sun hours of 21 June in 10-minute steps (docs/daylight.md:163-179)
    "box_sunhours_day": (DL_DAYLIGHT, ["--quantity", "sunhours", "--lat", "52.52", "--lon", "13.41", "--tz", "1", "--from", "06-21T00:00",
                                       "--to", "06-22T00:00", "--step", "10"]),
    # a week of time series with the box as glass (byte mode), reflected light (bounce pass, --sky-density 2 bins),
    # every quantity: gpu_trace bytes, gpu_bounce, gpu_reduce_dc, gpu_series with Sdc
    "box_week_glass": (DL_DAYLIGHT, ["--clear-sky", "--lat", "52.52", "--lon", "13.41", "--from", "06-01T00:00", "--to", "06-08T00:00",
                                     "--quantity", "radiation,irradiance,illuminance,sunhours", "--timeseries", "@TMP@/series.npy",
                                     "--optics", "box=0,0.64,glass;ground=0.25", "--transmission", "on", "--bounces", "2",
                                     "--bounce-samples", "256", "--sky-density", "2", "--patch-samples", "4"]),
    # views defaults (docs/views.md:333-349)
    "box_views": (DL_VIEWS, []),
    # views all around at 4 degree cells: isovist volume, reach 6/20/50, the box as a target group, jitter on
    "box_views360": (DL_VIEWS, ["--fov", "360", "--cell", "4", "--reach", "en17037", "--target", "box=landmark", "--distance",
                                "isovist,mean,min,group"]),
    # the urban block's sky: the direction table (577 Reinhart patches, their ground mirror, the sun-up hours)
    # and the per-quantity weights under the synthetic urban weather, from a one-quad run (they do not depend on the
    # geometry); the bench traces the full block with them
    "urban_sky": (DL_DAYLIGHT, ["--epw", "@TMP@/urban.epw", "--sky-density", "2", "--quantity", "radiation,irradiance,illuminance,sunhours"]),
    # ladybug mode on the same weather year (gendaymtx -A as ladybug runs it: .wea-rounded site and irradiance, float
    # accumulation, %.3g): its weights pin the ladybug goldens below (tests/golden/ladybug)
    "urban_ladybug": (DL_DAYLIGHT, ["--epw", "@TMP@/urban.epw", "--mode", "ladybug", "--sky-density", "2", "--quantity", "radiation,direct,diffuse"]),
}
MESH = {"urban_sky": "quad", "urban_ladybug": "quad"}   # cases on one 1 m quad instead of tests/box.obj
LADYBUG_COLS = 256   # series columns of the ladybug goldens kept (the first ones)


def urban_weather(ref, tmp):
    """The synthetic EPW of the urban configs: the reference's clear sky (Ineichen, TL 3) at Berlin, each hour's DNI and
    DHI times a cloud factor c ~ Beta(2, 1.5) with 3-day AR(1) persistence (Gaussian copula, rho = exp(-1/72),
    numpy seed 2024). Written as an 8760-row EPW with the LOCATION Berlin 52.52 N 13.41 E, UTC+1."""
    from scipy import special, stats
    dump = os.path.join(tmp, "sun.txt")
    L, run = _lib(ref)
    run(L, DL_DAYLIGHT, ["--clear-sky", "--lat", "52.52", "--lon", "13.41", "--tz", "1", "--quantity", "radiation", "--dump-sun", dump], "quad")
    rows = [l.split() for l in open(dump) if not l.startswith("#")]
    dni = np.array([float(r[10]) for r in rows])
    dhi = np.array([float(r[11]) for r in rows])
    assert len(dni) == 8760
    rng = np.random.default_rng(2024)
    rho = np.exp(-1 / 72)
    z = np.zeros(8760)
    z[0] = rng.standard_normal()
    for t in range(1, 8760):
        z[t] = rho * z[t - 1] + np.sqrt(1 - rho * rho) * rng.standard_normal()
    c = stats.beta.ppf(0.5 * special.erfc(-z / np.sqrt(2)), 2.0, 1.5)
    head = ["LOCATION,Berlin synthetic,,DEU,synthetic,000000,52.52,13.41,1.0,34.0", "DESIGN CONDITIONS,0", "TYPICAL/EXTREME PERIODS,0",
            "GROUND TEMPERATURES,0", "HOLIDAYS/DAYLIGHT SAVINGS,No,0,0,0", "COMMENTS 1,clear sky x Beta(2 1.5) AR(1) cloud factor",
            "COMMENTS 2,kit-sim GB300 urban configs", "DATA PERIODS,1,1,Data,Sunday, 1/ 1,12/31"]
    with open(os.path.join(tmp, "urban.epw"), "w") as f:
        f.write("\n".join(head) + "\n")
        t = 0
        for m, nd in enumerate([31, 28, 31, 30, 31, 30, 31, 31, 30, 31, 30, 31], 1):
            for d in range(1, nd + 1):
                for h in range(1, 25):
                    f.write("2017,%d,%d,%d,60,?,10,5,70,101325,0,0,300,0,%.1f,%.1f\n" % (m, d, h, c[t] * dni[t], c[t] * dhi[t]))
                    t += 1
    np.save(os.path.join(os.path.dirname(tmp), "cloud_factor.npy"), c.astype(np.float32))
    # the weather as written (%.1f W/m2), for the sky side of the bench's precision config
    w = np.stack([np.round(c * dni, 1), np.round(c * dhi, 1)]).astype(np.float32)
    np.save(os.path.join(os.path.dirname(tmp), "weather.npy"), w)


def lib_of(ref):
    return os.path.join(REPO, "oracle", "_ref", "libdaylight_ref.so")


def _lib(ref):
    L = ctypes.CDLL(lib_of(ref))
    L.dl_mesh_load.restype = ctypes.c_void_p
    L.dl_mesh_load.argtypes = [ctypes.c_char_p]
    L.dl_last_error.restype = ctypes.c_char_p
    L.dl_run.argtypes = [ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(ctypes.c_char_p), ctypes.POINTER(ctypes.c_void_p), ctypes.c_int32,
                         ctypes.POINTER(ctypes.c_void_p), ctypes.c_int32, ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)]
    L.dl_result_rows.argtypes = L.dl_result_cols.argtypes = [ctypes.c_void_p]
    L.dl_result_rows.restype = L.dl_result_cols.restype = ctypes.c_int64
    L.dl_result_values.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64]
    L.dl_result_manifest.argtypes = [ctypes.c_void_p]
    L.dl_result_manifest.restype = ctypes.c_char_p
    L.dl_mesh_create.restype = ctypes.c_void_p
    L.dl_mesh_create.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                 ctypes.c_int64, ctypes.c_void_p]

    def run(L, tool, argv, mesh_kind):
        if mesh_kind == "quad":   # one 1 m roof quad facing up
            xyz = np.array([0, 0, 10, 1, 0, 10, 1, 1, 10, 0, 1, 10], np.float64)
            counts = np.array([4], np.int32)
            idx = np.array([0, 1, 2, 3], np.int32)
            mesh = L.dl_mesh_create(b"roof", xyz.ctypes.data, 4, counts.ctypes.data, 1, idx.ctypes.data, 4, None)
        else:
            mesh = L.dl_mesh_load(os.path.join(ref, "tests", "box.obj").encode())
        assert mesh, L.dl_last_error()
        args = (ctypes.c_char_p * len(argv))(*[a.encode() for a in argv])
        sensors = (ctypes.c_void_p * 1)(mesh)
        res = ctypes.c_void_p()
        rc = L.dl_run(tool, len(argv), args, sensors, 1, None, 0, None, ctypes.byref(res))
        assert rc == 0, (rc, L.dl_last_error())
        return res
    return L, run


def run_case(name, ref):
    """In a child process: KGB_RECORD must be set before the library is loaded."""
    tool, argv = CASES[name]
    out = os.path.join(HERE, name)
    tmp = os.path.join(out, "_tmp")
    os.makedirs(tmp, exist_ok=True)
    argv = [a.replace("@TMP@", tmp) for a in argv]
    if name in ("urban_sky", "urban_ladybug"):
        urban_weather(ref, tmp)
    L, run = _lib(ref)
    res = run(L, tool, argv, MESH.get(name, "box"))
    rows, cols = L.dl_result_rows(res), L.dl_result_cols(res)
    vals = np.zeros(rows * cols, np.float64)
    L.dl_result_values(res, vals.ctypes.data, vals.size)
    np.save(os.path.join(out, "result.npy"), vals.reshape(rows, cols))
    with open(os.path.join(out, "manifest.json"), "w") as f:
        f.write(L.dl_result_manifest(res).decode())
    shutil.rmtree(tmp, ignore_errors=True)


def published(ref):
    """The example outputs the reference's docs print for tests/box.obj (numbers only, as printed)."""
    out = {}
    txt = open(os.path.join(ref, "docs", "daylight.md")).read()
    i = txt.index("daylight tests/box.obj --clear-sky --lat 52.52 --lon 13.41 --quantity radiation,sunhours")
    blk = txt[i:].split("```")[0].strip().splitlines()[1:]
    out["box_clearsky"] = {"source": "docs/daylight.md (tests/box.obj, a clear-sky year in Berlin)", "columns": ["radiation_front", "sunhours_front"],
                           "values": [[float(x) for x in l.split()] for l in blk]}
    i = txt.index("daylight tests/box.obj --quantity sunhours --lat 52.52 --lon 13.41 --tz 1 --from 06-21T00:00")
    blk = txt[i:].split("```")[0].strip().splitlines()[1:]
    out["box_sunhours_day"] = {"source": "docs/daylight.md (sun hours of one day)", "columns": ["sunhours_front"],
                               "values": [[float(x) for x in l.split()] for l in blk]}
    txt = open(os.path.join(ref, "docs", "views.md")).read()
    i = txt.index("views tests/box.obj\n")
    blk = txt[i:].split("```")[0].strip().splitlines()[1:]
    out["box_views"] = {"source": "docs/views.md (tests/box.obj, defaults)",
                        "columns": ["sky_front", "ground_front", "obstruction_front", "distance_front", "distance_min_front"],
                        "values": [[float(x) for x in l.split()] for l in blk]}
    return out


def sky_goldens(ref):
    """Inputs and the reference's own outputs for the GPU sky: sun_noaa on seeded rows; gendaymtx_step on seeded steps
    (sun positions from sun_noaa at Berlin, DNI 0..950, DHI 0..450 W/m2, night and low sun included) at sky densities
    1, 2, 4 and the flag sets run.cpp uses (sky only; sun only; sky visible; both)."""
    d = os.path.join(HERE, "sky")
    shutil.rmtree(d, ignore_errors=True)
    os.makedirs(d)
    exe = os.path.join(REPO, "oracle", "_ref", "ref_sky_golden")
    rng = np.random.default_rng(77)
    n = 3000
    lat = rng.uniform(-60, 70, n)
    lon = rng.uniform(-180, 180, n)
    tz = np.round(lon / 15) + rng.integers(-1, 2, n)
    month = rng.integers(1, 13, n)
    dim = np.array([31, 28, 31, 30, 31, 30, 31, 31, 30, 31, 30, 31])
    leap = rng.integers(0, 2, n)
    day = np.array([rng.integers(1, dim[m - 1] + (1 if (m == 2 and lp) else 0) + 1) for m, lp in zip(month, leap)])
    hour = np.round(rng.uniform(0, 24, n) * 60) / 60
    hour[:40] = np.arange(40) * 0.5 + 0.5   # exact half hours (the 0.01-day rounding's ties)
    sun_in = np.stack([lat, lon, tz, month, day, hour, leap], axis=1).astype(np.float64)
    sun_in.tofile(os.path.join(d, "sun_in.bin"))
    subprocess.check_call([exe, "sun", os.path.join(d, "sun_in.bin"), os.path.join(d, "sun_out.bin"), str(n)])
    cases = []
    for mf, T, flags in [(1, 192, [(0, 1, 0), (1, 0, 0), (0, 1, 1), (1, 1, 0)]), (2, 96, [(0, 1, 0), (1, 0, 1)]), (4, 48, [(0, 1, 0)])]:
        hrs = np.sort(rng.uniform(0, 8760, T))
        month_, day_, h_ = [], [], []
        for x in hrs:
            dd = int(x // 24)
            m = 1
            while dd >= dim[m - 1]:
                dd -= dim[m - 1]
                m += 1
            month_.append(m); day_.append(dd + 1); h_.append(x % 24)
        rows = np.stack([np.full(T, 52.52), np.full(T, 13.41), np.full(T, 1.0), month_, day_, h_, np.zeros(T)], axis=1)
        rows.astype(np.float64).tofile(os.path.join(d, "tmp_in.bin"))
        subprocess.check_call([exe, "sun", os.path.join(d, "tmp_in.bin"), os.path.join(d, "tmp_out.bin"), str(T)])
        sun = np.fromfile(os.path.join(d, "tmp_out.bin"), np.float64).reshape(T, 6)
        jd = np.array([int(sum(dim[:m - 1]) + dy) for m, dy in zip(month_, day_)])
        dni = rng.uniform(0, 950, T) * (rng.random(T) > 0.15)
        dhi = rng.uniform(0, 450, T) * (rng.random(T) > 0.05)
        steps = np.stack([jd, np.radians(sun[:, 0]), np.radians(sun[:, 1]), dni, dhi], axis=1).astype(np.float64)
        name = "mf%d" % mf
        steps.tofile(os.path.join(d, name + "_in.bin"))
        for sun_f, sky_f, vis_f in flags:
            tag = "%s_sun%d_sky%d_vis%d" % (name, sun_f, sky_f, vis_f)
            subprocess.check_call([exe, "sky", os.path.join(d, name + "_in.bin"), os.path.join(d, tag + ".bin"), str(T), str(mf), str(sun_f),
                                   str(sky_f), str(vis_f), "0.2"])
            cases.append({"mf": mf, "T": T, "sun": sun_f, "sky": sky_f, "visible": vis_f, "grefl": 0.2, "in": name + "_in.bin", "out": tag + ".bin"})
    for f in ("tmp_in.bin", "tmp_out.bin"):
        os.remove(os.path.join(d, f))
    json.dump({"sun": {"n": n, "in": "sun_in.bin", "out": "sun_out.bin"}, "sky": cases}, open(os.path.join(d, "index.json"), "w"), indent=1)
    print("sky: %d sun rows, %d sky cases" % (n, len(cases)))


def record(name, ref):
    """One case's run of the reference's dl_run with the boundary recorder on, into tests/golden/<name>/."""
    d = os.path.join(HERE, name)
    shutil.rmtree(d, ignore_errors=True)
    os.makedirs(d)
    env = dict(os.environ, KGB_RECORD=d, KGB_ORACLE_THREADS="8")
    subprocess.check_call([sys.executable, __file__, "--ref", ref, "--case", name], env=env)
    n = sum(1 for _ in open(os.path.join(d, "calls.jsonl")))
    print("%s: %d calls recorded" % (name, n))


def ladybug_goldens(ref):
    """Ladybug mode's sky on the urban weather year at sky densities 1 and 2, from the reference's own functions
    (oracle/ref_sky_golden.cpp, mode ladybug): the steps, the float accumulators, the weights, and the first
    LADYBUG_COLS series columns. tests/golden/ladybug/mf<k>.npz"""
    d = os.path.join(HERE, "ladybug")
    shutil.rmtree(d, ignore_errors=True)
    os.makedirs(d)
    tmp = os.path.join(d, "_tmp")
    os.makedirs(tmp)
    urban_weather(ref, tmp)
    exe = os.path.join(REPO, "oracle", "_ref", "ref_sky_golden")
    for mf in (1, 2):
        raw = os.path.join(tmp, "lb.bin")
        subprocess.check_call([exe, "ladybug", os.path.join(tmp, "urban.epw"), raw, "0", str(mf), "0.2"])
        b = open(raw, "rb").read()
        head = np.frombuffer(b, np.float64, 7)
        T, P, Tup = int(head[0]), int(head[1]), int(head[2])
        at = 56
        steps = np.frombuffer(b, np.float64, 4 * T, at).reshape(T, 4); at += 32 * T
        acc = np.frombuffer(b, np.float32, 4 * P + 6, at); at += 4 * (4 * P + 6)
        lb = np.frombuffer(b, np.float64, 3 * P + 1, at); at += 8 * (3 * P + 1)
        S = np.frombuffer(b, np.float32, P * Tup, at).reshape(P, Tup); at += 4 * P * Tup
        g = np.frombuffer(b, np.float32, Tup, at)
        np.savez_compressed(os.path.join(d, "mf%d.npz" % mf), head=head, steps=steps, acc=acc, lb=lb, S=np.ascontiguousarray(S[:, :LADYBUG_COLS]),
                            g=g[:LADYBUG_COLS].copy(), grefl=0.2)
        print("ladybug mf %d: %d steps, %d patches, %d series columns" % (mf, T, P, Tup))
    shutil.rmtree(tmp, ignore_errors=True)
    for f in ("weather.npy", "cloud_factor.npy"):   # the urban_sky case keeps the weather year
        if os.path.exists(os.path.join(d, f)):
            os.remove(os.path.join(d, f))


def golden_meshes(rng):
    """Seeded meshes for the triangulation and thin-solid goldens: (name, points, counts, indices, slots, centre)."""
    out = []
    # n-gons: star-shaped (concave) rings of 5..60 corners on tilted planes, convex rings, rings with duplicate and
    # collinear corners, a self-touching ring, degenerate faces; mixed with triangles, quads and faces of 0..2 corners
    pts, counts, idx, slots = [], [], [], []
    def add(ring, slot):
        base = len(pts)
        pts.extend(ring)
        counts.append(len(ring))
        idx.extend(range(base, base + len(ring)))
        slots.append(slot)
    for k in range(220):
        kind = rng.integers(0, 7)
        n = int(rng.integers(5, 61))
        ang = np.sort(rng.uniform(0, 2 * np.pi, n))
        rad = rng.uniform(0.3, 1.0, n) if kind in (0, 1) else np.ones(n)
        ring2 = np.stack([np.cos(ang) * rad, np.sin(ang) * rad], 1) * rng.uniform(0.5, 300)
        if kind == 2:   # duplicate and collinear corners
            ring2 = np.concatenate([ring2, ring2[:3]])[: n + 3]
            ring2[2] = ring2[1]
            ring2 = np.insert(ring2, 4, (ring2[3] + ring2[4]) / 2, axis=0)
        if kind == 3:   # clockwise
            ring2 = ring2[::-1]
        ax = rng.normal(size=3); ax /= np.linalg.norm(ax)
        u = np.cross(ax, [0.3, 0.5, 0.8]); u /= np.linalg.norm(u)
        w = np.cross(ax, u)
        o = rng.uniform(-2000, 2000, 3)
        ring = o + ring2[:, :1] * u + ring2[:, 1:2] * w
        if kind == 4:   # slightly warped
            ring = ring + ax * rng.normal(0, 1e-3, (len(ring), 1))
        if kind == 5:   # collinear: no area
            ring = o + np.linspace(0, 1, n)[:, None] * u
        if kind == 6:   # a bow tie (self-touching)
            ring = o + np.array([[0, 0], [2, 2], [2, 0], [1, 1.0001], [0, 2], [-1, 1]])[:, :1] * u + np.array([[0, 0], [2, 2], [2, 0], [1, 1.0001], [0, 2], [-1, 1]])[:, 1:2] * w
        add([tuple(p) for p in ring], int(rng.integers(0, 4)))
        if k % 5 == 0:
            add([tuple(o + [0, 0, 0]), tuple(o + [1, 0, 0]), tuple(o + [0, 1, 0])], 1)
            add([tuple(o + [0, 0, 1]), tuple(o + [1, 0, 1]), tuple(o + [1, 1, 1]), tuple(o + [0, 1, 1])], 2)
        if k % 37 == 0:
            add([], 0)
            add([tuple(o)], 0)
            add([tuple(o), tuple(o + 1)], 3)
    out.append(("ngons", np.array(pts, np.float64), np.array(counts, np.int32), np.array(idx, np.int32), np.array(slots, np.uint16),
                np.array([12.5, -7.25, 3.0])))
    # thin solids (check_mesh.cpp:278-309's shapes): a 20 x 20 x 0.01 m pane box (slot 0), the same box flipped (slot 1),
    # an open box (slot 2), a 3 m cube (slot 3), a double-faced sheet (slot 4), two touching thin boxes (slot 5)
    def box(x0, y0, z0, x1, y1, z1, flip=False):
        c = [(x0, y0, z0), (x1, y0, z0), (x1, y1, z0), (x0, y1, z0), (x0, y0, z1), (x1, y0, z1), (x1, y1, z1), (x0, y1, z1)]
        f = [[0, 3, 2, 1], [4, 5, 6, 7], [0, 1, 5, 4], [1, 2, 6, 5], [2, 3, 7, 6], [3, 0, 4, 7]]
        if flip:
            f = [q[::-1] for q in f]
        return c, f
    pts, counts, idx, slots = [], [], [], []
    def add_box(c, faces, slot, drop=0):
        base = len(pts)
        pts.extend(c)
        for q in faces[: len(faces) - drop]:
            counts.append(4)
            idx.extend(base + i for i in q)
            slots.append(slot)
    add_box(*box(0, 0, 1, 20, 20, 1.01), 0)
    add_box(*box(30, 0, 1, 50, 20, 1.01, flip=True), 1)
    add_box(*box(60, 0, 1, 80, 20, 1.01), 2, drop=1)
    add_box(*box(-1.5, -1.5, 1, 1.5, 1.5, 4), 3)
    sheet = [(0, 0, 10), (2, 0, 10), (2, 2, 10), (0, 2, 10)]
    base = len(pts)
    pts.extend(sheet)
    for q in ([0, 1, 2, 3], [3, 2, 1, 0]):
        counts.append(4); idx.extend(base + i for i in q); slots.append(4)
    add_box(*box(100, 0, 0, 101, 1, 0.01), 5)
    add_box(*box(101, 0, 0, 102, 1, 0.01), 5)
    out.append(("solids", np.array(pts, np.float64), np.array(counts, np.int32), np.array(idx, np.int32), np.array(slots, np.uint16),
                np.array([1e5, -3e5, 50.0])))
    return out


def mesh_goldens(ref):
    """The reference's own triangulate_into and thin_solid (oracle/ref_sky_golden.cpp, mode mesh) on seeded meshes: the
    n-gons through the engine's restatement of earcut (the reference's earcut stand-in here). tests/golden/mesh/<name>.npz"""
    d = os.path.join(HERE, "mesh")
    shutil.rmtree(d, ignore_errors=True)
    os.makedirs(d)
    exe = os.path.join(REPO, "oracle", "_ref", "ref_sky_golden")
    for name, P, C, I, S, c in golden_meshes(np.random.default_rng(31)):
        raw_in, raw_out = os.path.join(d, "in.bin"), os.path.join(d, "out.bin")
        with open(raw_in, "wb") as f:
            f.write(np.array([len(P), len(C), len(I)], np.uint64).tobytes() + c.astype(np.float64).tobytes() + P.tobytes() + C.tobytes() +
                    I.tobytes() + S.tobytes())
        subprocess.check_call([exe, "mesh", raw_in, raw_out, "0"])
        b = open(raw_out, "rb").read()
        made, skipped, nSlots = [int(x) for x in np.frombuffer(b, np.int64, 3)]
        at = 24
        v = np.frombuffer(b, np.float32, 3 * len(P), at).reshape(-1, 3); at += 12 * len(P)
        tri = np.frombuffer(b, np.uint32, 3 * made, at).reshape(-1, 3); at += 12 * made
        slot = np.frombuffer(b, np.uint32, made, at); at += 4 * made
        thin = np.frombuffer(b, np.uint32, nSlots, at)
        np.savez_compressed(os.path.join(d, name + ".npz"), points=P, counts=C, indices=I, slots=S, c=c, v=v, tri=tri, slot=slot, skipped=skipped,
                            thin=thin)
        os.remove(raw_in)
        os.remove(raw_out)
        print("mesh %s: %d faces, %d triangles, %d skipped, thin %s" % (name, len(C), made, skipped, thin.tolist()))


def dmesh_image(points, counts, indices, slots=None, flags=None, magic=b"DLM1", n=None):
    """A .dmesh image (the reference's layout, src/daylight.h:129-136); n overrides the header's three counts."""
    P = np.ascontiguousarray(points, np.float64).reshape(-1, 3)
    C = np.ascontiguousarray(counts, np.int32)
    I = np.ascontiguousarray(indices, np.int32)
    fl = (1 if slots is not None else 0) if flags is None else flags
    nP, nF, nI = n if n is not None else (len(P), len(C), len(I))
    head = magic + np.array([fl], np.uint32).tobytes() + np.array([nP, nF, nI], np.uint64).tobytes()
    body = P.tobytes() + C.tobytes() + I.tobytes() + (np.ascontiguousarray(slots, np.uint16).tobytes() if slots is not None else b"")
    return head + body


def dmesh_cases(rng):
    """Seeded images for the reader's rules: valid meshes (with and without the slot block, trailing bytes, an empty
    mesh), and one image per failure of the header and of the arrays, some failing two rules at once (the first in the
    reference's order must be reported)."""
    P = rng.uniform(-50, 80, (40, 3)).round(3)
    C = np.array([3, 4, 5, 3, 6, 4, 3, 7], np.int32)
    I = rng.integers(0, 40, int(C.sum())).astype(np.int32)
    S = rng.integers(0, 5, len(C)).astype(np.uint16)
    good = dmesh_image(P, C, I, S)
    cases = [("slots", good), ("no_slots", dmesh_image(P, C, I)), ("trailing_bytes", good + b"\x07" * 13),
             ("empty", dmesh_image(P[:3], [], [])), ("empty_with_indices", dmesh_image(P[:3], [], [0, 1, 2])),
             ("short_header", good[:20]), ("nothing", b""), ("bad_magic", dmesh_image(P, C, I, magic=b"DLM2")),
             ("bad_flags", dmesh_image(P, C, I, flags=2)), ("bad_flags_high", dmesh_image(P, C, I, S, flags=0x80000001)),
             ("truncated_arrays", dmesh_image(P, C, I)[:-10]), ("truncated_slot_block", good[:-1]),
             ("huge_points", dmesh_image(P, C, I, n=(1 << 62, len(C), len(I)))),
             ("sum_overflow", dmesh_image(P, C, I, n=(len(P), (1 << 61), len(I))))]
    c2 = C.copy(); c2[3] = 2
    cases.append(("face_of_two", dmesh_image(P, c2, I[:-1])))
    c3 = C.copy(); c3[1] = -4
    cases.append(("negative_count", dmesh_image(P, c3, I)))
    cases.append(("sum_mismatch", dmesh_image(P, C, np.concatenate([I, [0]]))))
    i2 = I.copy(); i2[7] = 40
    cases.append(("index_past_points", dmesh_image(P, C, i2)))
    i3 = I.copy(); i3[0] = -1
    cases.append(("negative_index", dmesh_image(P, C, i3, S)))
    cases.append(("face_of_two_and_bad_index", dmesh_image(P, c2, i2[:-1])))
    cases.append(("sum_mismatch_and_bad_index", dmesh_image(P, C, np.concatenate([i2, [0]]))))
    # a grid of quads with a slot per face (the ingest benchmark's mesh, small)
    g = 24
    xs, ys = np.meshgrid(np.arange(g + 1, dtype=np.float64), np.arange(g + 1, dtype=np.float64), indexing="ij")
    gp = np.stack([xs.ravel() * 1.5 + 1e5, ys.ravel() * 1.5 - 3e5, np.sin(xs.ravel()) * 0.1], 1)
    q = np.arange(g * (g + 1)).reshape(g, g + 1)[:, :g].ravel()
    gi = np.stack([q, q + g + 1, q + g + 2, q + 1], 1).astype(np.int32).ravel()
    cases.append(("quad_grid", dmesh_image(gp, np.full(g * g, 4, np.int32), gi, (np.arange(g * g) % 3).astype(np.uint16))))
    return cases


def dmesh_goldens(ref):
    """The reference's own read_dmesh (oracle/ref_sky_golden.cpp, mode dmesh) on seeded images:
    tests/golden/dmesh/cases.npz holds each image and the reference's answer (ok, message, the arrays it read)."""
    d = os.path.join(HERE, "dmesh")
    shutil.rmtree(d, ignore_errors=True)
    os.makedirs(d)
    exe = os.path.join(REPO, "oracle", "_ref", "ref_sky_golden")
    out = {}
    names = []
    for name, img in dmesh_cases(np.random.default_rng(41)):
        raw_in, raw_out = os.path.join(d, "in.bin"), os.path.join(d, "out.bin")
        open(raw_in, "wb").write(img)
        subprocess.check_call([exe, "dmesh", raw_in, raw_out, "0"])
        b = open(raw_out, "rb").read()
        ok, nm, ln = [int(x) for x in np.frombuffer(b, np.uint64, 3)]
        msg = b[24:24 + ln].decode()
        at = 24 + ln
        out[name + "/image"] = np.frombuffer(img, np.uint8)
        out[name + "/answer"] = np.array([ok, nm], np.int64)
        out[name + "/message"] = np.frombuffer(msg.encode(), np.uint8)
        for k in range(nm):
            nP, nF, nI, nS = [int(x) for x in np.frombuffer(b, np.uint64, 4, at)]
            at += 32
            for key, dt, cnt in (("points", np.float64, 3 * nP), ("counts", np.int32, nF), ("indices", np.int32, nI), ("slot", np.uint16, nS)):
                out[name + "/" + key] = np.frombuffer(b, dt, cnt, at).copy()
                at += np.dtype(dt).itemsize * cnt
        names.append(name)
        os.remove(raw_in)
        os.remove(raw_out)
        print("dmesh %s: %s" % (name, "ok, %d mesh" % nm if ok else msg))
    out["names"] = np.frombuffer("\n".join(names).encode(), np.uint8)
    np.savez_compressed(os.path.join(d, "cases.npz"), **out)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("KITSIM_REFERENCE") or os.path.join(os.path.dirname(REPO), "reference"))
    ap.add_argument("--case")
    ap.add_argument("--only", help="comma-separated parts to regenerate: recorded case names, sky, ladybug, mesh, dmesh")
    a = ap.parse_args()
    if a.case:
        run_case(a.case, a.ref)
        return
    if a.only:
        subprocess.check_call(["make", "-s", "-j8", "-C", os.path.join(REPO, "oracle"), "ref", "REF=" + a.ref])
        for part in a.only.split(","):
            if part == "sky":
                sky_goldens(a.ref)
            elif part == "ladybug":
                ladybug_goldens(a.ref)
            elif part == "mesh":
                mesh_goldens(a.ref)
            elif part == "dmesh":
                dmesh_goldens(a.ref)
            else:
                record(part, a.ref)
        return
    subprocess.check_call(["make", "-s", "-j8", "-C", os.path.join(REPO, "oracle"), "ref", "REF=" + a.ref])
    for name in CASES:
        record(name, a.ref)
    sky_goldens(a.ref)
    ladybug_goldens(a.ref)
    mesh_goldens(a.ref)
    dmesh_goldens(a.ref)
    pub = published(a.ref)
    with open(os.path.join(HERE, "published.json"), "w") as f:
        json.dump(pub, f, indent=1)
    for name, p in pub.items():
        got = np.load(os.path.join(HERE, name, "result.npy"))
        cols = json.load(open(os.path.join(HERE, name, "manifest.json")))["columns"]
        want = np.array(p["values"])
        for k, c in enumerate(p["columns"]):
            g = got[:, cols.index(c)]
            w = want[:, k]
            rel = np.abs(g - w) / np.maximum(np.abs(w), 1e-9)
            print("%s %s: max rel diff vs published %.3g (max abs %.3g)" % (name, c, rel.max(), np.abs(g - w).max()))


if __name__ == "__main__":
    main()
