"""ctypes binding of the engine's C ABI (include/kitsim_gb300.h), with numpy arrays in and out.

`Engine` mirrors the reference's GPU contract (kit-sim_daylight src/internal.h:125-220: gpu_build, gpu_set_scene,
gpu_trace, gpu_reduce, gpu_series, gpu_bounce, gpu_view, gpu_reduce_view, ...) call for call: the same arguments, the
same device layouts (bits word-major [nWords x nc], bytes / classes / distances direction-major [nDir x nc]), the same
errors (a failing call raises KgbError with the engine's message, e.g. "cancelled").
"""
import ctypes
from ctypes import POINTER, c_char_p, c_double, c_float, c_int, c_int32, c_size_t, c_uint32, c_uint64, c_void_p

import numpy as np


class KgbError(RuntimeError):
    pass


class Slot(ctypes.Structure):
    _fields_ = [("rho", c_float), ("tau", c_float), ("tn", c_float), ("flags", c_uint32)]


class SceneHandle(ctypes.Structure):
    _fields_ = [("handle", c_void_p), ("bytes", c_uint64)]


class Stats(ctypes.Structure):
    _fields_ = [("buildMs", c_double), ("traceMs", c_double), ("bounceMs", c_double), ("rays", c_uint64), ("gasBytes", c_uint64),
                ("launches", c_uint64), ("paths", c_uint64), ("bounceLaunches", c_uint64), ("buildTempBytes", c_uint64),
                ("buildOutputBytes", c_uint64), ("seriesMs", c_double), ("seriesOutputs", c_uint64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


CANCEL_FN = ctypes.CFUNCTYPE(c_int, c_void_p)


class SeriesIn(ctypes.Structure):
    _fields_ = [("nSky", c_uint32), ("row", POINTER(c_int32)), ("wsky", POINTER(c_float)), ("S", POINTER(c_float)), ("P", c_int32),
                ("T", c_int32), ("g", POINTER(c_float)), ("G", POINTER(c_float)), ("sun0", c_uint32), ("nSun", c_uint32),
                ("sunStep", POINTER(c_int32)), ("sunVec", POINTER(c_float)), ("sunW", POINTER(c_float)), ("Sdc", POINTER(c_float))]


class SkyStep(ctypes.Structure):
    _fields_ = [("jd", c_int32), ("pad", c_int32), ("alt", c_double), ("azi", c_double), ("dni", c_double), ("dhi", c_double)]


class BounceIn(ctypes.Structure):
    _fields_ = [("N", c_uint32), ("M", c_uint32), ("mf", c_int32), ("north", c_double), ("cancel", CANCEL_FN), ("cancelCtx", c_void_p)]


class ViewIn(ctypes.Structure):
    _fields_ = [("nAz", c_uint32), ("nEl", c_uint32), ("az0", c_float), ("dAz", c_float), ("rowSin", POINTER(c_float)),
                ("world", c_int32), ("cull", c_int32), ("jitter", c_int32), ("back", c_int32), ("vground", c_int32), ("nS", c_uint32),
                ("groundZ", c_float), ("north", c_double), ("cancel", CANCEL_FN), ("cancelCtx", c_void_p)]


class DaylightRequest(ctypes.Structure):
    _fields_ = [("scene", c_int32), ("nSensors", c_uint32), ("nDir", c_uint32), ("nQ", c_uint32), ("P", c_void_p), ("N", c_void_p),
                ("D", c_void_p), ("W", c_void_p), ("useCosMask", c_uint32), ("rayFlags", c_uint32), ("out", c_void_p)]


class SeriesRequest(ctypes.Structure):
    _fields_ = [("in", SeriesIn), ("gQ", c_uint32), ("E", c_void_p)]   # "in": the C field name


class ViewsRequest(ctypes.Structure):
    _fields_ = [("scene", c_int32), ("nSensors", c_uint32), ("P", c_void_p), ("N", c_void_p), ("label", c_void_p), ("view", ViewIn),
                ("rayFlags", c_uint32), ("wRow", c_void_p), ("nClass", c_uint32), ("farDist", c_double), ("reach", c_void_p),
                ("nReach", c_uint32), ("glazing", c_int32), ("isoDim", c_uint32), ("out", c_void_p)]


class MeshInfo(ctypes.Structure):
    _fields_ = [("id", c_uint32), ("slots", c_uint32), ("nPoints", c_uint64), ("nFaces", c_uint64), ("nIndices", c_uint64),
                ("hasSlots", c_uint32), ("maxCorners", c_uint32), ("triCap", c_uint64), ("lo", c_double * 3), ("hi", c_double * 3)]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_}
        d["lo"], d["hi"] = list(self.lo), list(self.hi)
        return d


NO_MESH = 0xFFFFFFFF
LIMIT_WITHHOLD_FILLS = 1
RAY_DISABLE_ANYHIT, RAY_TERMINATE_ON_FIRST_HIT, RAY_CULL_BACK_FACING = 1, 4, 16
SLOT_GLASS, SLOT_THIN, SLOT_INWARD, SLOT_TWIN = 1, 2, 4, 8
LABEL_PASS, MAX_PANES, VIEW_GLAZED = 255, 16, 0x80

# every exported symbol of include/kitsim_gb300.h: (name, restype, argtypes)
_E = c_void_p
SIGNATURES = [
    ("kgb_version", c_int32, []),
    ("kgb_last_error", c_char_p, []),
    ("kgb_init", _E, []),
    ("kgb_destroy", None, [_E]),
    ("kgb_build", c_int, [_E, c_void_p, c_size_t, c_void_p, c_size_t, c_void_p, c_void_p, c_size_t, c_int]),
    ("kgb_build_bytes", c_uint64, [_E, c_size_t, c_size_t, c_int]),
    ("kgb_trim", None, [_E, c_int]),
    ("kgb_set_slots", c_int, [_E, c_void_p, c_size_t]),
    ("kgb_detach", SceneHandle, [_E]),
    ("kgb_attach", None, [_E, SceneHandle]),
    ("kgb_free_scene", None, [POINTER(SceneHandle)]),
    ("kgb_free_bytes", c_uint64, []),
    ("kgb_set_scene", c_int, [_E, c_void_p, c_void_p, c_size_t, c_void_p, c_size_t]),
    ("kgb_set_labels", c_int, [_E, c_void_p, c_size_t]),
    ("kgb_trace", c_int, [_E, c_size_t, c_size_t, c_uint32]),
    ("kgb_reduce", c_int, [_E, c_size_t, c_void_p, c_int, c_void_p]),
    ("kgb_series", c_int, [_E, c_size_t, POINTER(SeriesIn), c_void_p]),
    ("kgb_bounce", c_int, [_E, c_size_t, c_size_t, c_uint32, POINTER(BounceIn)]),
    ("kgb_reduce_dc", c_int, [_E, c_size_t, c_void_p, c_void_p]),
    ("kgb_download_dc", c_int, [_E, c_size_t, c_void_p, c_size_t]),
    ("kgb_download_bits", c_int, [_E, c_size_t, c_void_p, c_size_t]),
    ("kgb_download_bytes", c_int, [_E, c_size_t, c_void_p, c_size_t]),
    ("kgb_download_bits_rows", c_int, [_E, c_size_t, c_void_p, c_size_t]),
    ("kgb_series_file", c_int, [_E, c_size_t, c_void_p, c_int, c_uint64]),
    ("kgb_download_bytes_rows", c_int, [_E, c_size_t, c_void_p, c_size_t]),
    ("kgb_view", c_int, [_E, c_size_t, c_size_t, c_uint32, POINTER(ViewIn), POINTER(c_size_t)]),
    ("kgb_reduce_view", c_int, [_E, c_size_t, c_void_p, c_size_t, c_uint32, c_double, c_void_p, c_size_t, c_int, c_uint32, c_void_p]),
    ("kgb_download_view", c_int, [_E, c_size_t, c_void_p, c_void_p, c_size_t]),
    ("kgb_get_stats", Stats, [_E]),
    ("kgb_ray_flags", c_uint32, [c_int, c_int]),
    ("kgb_bounce_flags", c_uint32, [c_int]),
    ("kgb_dims", None, [_E, POINTER(c_uint64)]),
    ("kgb_set_stream", c_int, [_E, c_void_p]),
    ("kgb_server_create", c_void_p, [c_uint64]),
    ("kgb_server_destroy", None, [c_void_p]),
    ("kgb_server_add_scene", c_int, [c_void_p, c_void_p, c_size_t, c_void_p, c_size_t, POINTER(c_int32)]),
    ("kgb_server_autotune", c_int, [c_void_p]),
    ("kgb_server_set_tuning", c_int, [c_void_p, c_uint32, c_uint64, c_uint64]),
    ("kgb_server_set_priority", c_int, [c_void_p, c_double, c_double]),
    ("kgb_server_tuning", None, [c_void_p, POINTER(c_uint64)]),
    ("kgb_server_submit", c_int, [c_void_p, POINTER(DaylightRequest), POINTER(c_uint64)]),
    ("kgb_server_submit_views", c_int, [c_void_p, POINTER(ViewsRequest), POINTER(c_uint64)]),
    ("kgb_server_submit_series", c_int, [c_void_p, POINTER(DaylightRequest), POINTER(SeriesRequest), POINTER(c_uint64)]),
    ("kgb_server_wait", c_int, [c_void_p, c_uint64, c_double]),
    ("kgb_server_stats", None, [c_void_p, POINTER(c_double)]),
    ("kgb_server_timing", None, [c_void_p, POINTER(c_double)]),
    ("kgb_sky", c_int, [_E, c_int32, c_void_p, c_size_t, c_double, c_int32, c_int32, c_int32, c_void_p]),
    ("kgb_sun_noaa", c_int, [_E, c_void_p, c_size_t, c_void_p]),
    ("kgb_triangulate", c_int, [_E, c_void_p, c_size_t, c_void_p, c_size_t, c_void_p, c_void_p, c_void_p, c_uint32, c_uint32, c_void_p, c_void_p,
                                c_void_p, POINTER(c_size_t), POINTER(c_int32)]),
    ("kgb_thin_solids", c_int, [_E, c_void_p, c_size_t, c_void_p, c_size_t, c_void_p, c_void_p, c_uint32, c_void_p, c_void_p]),
    ("kgb_sky_ladybug", c_int, [_E, c_int32, c_void_p, c_size_t, c_double, c_double, c_double, c_double, c_double, c_void_p, c_void_p, c_void_p,
                                c_void_p]),
    ("kgb_set_builder", c_int, [_E, c_int]),
    ("kgb_set_series_form", c_int, [_E, c_int]),
    ("kgb_trace_counters", c_int, [_E, c_size_t, c_size_t, c_uint32, POINTER(c_uint64)]),
    ("kgb_set_limits", c_int, [_E, c_uint32, c_uint64, c_uint64, c_uint32]),
    ("kgb_mesh_read", c_int, [_E, c_void_p, c_size_t, c_char_p, POINTER(MeshInfo)]),
    ("kgb_mesh_file", c_int, [_E, c_char_p, POINTER(MeshInfo)]),
    ("kgb_mesh_download", c_int, [_E, c_uint32, c_void_p, c_void_p, c_void_p, c_void_p]),
    ("kgb_mesh_free", c_int, [_E, c_uint32]),
    ("kgb_mesh_thin_solids", c_int, [_E, c_uint32, c_void_p, c_void_p]),
    ("kgb_build_meshes", c_int, [_E, c_void_p, c_size_t, c_void_p, c_void_p, c_void_p, c_size_t, c_int, c_void_p, POINTER(c_int32)]),
]


class Lib:
    """A library that exports the engine's C ABI (the engine itself, or a restatement with the same symbols)."""

    def __init__(self, path):
        self.path = path
        self.dll = ctypes.CDLL(path)
        for name, res, args in SIGNATURES:
            f = getattr(self.dll, name)
            f.restype = res
            f.argtypes = args

    def err(self):
        return (self.dll.kgb_last_error() or b"").decode()

    def ray_flags(self, cull=False, translucent=False):
        return self.dll.kgb_ray_flags(int(cull), int(translucent))

    def bounce_flags(self, cull=False):
        return self.dll.kgb_bounce_flags(int(cull))


def _p(a):
    return a.ctypes.data_as(c_void_p) if a is not None and a.size else None


def _f32(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float32)
    return a if shape is None else a.reshape(shape)


def _typed(a, ctype):
    return a.ctypes.data_as(POINTER(ctype)) if a is not None else None


class Engine:
    """One engine (one device state) behind a Lib: the reference's Gpu."""

    def __init__(self, lib):
        self.lib = lib
        self.d = lib.dll
        self.h = self.d.kgb_init()
        if not self.h:
            raise KgbError(lib.err())
        self._keep = []

    def close(self):
        if self.h:
            self.d.kgb_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ok(self, r):
        if not r:
            raise KgbError(self.lib.err())

    # --- scene
    def build(self, v, tri, slot=None, slots=None, per_slot=False):
        v = _f32(v, (-1, 3))
        tri = np.ascontiguousarray(tri, dtype=np.uint32).reshape(-1, 3)
        slot = None if slot is None else np.ascontiguousarray(slot, dtype=np.uint32)
        sl = slots_array(slots if slots is not None else [Slot(0.2, 0, 0, 0)])
        self._ok(self.d.kgb_build(self.h, _p(v), len(v), _p(tri), len(tri), _p(slot), ctypes.cast(sl, c_void_p), len(sl), int(per_slot)))

    def build_bytes(self, nv, nt, slotted=False):
        return self.d.kgb_build_bytes(self.h, nv, nt, int(slotted))

    def set_slots(self, slots):
        sl = slots_array(slots)
        self._ok(self.d.kgb_set_slots(self.h, ctypes.cast(sl, c_void_p), len(sl)))

    def trim(self, sensors=False):
        self.d.kgb_trim(self.h, int(sensors))

    def detach(self):
        return self.d.kgb_detach(self.h)

    def attach(self, s):
        self.d.kgb_attach(self.h, s)

    def free_scene(self, s):
        self.d.kgb_free_scene(ctypes.byref(s))

    def set_scene(self, P, N, D):
        P, N, D = _f32(P, (-1, 3)), _f32(N, (-1, 3)), _f32(D, (-1, 3))
        self._ok(self.d.kgb_set_scene(self.h, _p(P), _p(N), len(P), _p(D), len(D)))

    def set_labels(self, label):
        label = np.ascontiguousarray(label, dtype=np.uint8)
        self._ok(self.d.kgb_set_labels(self.h, _p(label), label.size))

    def dims(self):
        out = (c_uint64 * 6)()
        self.d.kgb_dims(self.h, out)
        return dict(nSensors=out[0], nDir=out[1], nWords=out[2], nBins=out[3], K=out[4], bytes=bool(out[5]))

    def stats(self):
        return self.d.kgb_get_stats(self.h).as_dict()

    def set_stream(self, stream_handle):
        """Run on this cudaStream_t (an int handle, e.g. torch.cuda.Stream().cuda_stream); None: the engine's own."""
        self._ok(self.d.kgb_set_stream(self.h, c_void_p(stream_handle) if stream_handle else None))

    def sky(self, mf, steps, grefl=0.2, sun=False, sky=True, visible=False):
        """steps: [T x 5] (jd, alt, azi, dni, dhi). Returns [T x (P + 1) x 3] floats (gendaymtx_step rows)."""
        steps = np.asarray(steps, np.float64).reshape(-1, 5)
        st = np.zeros(len(steps), dtype=[("jd", "<i4"), ("pad", "<i4"), ("alt", "<f8"), ("azi", "<f8"), ("dni", "<f8"), ("dhi", "<f8")])
        st["jd"] = steps[:, 0].astype(np.int32)
        st["alt"], st["azi"], st["dni"], st["dhi"] = steps[:, 1], steps[:, 2], steps[:, 3], steps[:, 4]
        P = 144 * mf * mf + 1
        out = np.zeros((len(steps), P + 1, 3), np.float32)
        self._ok(self.d.kgb_sky(self.h, mf, st.ctypes.data_as(c_void_p), len(st), grefl, int(sun), int(sky), int(visible), _p(out)))
        return out

    def triangulate(self, points, counts, indices, face_slot=None, c=(0.0, 0.0, 0.0), base=0, slot_base=0):
        """One mesh's faces as triangles (the reference's triangulate_into): (v [nPoints x 3] float32, tri [made x 3],
        slot [made], skipped faces)."""
        points = np.ascontiguousarray(points, np.float64).reshape(-1, 3)
        counts = np.ascontiguousarray(counts, np.int32)
        indices = np.ascontiguousarray(indices, np.int32)
        fs = None if face_slot is None else np.ascontiguousarray(face_slot, np.uint32)
        cap = int(np.maximum(counts.astype(np.int64) - 2, 0).sum())
        v = np.zeros((len(points), 3), np.float32)
        tri = np.zeros((max(cap, 1), 3), np.uint32)
        slot = np.zeros(max(cap, 1), np.uint32)
        cc = np.ascontiguousarray(c, np.float64)
        made, skipped = c_size_t(0), c_int32(0)
        self._ok(self.d.kgb_triangulate(self.h, _p(points), len(points), _p(counts), len(counts), _p(indices), _p(fs), _p(cc), base, slot_base,
                                        _p(v), _p(tri), _p(slot), ctypes.byref(made), ctypes.byref(skipped)))
        return v, tri[:made.value], slot[:made.value], skipped.value

    def thin_solids(self, points, counts, indices, face_slot=None, n_slots=1, c=(0.0, 0.0, 0.0)):
        """Per slot: KGB_SLOT_THIN (| TWIN or INWARD) when its faces form a closed thin solid, else 0 (the reference's
        thin_solid for every slot)."""
        points = np.ascontiguousarray(points, np.float64).reshape(-1, 3)
        counts = np.ascontiguousarray(counts, np.int32)
        indices = np.ascontiguousarray(indices, np.int32)
        fs = None if face_slot is None else np.ascontiguousarray(face_slot, np.uint32)
        flags = np.zeros(n_slots, np.uint32)
        cc = np.ascontiguousarray(c, np.float64)
        self._ok(self.d.kgb_thin_solids(self.h, _p(points), len(points), _p(counts), len(counts), _p(indices), _p(fs), n_slots, _p(cc), _p(flags)))
        return flags

    # --- meshes read to the device
    def mesh_read(self, image, name="mesh"):
        """A .dmesh image (bytes) read to the device (the reference's read_dmesh of memory): its MeshInfo (id NO_MESH
        for an image without faces)."""
        buf = np.frombuffer(bytes(image), np.uint8) if not isinstance(image, np.ndarray) else np.ascontiguousarray(image, np.uint8)
        info = MeshInfo()
        self._ok(self.d.kgb_mesh_read(self.h, _p(buf), buf.size, name.encode(), ctypes.byref(info)))
        return info

    def mesh_file(self, path):
        """A .dmesh file read to the device (the reference's read_dmesh of a path): its MeshInfo."""
        info = MeshInfo()
        self._ok(self.d.kgb_mesh_file(self.h, str(path).encode(), ctypes.byref(info)))
        return info

    def mesh_download(self, info):
        """A kept mesh's arrays: (points [nPoints x 3], counts, indices, slot or None)."""
        P = np.zeros((info.nPoints, 3), np.float64)
        C = np.zeros(info.nFaces, np.int32)
        I = np.zeros(info.nIndices, np.int32)
        S = np.zeros(info.nFaces, np.uint16) if info.hasSlots else None
        self._ok(self.d.kgb_mesh_download(self.h, info.id, _p(P), _p(C), _p(I), _p(S)))
        return P, C, I, S

    def mesh_free(self, mesh_id):
        self._ok(self.d.kgb_mesh_free(self.h, mesh_id))

    def mesh_thin_solids(self, info, c=(0.0, 0.0, 0.0)):
        flags = np.zeros(info.slots, np.uint32)
        cc = np.ascontiguousarray(c, np.float64)
        self._ok(self.d.kgb_mesh_thin_solids(self.h, info.id, _p(cc), _p(flags)))
        return flags

    def build_meshes(self, ids, c, blocks=None, slots=None, per_slot=False):
        """The scene from kept meshes (the reference's scene assembly + gpu_build): (made per mesh, skipped faces)."""
        ids = np.ascontiguousarray(ids, np.uint32)
        bl = None if blocks is None else np.ascontiguousarray(blocks, np.uint8)
        sl = slots_array(slots if slots is not None else [Slot(0.2, 0, 0, 0)])
        cc = np.ascontiguousarray(c, np.float64)
        made = np.zeros(len(ids), np.uint64)
        skipped = c_int32(0)
        self._ok(self.d.kgb_build_meshes(self.h, _p(ids), len(ids), _p(bl), _p(cc), ctypes.cast(sl, c_void_p), len(sl), int(per_slot), _p(made),
                                         ctypes.byref(skipped)))
        return made, skipped.value

    def sky_ladybug(self, mf, steps, lat, lon, tz, grefl=0.2, duration_hours=None, series=False):
        """Ladybug mode's sky: steps [T x 4] (jd, hour, dni, dhi). Returns (lb [3P + 1] doubles, acc [4P + 6] floats) and,
        with series, also (S [P x Tup], g [Tup]) of the steps with DNI + DHI > 1e-4."""
        steps = np.ascontiguousarray(steps, np.float64).reshape(-1, 4)
        T = len(steps)
        P = 144 * mf * mf + 1
        dur = float(T) if duration_hours is None else float(duration_hours)
        lb = np.zeros(3 * P + 1, np.float64)
        acc = np.zeros(4 * P + 6, np.float32)
        Tup = int(np.sum(steps[:, 2].astype(np.float32) + steps[:, 3].astype(np.float32) > 1e-4))
        S = np.zeros((P, Tup), np.float32) if series else None
        g = np.zeros(Tup, np.float32) if series else None
        self._ok(self.d.kgb_sky_ladybug(self.h, mf, _p(steps), T, lat, lon, tz, grefl, dur, _p(lb), _p(acc), _p(S) if series else None,
                                        _p(g) if series else None))
        return (lb, acc, S, g) if series else (lb, acc)

    def sun_noaa(self, rows):
        """rows: [T x 7] (lat, lon, tz, month, day, hour, leap). Returns [T x 6] (alt, azi, up, x, y, z)."""
        rows = np.ascontiguousarray(rows, np.float64).reshape(-1, 7)
        out = np.zeros((len(rows), 6), np.float64)
        self._ok(self.d.kgb_sun_noaa(self.h, _p(rows), len(rows), _p(out)))
        return out

    def set_builder(self, which):
        """1: device LBVH with treelet restructuring (default); 0: host binned-SAH tree. Applies to the following build() calls."""
        self._ok(self.d.kgb_set_builder(self.h, int(which)))

    def set_series_form(self, form):
        """0: split-BF16 on the tensor cores (default); 1: the plain FP32 form."""
        self._ok(self.d.kgb_set_series_form(self.h, form))

    def set_limits(self, node_limit=0, bounce_limit_ns=0, series_wait_ns=0, withhold_fills=False):
        """Lowers the traversal's node limit (the walks see only the BVH's first node_limit nodes), the bounce step's
        time limit and the series pipeline's wait limit; 0 restores a default. withhold_fills: the series pipeline's
        producer issues no fills, so that its waits run out (the test of that path)."""
        self._ok(self.d.kgb_set_limits(self.h, int(node_limit), int(bounce_limit_ns), int(series_wait_ns), LIMIT_WITHHOLD_FILLS if withhold_fills else 0))

    def trace_counters(self, i0, nc, flags):
        """The instrumented trace: dict(nodes, tris, rays, bvh_bytes) for the roofline (results as trace())."""
        out = (c_uint64 * 4)()
        self._ok(self.d.kgb_trace_counters(self.h, i0, nc, flags, out))
        return dict(nodes=out[0], tris=out[1], rays=out[2], bvh_bytes=out[3])

    # --- daylight
    def trace(self, i0, nc, flags):
        self._ok(self.d.kgb_trace(self.h, i0, nc, flags))

    def reduce(self, nc, W, use_cos=True):
        W = _f32(W)
        out = np.zeros(nc, np.float64)
        self._ok(self.d.kgb_reduce(self.h, nc, _p(W), int(use_cos), _p(out)))
        return out

    def download_bits(self, nc):
        n = self.dims()["nWords"] * nc
        out = np.zeros(n, np.uint32)
        self._ok(self.d.kgb_download_bits(self.h, nc, _p(out), n))
        return out.reshape(-1, nc) if nc else out

    def download_bytes(self, nc):
        n = self.dims()["nDir"] * nc
        out = np.zeros(n, np.uint8)
        self._ok(self.d.kgb_download_bytes(self.h, nc, _p(out), n))
        return out.reshape(-1, nc) if nc else out

    def download_bits_rows(self, nc):
        """The last trace's bits as [nc x nWords] rows (transposed on the device)."""
        nw = self.dims()["nWords"]
        out = np.zeros(nw * nc, np.uint32)
        self._ok(self.d.kgb_download_bits_rows(self.h, nc, _p(out), nw * nc))
        return out.reshape(nc, nw)

    def download_bytes_rows(self, nc):
        """The last trace's bytes as [nc x nDir] rows (transposed on the device)."""
        nd = self.dims()["nDir"]
        out = np.zeros(nd * nc, np.uint8)
        self._ok(self.d.kgb_download_bytes_rows(self.h, nc, _p(out), nd * nc))
        return out.reshape(nc, nd)

    def series(self, nc, nSky, row, wsky, S, g, G, sun0, sunStep, sunVec, sunW, Sdc=None, out=None):
        """E [nc x T] (float32); out: a C-contiguous float32 buffer of that shape to write into (the reference's caller
        reuses one E vector across chunks, run.cpp:683-686), else a new array."""
        row = np.ascontiguousarray(row, dtype=np.int32)
        wsky, S, g, G = _f32(wsky), _f32(S), _f32(g), _f32(G)
        P, T = S.shape
        sunStep = np.ascontiguousarray(sunStep, dtype=np.int32)
        sunVec, sunW = _f32(sunVec, (-1, 3)), _f32(sunW)
        Sdc = None if Sdc is None else _f32(Sdc)
        s = SeriesIn(nSky, _typed(row, c_int32), _typed(wsky, c_float), _typed(S, c_float), P, T, _typed(g, c_float), _typed(G, c_float),
                     sun0, len(sunStep), _typed(sunStep, c_int32), _typed(sunVec, c_float), _typed(sunW, c_float),
                     _typed(Sdc, c_float) if Sdc is not None else None)
        if out is None:
            E = np.zeros((nc, T), np.float32)
        else:
            E = out
            if E.dtype != np.float32 or E.shape != (nc, T) or not E.flags.c_contiguous:
                raise ValueError("series: out must be a C-contiguous float32 [nc x T] array")
        self._ok(self.d.kgb_series(self.h, nc, ctypes.byref(s), _p(E)))
        return E

    def series_file(self, nc, fd, offset, nSky, row, wsky, S, g, G, sun0, sunStep, sunVec, sunW, Sdc=None):
        """The series' rows [nc x T] float32 written to the open file descriptor fd at byte offset."""
        row = np.ascontiguousarray(row, dtype=np.int32)
        wsky, S, g, G = _f32(wsky), _f32(S), _f32(g), _f32(G)
        P, T = S.shape
        sunStep = np.ascontiguousarray(sunStep, dtype=np.int32)
        sunVec, sunW = _f32(sunVec, (-1, 3)), _f32(sunW)
        Sdc = None if Sdc is None else _f32(Sdc)
        s = SeriesIn(nSky, _typed(row, c_int32), _typed(wsky, c_float), _typed(S, c_float), P, T, _typed(g, c_float), _typed(G, c_float),
                     sun0, len(sunStep), _typed(sunStep, c_int32), _typed(sunVec, c_float), _typed(sunW, c_float),
                     _typed(Sdc, c_float) if Sdc is not None else None)
        self._ok(self.d.kgb_series_file(self.h, nc, ctypes.byref(s), int(fd), int(offset)))

    def bounce(self, i0, nc, flags, N=1, M=1024, mf=1, north=0.0, cancel=None):
        cb = CANCEL_FN(lambda _ctx: int(bool(cancel()))) if cancel else CANCEL_FN()
        b = BounceIn(N, M, mf, north, cb, None)
        self._ok(self.d.kgb_bounce(self.h, i0, nc, flags, ctypes.byref(b)))

    def reduce_dc(self, nc, W):
        W = _f32(W)
        out = np.zeros(nc, np.float64)
        self._ok(self.d.kgb_reduce_dc(self.h, nc, _p(W), _p(out)))
        return out

    def download_dc(self, nc):
        n = self.dims()["nBins"] * nc
        out = np.zeros(n, np.float32)
        self._ok(self.d.kgb_download_dc(self.h, nc, _p(out), n))
        return out.reshape(-1, nc) if nc else out

    # --- views
    def view(self, i0, nc, flags, nAz, nEl, az0, dAz, rowSin, world=False, cull=False, jitter=True, back=False, vground=True, nS=1,
             groundZ=0.0, north=0.0, launch=0, cancel=None):
        rowSin = _f32(rowSin)
        cb = CANCEL_FN(lambda _ctx: int(bool(cancel()))) if cancel else CANCEL_FN()
        v = ViewIn(nAz, nEl, az0, dAz, _typed(rowSin, c_float), int(world), int(cull), int(jitter), int(back), int(vground), nS, groundZ,
                   north, cb, None)
        ln = c_size_t(launch)
        self._ok(self.d.kgb_view(self.h, i0, nc, flags, ctypes.byref(v), ctypes.byref(ln)))
        return ln.value

    def reduce_view(self, nc, wRow, nClass, farDist, reach=(), glazing=False, isoDim=0):
        wRow = np.ascontiguousarray(wRow, dtype=np.float64)
        reach = np.ascontiguousarray(reach, dtype=np.float32)
        NA = 3 * nClass + 1 + len(reach) + int(bool(glazing)) + int(bool(isoDim))
        out = np.zeros((nc, NA), np.float64)
        self._ok(self.d.kgb_reduce_view(self.h, nc, _p(wRow), wRow.size, nClass, farDist, _p(reach), reach.size, int(glazing), isoDim, _p(out)))
        return out

    def download_view(self, nc, out=None):
        """Classes [nc x K] uint8 and distances [nc x K] float32; out: a (cls, dist) pair of C-contiguous arrays of
        those shapes to write into (the reference's caller resizes its vectors before gpu_download_view), else new ones."""
        K = self.dims()["K"]
        if out is None:
            cls, dist = np.zeros((nc, K), np.uint8), np.zeros((nc, K), np.float32)
        else:
            cls, dist = out
            if cls.shape != (nc, K) or dist.shape != (nc, K) or cls.dtype != np.uint8 or dist.dtype != np.float32 or \
                    not (cls.flags.c_contiguous and dist.flags.c_contiguous):
                raise ValueError("download_view: out must be C-contiguous uint8 and float32 [nc x K] arrays")
        self._ok(self.d.kgb_download_view(self.h, nc, _p(cls), _p(dist), nc * K))
        return cls, dist


class Server:
    """The engine's serving loop: resident scenes, continuous batching of daylight and views requests."""

    def __init__(self, lib, hbm_budget_bytes):
        self.lib, self.d = lib, lib.dll
        self.h = self.d.kgb_server_create(int(hbm_budget_bytes))
        if not self.h:
            raise KgbError(lib.err())
        self._live = {}

    def close(self):
        if self.h:
            self.d.kgb_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_scene(self, v, tri):
        v = _f32(v, (-1, 3))
        tri = np.ascontiguousarray(tri, dtype=np.uint32).reshape(-1, 3)
        sid = c_int32(-1)
        if not self.d.kgb_server_add_scene(self.h, _p(v), len(v), _p(tri), len(tri), ctypes.byref(sid)):
            raise KgbError(self.lib.err())
        return sid.value

    def autotune(self):
        if not self.d.kgb_server_autotune(self.h):
            raise KgbError(self.lib.err())

    def set_tuning(self, chunk_sensors=0, batch_rays=0, view_rays=0):
        """Chunk sensors, daylight batch rays and views chunk rays by hand (0 keeps a value)."""
        if not self.d.kgb_server_set_tuning(self.h, int(chunk_sensors), int(batch_rays), int(view_rays)):
            raise KgbError(self.lib.err())

    def tuning(self):
        """The tuning in use: chunk sensors, daylight batch rays, views chunk rays."""
        out = (c_uint64 * 3)()
        self.d.kgb_server_tuning(self.h, out)
        return {"chunk_sensors": int(out[0]), "batch_rays": int(out[1]), "view_rays": int(out[2])}

    def set_priority(self, old_seconds=1.0, age_seconds=0.3):
        """The scheduler's priority: requests older than old_seconds first, in arrival order; the others by remaining
        work / (age + age_seconds)."""
        if not self.d.kgb_server_set_priority(self.h, float(old_seconds), float(age_seconds)):
            raise KgbError(self.lib.err())

    def submit(self, scene, P, N, D, W, use_cos, flags=5):
        """Daylight request: W [nQ x nDir]; use_cos per quantity. Returns a ticket; wait() gives out [nQ x nSensors]."""
        P, N, D = _f32(P, (-1, 3)), _f32(N, (-1, 3)), _f32(D, (-1, 3))
        W = _f32(W).reshape(len(use_cos), len(D))
        out = np.zeros((len(use_cos), len(P)), np.float64)
        mask = sum(1 << q for q, c in enumerate(use_cos) if c)
        r = DaylightRequest(scene, len(P), len(D), len(use_cos), _p(P), _p(N), _p(D), _p(W), mask, flags, _p(out))
        t = c_uint64(0)
        if not self.d.kgb_server_submit(self.h, ctypes.byref(r), ctypes.byref(t)):
            raise KgbError(self.lib.err())
        self._live[t.value] = (P, N, D, W, out, r)
        return t.value

    def submit_series(self, scene, P, N, D, W, use_cos, gQ, nSky, row, wsky, S, g, sun0, sunStep, sunVec, sunW, flags=5):
        """Daylight request with its time series: wait() gives (out [nQ x nSensors], E [nSensors x T]); G of the series is
        quantity gQ's sums (as float), as the reference's run loop passes its ground reduce."""
        P, N, D = _f32(P, (-1, 3)), _f32(N, (-1, 3)), _f32(D, (-1, 3))
        W = _f32(W).reshape(len(use_cos), len(D))
        out = np.zeros((len(use_cos), len(P)), np.float64)
        mask = sum(1 << q for q, c in enumerate(use_cos) if c)
        r = DaylightRequest(scene, len(P), len(D), len(use_cos), _p(P), _p(N), _p(D), _p(W), mask, flags, _p(out))
        row = np.ascontiguousarray(row, dtype=np.int32)
        wsky, S, g = _f32(wsky), _f32(S), _f32(g)
        Pp, T = S.shape
        sunStep = np.ascontiguousarray(sunStep, dtype=np.int32)
        sunVec, sunW = _f32(sunVec, (-1, 3)), _f32(sunW)
        E = np.zeros((len(P), T), np.float32)
        si = SeriesIn(nSky, _typed(row, c_int32), _typed(wsky, c_float), _typed(S, c_float), Pp, T, _typed(g, c_float), None, sun0,
                      len(sunStep), _typed(sunStep, c_int32), _typed(sunVec, c_float), _typed(sunW, c_float), None)
        q = SeriesRequest(si, gQ, _p(E))
        t = c_uint64(0)
        if not self.d.kgb_server_submit_series(self.h, ctypes.byref(r), ctypes.byref(q), ctypes.byref(t)):
            raise KgbError(self.lib.err())
        self._live[t.value] = ("series", (P, N, D, W, row, wsky, S, g, sunStep, sunVec, sunW, r, q), out, E)
        return t.value

    def submit_views(self, scene, P, N, nAz, nEl, az0, dAz, rowSin, wRow, nClass, farDist, reach=(), glazing=False, isoDim=0,
                     label=None, world=False, cull=False, jitter=True, back=False, vground=True, nS=1, groundZ=0.0, north=0.0, flags=1):
        P, N, rowSin = _f32(P, (-1, 3)), _f32(N, (-1, 3)), _f32(rowSin)
        wRow = np.ascontiguousarray(wRow, np.float64)
        reach = np.ascontiguousarray(reach, np.float32)
        label = None if label is None else np.ascontiguousarray(label, np.uint8)
        NA = 3 * nClass + 1 + len(reach) + int(bool(glazing)) + int(bool(isoDim))
        out = np.zeros((len(P), NA), np.float64)
        v = ViewIn(nAz, nEl, az0, dAz, _typed(rowSin, c_float), int(world), int(cull), int(jitter), int(back), int(vground), nS, groundZ,
                   north, CANCEL_FN(), None)
        r = ViewsRequest(scene, len(P), _p(P), _p(N), _p(label), v, flags, _p(wRow), nClass, farDist, _p(reach), len(reach), int(glazing),
                         isoDim, _p(out))
        t = c_uint64(0)
        if not self.d.kgb_server_submit_views(self.h, ctypes.byref(r), ctypes.byref(t)):
            raise KgbError(self.lib.err())
        self._live[t.value] = (P, N, rowSin, wRow, reach, label, out, r)
        return t.value

    def wait(self, ticket, timeout=600.0):
        if not self.d.kgb_server_wait(self.h, ticket, timeout):
            raise KgbError(self.lib.err())
        keep = self._live.pop(ticket)
        if isinstance(keep[0], str):   # a series request: its sums and its rows of E
            return keep[2], keep[3]
        return keep[4] if len(keep) == 6 else keep[6]

    def stats(self):
        out = (c_double * 10)()
        self.d.kgb_server_stats(self.h, out)
        keys = ["completed", "p50_s", "p90_s", "p99_s", "max_s", "rays", "items", "hbm_bytes", "chunk_sensors", "batch_rays"]
        return dict(zip(keys, list(out)))

    def timing(self):
        """GPU seconds and rays of daylight batches and of views chunks, and wall seconds with work queued."""
        out = (c_double * 5)()
        self.d.kgb_server_timing(self.h, out)
        return dict(zip(["day_gpu_s", "day_rays", "views_gpu_s", "views_rays", "queued_s"], list(out)))


def slots_array(slots):
    """A ctypes array of Slot from Slot objects or (rho, tau, tn, flags) tuples."""
    arr = (Slot * max(1, len(slots)))()
    for k, s in enumerate(slots):
        arr[k] = s if isinstance(s, Slot) else Slot(*s)
    if not len(slots):
        arr[0] = Slot(0.2, 0.0, 0.0, 0)
    return arr


def tn_from_Tn(Tn):
    """Glass transmissivity from the transmittance at normal incidence (the reference's glass.h:11-13)."""
    import math
    return max(0.0, (math.sqrt(0.8402528435 + 0.0072522239 * Tn * Tn) - 0.9166530661) / 0.0036261119 / Tn)
