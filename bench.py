#!/usr/bin/env python3
"""Benchmark of the ray-cast-and-accumulate hot path on GB300: the urban block (200k sensor faces, 403k triangles, 5610 directions).

Workload (one step): the seeded 20 x 20 urban block (199,976 sensor faces, 403,152 triangles, resident BVH) traced
against 5610 directions (577 Reinhart sky patches, their ground mirror, 4456 sun-up hours of the synthetic urban
weather year) - 1.12 G any-hit rays - then the four cumulative quantities reduced per sensor (radiation, irradiance,
illuminance, sun hours), as the reference's chunk loop does (src/run.cpp:642-657: gpu_trace + gpu_reduce per quantity).
The direction table and weights are the reference's own (tests/golden/urban_sky: recorded from its host code).

Metric: Mrays/s (sensor x direction slots per second, the reference's GRays/s counting, x1000), higher is better.
 value: inputs resident in HBM, CUDA events on the engine's stream around trace + reduces; L2 flushed between steps.
 e2e:   the same through the C ABI with host buffers: set_scene (sensors, directions) from pinned memory, trace, the
        four reduces with their weights up and sums down, every step.
--impl reference: the oracle (the CPU restatement of the reference's path) on the host's cores, bounded samples.
"""
import argparse
import importlib.util
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(REPO, "tests", "golden")
NODE_BYTES = 208   # the BVH8 node record (kNodeBytes of the engine)


def package():
    if "kitsim_gb300" in sys.modules:
        return sys.modules["kitsim_gb300"]
    d = os.path.join(REPO, "kit-sim_daylight_gb300")
    spec = importlib.util.spec_from_file_location("kitsim_gb300", os.path.join(d, "__init__.py"), submodule_search_locations=[d])
    m = importlib.util.module_from_spec(spec)
    sys.modules["kitsim_gb300"] = m
    spec.loader.exec_module(m)
    return m


def urban_sky():
    """Direction table and per-quantity weights of the urban block (the reference's host code, recorded)."""
    calls = [json.loads(l) for l in open(os.path.join(GOLDEN, "urban_sky", "calls.jsonl"))]
    last = max(i for i, c in enumerate(calls) if c["call"] == "gpu_set_scene")
    c = calls[last]
    D = np.fromfile(os.path.join(GOLDEN, "urban_sky", c["D"][2]), np.float32).reshape(-1, 3)
    Ws = []
    for c in calls[last:]:
        if c["call"] == "gpu_reduce":
            Ws.append((np.fromfile(os.path.join(GOLDEN, "urban_sky", c["W"][2]), np.float32), bool(c["useCos"])))
    manifest = json.load(open(os.path.join(GOLDEN, "urban_sky", "manifest.json")))
    return D, Ws, manifest


class Clocks:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""
    Q = "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown," \
        "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"

    def __init__(self, index=0):
        self.rows, self.proc, self.index = [], None, index

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q, "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            p = [x.strip() for x in line.split(",")]
            if len(p) >= 8:
                self.rows.append(p)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows for k in range(4) if r[4 + k].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.rows)}


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        m = json.load(open(p))
        return m["hbm_gbs"], "measured"
    return 6800.0, "fallback"


def measured_peak(key):
    """(value, kind) of a MEASURED_PEAKS.json entry, else the fallback figure (bf16 dense burst 1900 TFLOP/s)."""
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        m = json.load(open(p))
        if key in m:
            return float(m[key]), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}[key], "fallback"


def profiled(key, summary="k_bits_urban.md"):
    """A figure of a committed ncu summary (profiles/<summary>: lines `key: value`), or None. k_bits_urban.md (k_bits on
    the urban block): traffic_per_full_trace_bytes (DRAM read + write of one trace), inst_per_full_trace (warp
    instructions of one trace), thread_inst_per_full_trace (the same counted per active thread). k_view_views.md
    (k_view on the views city): inst_per_fov120_trace, thread_inst_per_fov120_trace (the whole city at fov 120)."""
    p = os.path.join(REPO, "profiles", summary)
    if os.path.exists(p):
        for line in open(p):
            if line.startswith(key + ":"):
                return float(line.split(":")[1])
    return None


def oracle_lib(pkg):
    """The oracle (the checker, and the CPU legs' restatement), built from oracle/ if needed."""
    subprocess.check_call(["make", "-s", "-C", os.path.join(REPO, "oracle"), "all"])
    return pkg.kgb.Lib(os.path.join(REPO, "oracle", "_build", "liboracle.so"))


def cpu_baseline(pkg, scene, D, Ws, sample, seed=0):
    """The oracle (the CPU restatement) on the host's cores: trace + the four reduces of a seeded sensor sample."""
    sys.path.insert(0, os.path.join(REPO, "tests"))
    lib = oracle_lib(pkg)
    o = pkg.kgb.Engine(lib)
    o.build(scene["v"], scene["tri"])
    pick = np.sort(np.random.default_rng(seed).choice(len(scene["P"]), sample, replace=False))
    o.set_scene(scene["P"][pick], scene["N"][pick], D)
    t0 = time.perf_counter()
    o.trace(0, sample, lib.ray_flags(False, False))
    for W, use_cos in Ws:
        o.reduce(sample, W, use_cos)
    dt = time.perf_counter() - t0
    o.close()
    return sample * len(D) / dt / 1e6, dt


def exact_geometry(pkg, scene, D, sensors=1024, seed=11):
    """The checker (the oracle, untimed): how many rays of a seeded sample of the block the shared float decision takes
    differently from every test and rule evaluated in double (oracle kgbo_recheck_bits; categories as in
    tests/test_grazing.py)."""
    import ctypes
    lib = pkg.kgb.Lib(os.path.join(REPO, "oracle", "_build", "liboracle.so"))
    f = lib.dll.kgbo_recheck_bits
    f.restype, f.argtypes = ctypes.c_int, [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_uint32, ctypes.c_double, ctypes.c_void_p]
    o = pkg.kgb.Engine(lib)
    o.build(scene["v"], scene["tri"])
    o.set_scene(scene["P"], scene["N"], D)
    tot = np.zeros(24)
    t0 = time.perf_counter()
    for i0 in np.random.default_rng(seed).choice(len(scene["P"]) // 128, sensors // 128, replace=False) * 128:
        out = np.zeros(24)
        if not f(o.h, int(i0), 128, lib.ray_flags(False, False), 2.0 ** -16, out.ctypes.data_as(ctypes.c_void_p)):
            o.close()
            return {"error": lib.err()}
        tot[:17] += out[:17]
        tot[[17, 18]] = np.maximum(tot[[17, 18]], out[[17, 18]])
    o.close()
    keys = ["rays", "decided_differently", "edge", "grazing", "threshold", "tie", "rounding", "other"]
    r = {k: int(x) for k, x in zip(keys, tot[:8])}
    r.update(edge_band="2^-16 x (|o|max + t)", max_edge_distance_m=float(tot[17]), sample="%d seeded sensors x %d directions" % (sensors, len(D)),
             seconds=time.perf_counter() - t0)
    return r


def run_reference(args, pkg):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    scene = pkg.workloads.urban_block()
    D, Ws, _ = urban_sky()
    cores = os.cpu_count()
    sample = args.ref_sample
    for _ in range(args.warmup):
        cpu_baseline(pkg, scene, D, Ws, max(64, sample // 8), seed=1)
    vals, secs = [], []
    for k in range(args.steps):
        v, dt = cpu_baseline(pkg, scene, D, Ws, sample, seed=100 + k)
        vals.append(v)
        secs.append(dt)
    value = float(np.median(vals))
    line = {"metric": "Mrays/s", "value": value, "unit": "Mrays/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000 * float(np.median(secs)), "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded urban block; the reference's direction table and weights)", "impl": "reference",
            "config": {"workload": "urban block: 20x20 boxes, %d sensors, %d triangles, %d directions (577 sky + ground + sun), "
                                   "4 quantities" % (len(scene["P"]), len(scene["tri"]), len(D)), "l2": "n/a (CPU)"},
            "cpu_baseline": {"value": value, "unit": "Mrays/s", "cores": cores, "kind": "port",
                             "sample": "%d seeded sensors of the block x %d directions per step (+ the 4 reduces)" % (sample, len(D))},
            "e2e": {"value": value, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args, pkg):
    import torch
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    pkg.load()
    scene = pkg.workloads.urban_block(seed=42 + rank)   # weak scaling: every rank its own block of the same shape
    if args.sensors:   # a smaller case of the same kernel (profiling): the block's first sensors
        scene = dict(scene, P=scene["P"][:args.sensors], N=scene["N"][:args.sensors])
    D, Ws, manifest = urban_sky()
    nc, nDir = len(scene["P"]), len(D)
    stream = torch.cuda.Stream()
    e = pkg.engine()
    e.set_stream(stream.cuda_stream)
    e.set_builder(args.builder)
    e.build(scene["v"], scene["tri"])
    flags = e.lib.ray_flags(False, False)
    # pinned host copies of the step's inputs (e2e) and outputs
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    P, N, Dp = pin(scene["P"]), pin(scene["N"]), pin(D)
    Wp = [(pin(W), c) for W, c in Ws]
    flush = torch.empty(int(512e6) // 4, dtype=torch.float32, device="cuda")   # > the 129 MB L2
    e.set_scene(P, N, Dp)

    def step_device():
        e.trace(0, nc, flags)
        for W, c in Wp:
            e.reduce(nc, W, c)

    def step_e2e():
        e.set_scene(P, N, Dp)
        step_device()

    # roofline accounting: the instrumented traversal on the same inputs (untimed)
    cnt = e.trace_counters(0, nc, flags)
    for _ in range(args.warmup):
        step_device()
        step_e2e()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    st0 = e.stats()
    times, ttrace = [], []
    with Clocks(local) as clk:
        for _ in range(args.steps):
            with torch.cuda.stream(stream):
                flush.zero_()
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
            ev[0].record(stream)
            e.trace(0, nc, flags)
            ev[1].record(stream)
            for W, c in Wp:
                e.reduce(nc, W, c)
            ev[2].record(stream)
            ev[2].synchronize()
            times.append(ev[0].elapsed_time(ev[2]))
            ttrace.append(ev[0].elapsed_time(ev[1]))
        st1 = e.stats()   # the device-timed steps' launches (the e2e steps below run the same ones again)
        e2e_t = []
        for _ in range(args.steps):
            with torch.cuda.stream(stream):
                flush.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            step_e2e()
            e2e_t.append((time.perf_counter() - t0) * 1000)
    if world > 1:
        torch.distributed.barrier()
    ms = float(sum(times) / len(times))
    ms_e2e = float(sum(e2e_t) / len(e2e_t))
    ms, ms_e2e = pkg.shard.max_over_ranks([ms, ms_e2e], device="cuda")   # the slowest rank's times (NCCL when N > 1)
    rays = nc * nDir
    launches = (st1["launches"] - st0["launches"]) // args.steps + len(Wp)
    # roofline of k_bits: algorithmic bytes = nodes x 208 (the node record) + triangles tested x 48 + bits out + sensor
    # reads per task
    tasks = (nc + 31) // 32 * ((nDir + 31) // 32)
    alg = cnt["nodes"] * NODE_BYTES + cnt["tris"] * 48 + nc * ((nDir + 31) // 32) * 4 + tasks * 32 * 24
    ms_trace = float(np.median(ttrace))
    peak, kind = peaks()
    traffic, inst, tinst = profiled("traffic_per_full_trace_bytes"), profiled("inst_per_full_trace"), profiled("thread_inst_per_full_trace")
    sm_mhz = clk.summary()["sm_mhz"] or 2070.0
    num_sms = torch.cuda.get_device_properties(local).multi_processor_count
    issue_peak = 4.0 * num_sms * sm_mhz * 1e6   # four schedulers per SM, one warp instruction each per cycle
    if rank == 0:
        line = {"metric": "Mrays/s", "value": world * rays / (ms / 1000) / 1e6, "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (seeded urban block; the reference's direction table and weights, tests/golden/urban_sky)",
                "config": {"workload": (("urban block: 20x20 boxes, %d sensors, %d triangles, %d directions (%d sky + %d ground + %d sun), " if not args.sensors else
                                         "urban block, first %d sensors only (profiling case), %d triangles, %d directions (%d sky + %d ground + %d sun), ") +
                                        "trace + 4 reduces (radiation, irradiance, illuminance, sunhours)") %
                                       (nc, len(scene["tri"]), nDir, manifest["dirs"]["sky"], manifest["dirs"]["ground"], manifest["dirs"]["sun"]),
                           "rays_per_step": rays, "l2": "flushed between steps (512 MB write)", "parallelism": "replicas (weak)" if world > 1 else "1 GPU",
                           "bvh": "device LBVH + treelet restructuring" if args.builder else "host binned SAH"},
                "e2e": {"value": world * rays / (ms_e2e / 1000) / 1e6, "unit": "Mrays/s",
                        "h2d_bytes_per_step": int(P.nbytes + N.nbytes + Dp.nbytes + sum(W.nbytes for W, _ in Wp)),
                        "d2h_bytes_per_step": int(8 * nc * len(Wp))},
                "gpu_launches": int(launches),
                "roofline": {"bound": "issue", "kernel": "k_bits",
                             "achieved": inst / (ms_trace / 1000) if inst else None, "peak": issue_peak, "unit": "warp-inst/s",
                             "frac": inst / (ms_trace / 1000) / issue_peak if inst else None,
                             "peak_kind": "4 issue slots per SM per cycle x %d SMs at the sampled median SM clock (%.0f MHz)" % (num_sms, sm_mhz),
                             "lanes_active_of_32": tinst / inst if (inst and tinst) else None,
                             "traffic": traffic, "trace_ms": ms_trace,
                             "hbm": {"achieved": traffic / (ms_trace / 1000) / 1e9 if traffic else None, "peak": peak, "unit": "GB/s",
                                     "frac": traffic / (ms_trace / 1000) / 1e9 / peak if traffic else None, "peak_kind": kind,
                                     "bytes": "traffic: dram__bytes_read.sum + dram__bytes_write.sum of one full trace"},
                             "cache_bytes": {"per_trace": alg, "per_s": alg / (ms_trace / 1000),
                                             "what": "node records x 208 B + triangle records x 48 B read by the rays (L1 93 %, L2), "
                                                     "+ bits out + sensor reads, from the instrumented traversal on the same inputs"},
                             "nodes_visited": cnt["nodes"], "tris_tested": cnt["tris"], "rays_traced": cnt["rays"], "bvh_bytes": cnt["bvh_bytes"],
                             "inst_per_trace": inst, "note": "the traversal is bound by instruction issue: its 27 MB tree stays in L2 and "
                                                             "93 % of its loads hit L1, so HBM is nearly idle (hbm.frac); achieved = warp "
                                                             "instructions of one trace (ncu, profiles/k_bits_urban.md) / the trace's "
                                                             "CUDA-event time"},
                "step_ms": {"device": [float(x) for x in times], "e2e": [float(x) for x in e2e_t]},
                "clocks": clk.summary()}
        if not args.no_cpu_baseline:
            v, dt = cpu_baseline(pkg, scene, D, Ws, args.cpu_sample)
            line["cpu_baseline"] = {"value": v, "unit": "Mrays/s", "cores": os.cpu_count(), "kind": "port",
                                    "sample": "%d seeded sensors of the block x %d directions + the 4 reduces (%.1f s)" % (args.cpu_sample, nDir, dt)}
            line["exact_geometry"] = exact_geometry(pkg, scene, D)
    e.close()
    if rank == 0 and world == 1 and not args.no_extras and not args.sensors:
        # the other measured configurations, after the timed region: each keeps its own metric and config
        for key, fn in (("precision", run_precision), ("views", run_views), ("serving", run_serving), ("serving_series", run_serving_series),
                        ("ingest", run_ingest)):
            t0 = time.perf_counter()
            try:
                line[key] = fn(args, pkg)
            except Exception as ex:   # the headline stands without them
                line[key] = {"error": "%s: %s" % (type(ex).__name__, ex)}
            line[key]["config_wall_s"] = time.perf_counter() - t0   # the whole configuration, its set-up included
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


# ---------------------------------------------------------------------------------------------- precision: 2305-patch series
def run_precision(args, pkg):
    """The precision configuration: the urban block at 2305 patches, 20 % glass (byte mode), one diffuse bounce of 1024 paths per sensor,
    and the hourly series of the non-night hours with reflected light, chunk by chunk as the reference's run() does
    (run.cpp:623-688: trace, bounce, ground reduce, series). The split-BF16 tensor-core series is timed against the
    plain FP32 form on the same inputs, and its error per output column is measured against the oracle's FP64
    contraction on a contiguous 64-sensor range (the same global indices, so the same reflected-light paths)."""
    import torch
    torch.cuda.set_device(0)
    kgb = pkg.kgb
    lib = pkg.load()
    e = pkg.engine()
    mf, M = 4, 1024
    Dsky, omega = pkg.workloads.patch_dirs(mf)
    P = len(Dsky)
    yr = pkg.workloads.urban_year_sky(e, mf, np.load(os.path.join(GOLDEN, "urban_sky", "weather.npy")))
    # ladybug mode's sky of the same weather year on the device (sky density 2; the steps as the reference makes them,
    # tests/golden/ladybug): the faster of two calls
    lbg = np.load(os.path.join(GOLDEN, "ladybug", "mf2.npz"))
    _, _, _, lb_hours, lb_lat, lb_lon, lb_tz = lbg["head"]
    lb_s = []
    for _ in range(2):
        t0 = time.perf_counter()
        e.sky_ladybug(2, lbg["steps"], lb_lat, lb_lon, lb_tz, float(lbg["grefl"]), lb_hours, series=True)
        lb_s.append(time.perf_counter() - t0)
    D = np.concatenate([Dsky, -Dsky, yr["sunVec"]]).astype(np.float32)
    nSky, sun0 = P, 2 * P
    scene = pkg.workloads.urban_block(glass_share=0.2)
    if args.sensors:   # a smaller case of the same kernels (profiling): the block's first sensors
        scene = dict(scene, P=scene["P"][:args.sensors], N=scene["N"][:args.sensors])
    slots = [(0.2, 0, 0, 0), (0.0, 0.64, kgb.tn_from_Tn(0.64), kgb.SLOT_GLASS), (0.2, 0, 0, 0)]
    e.build(scene["v"], scene["tri"], scene["slot"], slots, per_slot=True)
    e.set_slots(slots)
    e.set_scene(scene["P"], scene["N"], D)
    nc_all, T = len(scene["P"]), yr["T"]
    Wg = np.zeros(len(D), np.float32)
    Wg[nSky:2 * nSky] = omega
    flags = lib.ray_flags(False, True)   # a slot transmits: bytes
    bflags = lib.bounce_flags(False)
    chunk = max(1, (256 << 20) // len(D))   # the reference's 256 MiB cap on the per-chunk visibility
    sargs = dict(nSky=nSky, row=np.arange(nSky), wsky=omega, S=yr["S"], g=yr["g"], sun0=sun0, sunStep=yr["sunStep"], sunVec=yr["sunVec"],
                 sunW=yr["sunW"], Sdc=yr["Sdc"])
    tt = {"trace": 0.0, "bounce": 0.0, "tc": 0.0, "fp32": 0.0, "copy": 0.0, "fwrite": 0.0, "direct": 0.0, "tc_repeat": 0.0}
    first = fp32_first = None
    Ebuf = np.empty((min(chunk, nc_all), T), np.float32)   # one E for every chunk, written with zeros first (run.cpp:683-686)
    Ebuf.fill(0.0)
    # the --timeseries file, two ways: the reference's (gpu_series into E, then fwrite) and kgb_series_file (the rows
    # written from the engine's pinned staging); both files under a 128-byte header, compared byte for byte after
    import shutil
    import tempfile
    E_bytes = nc_all * T * 4
    tmpdir = tempfile.mkdtemp(prefix="kgb_series_")
    files = shutil.disk_usage(tmpdir).free > 2 * E_bytes + (2 << 30)
    if files:
        f_ref = open(os.path.join(tmpdir, "ref.npy"), "wb")
        f_ref.write(b"\0" * 128)
        fd_dir = os.open(os.path.join(tmpdir, "direct.npy"), os.O_CREAT | os.O_RDWR | os.O_TRUNC, 0o644)
    st0 = e.stats()
    tc_calls = 0   # tensor-core series calls (the timed ones, their repeats and the file-writing ones)
    t_all = time.perf_counter()
    for i0 in range(0, nc_all, chunk):
        nc = min(chunk, nc_all - i0)
        t0 = time.perf_counter()
        e.trace(i0, nc, flags)
        torch.cuda.synchronize()
        tt["trace"] += time.perf_counter() - t0
        t0 = time.perf_counter()
        e.bounce(i0, nc, bflags, N=1, M=M, mf=mf, north=0.0)
        tt["bounce"] += time.perf_counter() - t0
        G = e.reduce(nc, Wg, True).astype(np.float32)
        for form, key in ((0, "tc"), (1, "fp32")):
            if key == "fp32" and i0 > 0 and not args.full_fp32:
                continue   # the plain FP32 form is timed on the first chunk (it is the slow one)
            e.set_series_form(form)
            # the tensor-core series twice per chunk into the same E, the faster call counted (the rows go to pageable
            # host memory, whose copy rate varies from box to box); the plain form once (it is the slow one)
            best = None
            for _ in range(2 if key == "tc" else 1):
                t0 = time.perf_counter()
                E = e.series(nc, G=G, out=Ebuf[:nc], **sargs)
                tc_calls += 1 if key == "tc" else 0
                dt = time.perf_counter() - t0
                if best is not None:
                    tt["tc_repeat"] += max(dt, best)   # the pipeline's wall time counts one call
                best = dt if best is None else min(best, dt)
            tt[key] += best
            if key == "tc" and files:   # untimed by the pipeline: the file output of the same chunk, both ways
                t1 = time.perf_counter()
                E.tofile(f_ref)
                f_ref.flush()
                d1 = time.perf_counter() - t1
                t1 = time.perf_counter()
                e.series_file(nc, fd_dir, 128 + i0 * T * 4, G=G, **sargs)
                tc_calls += 1
                d2 = time.perf_counter() - t1
                tt["fwrite"] += d1
                tt["direct"] += d2
                tt["copy"] += d1 + d2
            if i0 == 0:   # kept for the accuracy check; the copy is not part of the pipeline
                t0 = time.perf_counter()
                if form == 0:
                    first = (E.copy(), G)
                else:
                    fp32_first = E.copy()
                tt["copy"] += time.perf_counter() - t0
    e.set_series_form(0)
    pipeline_s = time.perf_counter() - t_all - tt["copy"] - tt["tc_repeat"]
    st1 = e.stats()
    # roofline of k_series_tc: 6 bf16 products x 2 x Kp flop per output, over the kernels' CUDA-event time (every
    # tensor-core series call of the run, the file-writing ones included)
    Kp = (P + 1 + (P + 1) + 63) // 64 * 64
    series_ms = st1["seriesMs"] - st0["seriesMs"]
    series_flop = (st1["seriesOutputs"] - st0["seriesOutputs"]) * 12 * Kp
    tc_peak = measured_peak("bf16_tflops_sustained")   # the kernels run inside a pipeline of seconds
    series_file = {"skipped": "less than twice the file's size free in %s" % tmpdir}
    if files:
        f_ref.close()
        os.close(fd_dir)
        same = True
        with open(os.path.join(tmpdir, "ref.npy"), "rb") as a, open(os.path.join(tmpdir, "direct.npy"), "rb") as b:
            while True:
                x, y = a.read(1 << 28), b.read(1 << 28)
                if x != y:
                    same = False
                    break
                if not x:
                    break
        series_file = {"bytes": E_bytes, "reference_way_s": tt["tc"] + tt["fwrite"], "fwrite_s": tt["fwrite"], "direct_s": tt["direct"],
                       "direct_gb_s": E_bytes / tt["direct"] / 1e9, "files_identical": same,
                       "note": "reference way: gpu_series into one reused E, then fwrite per chunk; direct: kgb_series_file per chunk"}
    shutil.rmtree(tmpdir, ignore_errors=True)
    # accuracy (the checker, untimed): a contiguous range of the first chunk's sensors, traced and bounced by the oracle
    # at the same global indices, its series in FP64 from the same FP32 inputs; the error per output column
    # (max_i |E - E64| / max_i |E64|) and per output (|E - E64| / E64 for outputs at or above 1e-6 of their column's
    # maximum: every term of the contraction is non-negative, so no output is a cancellation)
    ns = min(args.accuracy_sensors, min(chunk, nc_all))
    s0 = int(np.random.default_rng(9).integers(0, min(chunk, nc_all) - ns + 1))
    sub = np.arange(s0, s0 + ns)
    subprocess.check_call(["make", "-s", "-C", os.path.join(REPO, "oracle"), "all"])
    o = kgb.Engine(kgb.Lib(os.path.join(REPO, "oracle", "_build", "liboracle.so")))
    o.build(scene["v"], scene["tri"], scene["slot"], slots, per_slot=True)
    o.set_slots(slots)
    o.set_scene(scene["P"], scene["N"], D)
    o.trace(s0, ns, flags)
    o.bounce(s0, ns, bflags, N=1, M=M, mf=mf, north=0.0)
    E64 = o.series(ns, G=first[1][sub], **sargs).astype(np.float64)
    o.close()
    cmax = np.abs(E64).max(axis=0)
    live = cmax > 0
    mask = (E64 > 0) & (E64 >= 1e-6 * cmax[None, :])
    def colerr(E):
        return np.abs(E[sub] - E64).max(axis=0)[live] / cmax[live]
    def elemerr(E):
        rel = np.abs(E[sub].astype(np.float64) - E64)[mask] / E64[mask]
        return {"max": float(rel.max()), "p99": float(np.percentile(rel, 99)), "median": float(np.median(rel)), "outputs": int(mask.sum()),
                "floor": "E64 >= 1e-6 x its column's maximum"}
    ce, ce32 = colerr(first[0]), colerr(fp32_first)
    n_fp32 = nc_all if args.full_fp32 else min(chunk, nc_all)
    paths = nc_all * M
    line = {"metric": "radiation solves/s", "unit": "sensor-steps/s",
            "value": nc_all * T / tt["tc"], "fp32_value": n_fp32 * T / tt["fp32"], "speedup_vs_fp32": (nc_all * T / tt["tc"]) / (n_fp32 * T / tt["fp32"]),
            # the plain FP32 form is the reference's k_series restated (a thread per sensor, one product a term): its own
            # rate, 2 K flop an output, beside the GPU's FP32 rate, so the speed-up reads as over that form
            "fp32_form_tflops": n_fp32 * T * 2.0 * Kp / tt["fp32"] / 1e12,
            "config": {"workload": "precision: urban block, %d sensors, %d patches + ground, %d directions, %d series columns (non-night hours), "
                                   "20%% glass tau 0.64 (byte mode), 1 bounce x %d paths (%d reflected-light bins in K), chunks of %d sensors"
                                   % (nc_all, P, len(D), T, M, P + 1, chunk)},
            "dtype": "split-bf16 (3 pieces, 6 products) on tcgen05, fp32 accumulate in chains of 64 of K, each chain added into fp32 sums with Kahan compensation; sun term fp32",
            "roofline": {"bound": "tensor", "kernel": "k_series_tc", "achieved": series_flop / (series_ms / 1000) / 1e12 if series_ms else None,
                         "peak": tc_peak[0], "unit": "TFLOP/s", "peak_kind": tc_peak[1] + " bf16 sustained",
                         "frac": series_flop / (series_ms / 1000) / 1e12 / tc_peak[0] if series_ms else None, "traffic": None,
                         "flop_per_output": 12 * Kp, "kernel_ms": series_ms},
            "column_error_vs_fp64": {"max": float(ce.max()), "p99": float(np.percentile(ce, 99)), "median": float(np.median(ce)),
                                     "columns_over_1e-6": int((ce > 1e-6).sum()), "columns": int(ce.size), "sample_sensors": len(sub)},
            "element_error_vs_fp64": elemerr(first[0]),
            "fp32_column_error_vs_fp64": {"max": float(ce32.max()), "median": float(np.median(ce32))},
            "fp32_element_error_vs_fp64": elemerr(fp32_first),
            "trace_mrays_s": nc_all * len(D) / tt["trace"] / 1e6, "bounce_mpaths_s": paths / tt["bounce"] / 1e6, "sky_build_s": yr["sky_s"],
            "ladybug_sky_s": min(lb_s), "ladybug_sky": "mf 2 (577 patches), %d steps: sun.c, the Perez sky twice a step, the float sums and the %%.3g weights, with the series columns" % len(lbg["steps"]),
            "trace_s": tt["trace"], "bounce_s": tt["bounce"], "series_tc_s": tt["tc"], "series_fp32_s_timed": tt["fp32"],
            "device_s": {"trace": (st1["traceMs"] - st0["traceMs"]) / 1000, "bounce": (st1["bounceMs"] - st0["bounceMs"]) / 1000,
                         "series_tc": series_ms / 1000, "series_tc_calls": tc_calls, "series_tc_per_pass": series_ms / 1000 / max(tc_calls, 1) * ((nc_all + chunk - 1) // chunk),
                         "bounce_launches": int(st1["bounceLaunches"] - st0["bounceLaunches"])},
            "pipeline_s": pipeline_s - (tt["fp32"] if not args.full_fp32 else 0.0),
            "pipeline_solves_s": nc_all * T / (pipeline_s - (tt["fp32"] if not args.full_fp32 else 0.0)),
            "E_bytes": nc_all * T * 4, "series_file": series_file, "note": "series times include the E download to host memory (pageable, one buffer reused across chunks), as the reference's gpu_series"}
    e.close()
    return line


# ---------------------------------------------------------------------------------------------- views: the 2 M-triangle city
def run_views(args, pkg):
    import torch
    torch.cuda.set_device(0)
    lib = pkg.load()
    e = pkg.engine()
    city = pkg.workloads.views_city()
    if args.sensors:   # a smaller case of the same kernels (profiling): the city's first sensors
        city = dict(city, P=city["P"][:args.sensors], N=city["N"][:args.sensors])
    e.build(np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32), np.array([[0, 1, 2]], np.uint32))   # warm-up of the device builder
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e.build(city["v"], city["tri"])
    torch.cuda.synchronize()
    build_s = time.perf_counter() - t0
    e.set_labels(city["label"])
    nc = len(city["P"])
    e.set_scene(city["P"], city["N"], np.zeros((0, 3), np.float32))
    flags = lib.bounce_flags(False)
    res = {}
    for name, fov, world, iso, reach in (("fov120", 120.0, False, 0, []), ("fov360", 360.0, True, 3, [6.0, 20.0, 50.0])):
        nAz, nEl, dAz, rowSin, wRow = pkg.workloads.views_grid(fov, 2.0)
        kw = dict(world=world, cull=world, jitter=True, vground=True, groundZ=city["groundZ"])
        e.view(0, min(nc, 4096), flags, nAz, nEl, 0.0 if world else -fov / 2, dAz, rowSin, **kw)   # warm-up
        torch.cuda.synchronize()
        best = None
        with Clocks(0) as clk:
            for _ in range(max(1, args.steps)):
                st0 = e.stats()
                t0 = time.perf_counter()
                e.view(0, nc, flags, nAz, nEl, 0.0 if world else -fov / 2, dAz, rowSin, **kw)
                t1 = time.perf_counter()
                st1 = e.stats()
                out = e.reduce_view(nc, wRow, 6, 1000.0, reach=reach, glazing=False, isoDim=iso)
                t2 = time.perf_counter()
                if best is None or t1 - t0 < best[0]:
                    best = (t1 - t0, t2 - t1, (st1["traceMs"] - st0["traceMs"]) / 1e3, st1["launches"] - st0["launches"])
        K = nAz * nEl
        res[name] = {"rays": nc * K, "trace_s": best[0], "reduce_s": best[1], "mrays_s": nc * K / best[0] / 1e6, "kernel_s": best[2],
                     "launches": int(best[3]), "clocks": clk.summary(),
                     "shares_sum_check": float(np.abs(out[:, 0] + out[:, 3] + out[:, 6] + out[:, 9] + out[:, 12] + out[:, 15] + out[:, 18] - 1).max())}
        if world:   # the per-ray rows (gpu_download_view: classes + distances, [nc x K]), transposed on the device, into
            # buffers already written (the reference's caller resizes its vectors first, gpu.cu:730-731)
            cls, dist = np.zeros((nc, K), np.uint8), np.zeros((nc, K), np.float32)
            cls.fill(0)
            dist.fill(0.0)
            t0 = time.perf_counter()
            e.download_view(nc, out=(cls, dist))
            dl_s = time.perf_counter() - t0
            back_c, back_d = np.zeros((K, nc), np.uint8), np.zeros((K, nc), np.float32)   # the same transpose on the host,
            back_c.fill(0)                                                              # one thread, into written buffers
            back_d.fill(0.0)
            t1 = time.perf_counter()
            np.copyto(back_c, cls.T)
            np.copyto(back_d, dist.T)
            t2 = time.perf_counter()
            del back_c, back_d
            res[name]["download_rows"] = {"bytes": nc * K * 5, "s": dl_s, "gb_s": nc * K * 5 / dl_s / 1e9, "host_transpose_s": t2 - t1}
            del cls, dist
    # many sensor meshes: 40 meshes of sizes log-uniform 500..50k (seeded), each a contiguous run of the city's facade
    # sensors from a seeded start, their sensors one after another in the engine's sensor array. Fov 120: one
    # kgb_view + kgb_reduce_view per mesh, against all meshes packed into one call (what the reference's views run does:
    # every mesh's sensors in one array, chunked by memory); the same sums either way
    rng = np.random.default_rng(4)
    sizes = [int(np.exp(rng.uniform(np.log(500), np.log(50_000)))) for _ in range(40)]
    firsts = [int(rng.integers(0, nc - n + 1)) for n in sizes]
    Pm = np.concatenate([city["P"][a:a + n] for a, n in zip(firsts, sizes)])
    Nm = np.concatenate([city["N"][a:a + n] for a, n in zip(firsts, sizes)])
    ncm = len(Pm)
    e.set_scene(Pm, Nm, np.zeros((0, 3), np.float32))
    nAz, nEl, dAz, rowSin, wRow = pkg.workloads.views_grid(120.0, 2.0)
    kw = dict(world=False, cull=False, jitter=True, vground=True, groundZ=city["groundZ"])
    starts = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(int)
    per_mesh, packed = [], []
    for rep in range(2):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sums_m = []
        for a, n in zip(starts, sizes):
            e.view(int(a), n, flags, nAz, nEl, -60.0, dAz, rowSin, **kw)
            sums_m.append(e.reduce_view(n, wRow, 6, 1000.0))
        per_mesh.append(time.perf_counter() - t0)
        t0 = time.perf_counter()
        e.view(0, ncm, flags, nAz, nEl, -60.0, dAz, rowSin, **kw)
        sums_p = e.reduce_view(ncm, wRow, 6, 1000.0)
        packed.append(time.perf_counter() - t0)
    same = bool(np.array_equal(np.concatenate(sums_m).view(np.uint64), sums_p.view(np.uint64)))
    meshes = {"meshes": len(sizes), "sensors": ncm, "smallest": int(min(sizes)), "largest": int(max(sizes)),
              "per_mesh_s": min(per_mesh), "packed_s": min(packed), "per_mesh_mrays_s": ncm * nAz * nEl / min(per_mesh) / 1e6,
              "packed_mrays_s": ncm * nAz * nEl / min(packed) / 1e6, "speedup": min(per_mesh) / min(packed), "sums_identical": same,
              "what": "fov 120 view + reduce_view of 40 sensor meshes: one call per mesh against one call for all (wall time, sums in host memory)"}
    e.set_scene(city["P"], city["N"], np.zeros((0, 3), np.float32))
    # the host binned-SAH builder on the same city: build time, and the fov 120 trace on its tree (same results)
    e.set_builder(0)
    t0 = time.perf_counter()
    e.build(city["v"], city["tri"])
    torch.cuda.synchronize()
    host_build_s = time.perf_counter() - t0
    e.set_labels(city["label"])
    e.set_scene(city["P"], city["N"], np.zeros((0, 3), np.float32))
    nAz, nEl, dAz, rowSin, wRow = pkg.workloads.views_grid(120.0, 2.0)
    kw = dict(world=False, cull=False, jitter=True, vground=True, groundZ=city["groundZ"])
    best = None
    for _ in range(max(1, args.steps)):
        t0 = time.perf_counter()
        e.view(0, nc, flags, nAz, nEl, -60.0, dAz, rowSin, **kw)
        t1 = time.perf_counter()
        best = t1 - t0 if best is None else min(best, t1 - t0)
    host_tree = {"build_s": host_build_s, "fov120_mrays_s": nc * nAz * nEl / best / 1e6, "gas_bytes": e.stats()["gasBytes"]}
    # k_view's ceiling is instruction issue, as k_bits': the warp instructions of a whole-city fov 120 trace (ncu,
    # profiles/k_view_views.md) over its kernels' CUDA-event time, against 4 issue slots per SM per cycle
    inst = profiled("inst_per_fov120_trace", "k_view_views.md") if not args.sensors else None
    tinst = profiled("thread_inst_per_fov120_trace", "k_view_views.md") if not args.sensors else None
    sm_mhz = res["fov120"]["clocks"]["sm_mhz"] or 2070.0
    num_sms = torch.cuda.get_device_properties(0).multi_processor_count
    issue_peak = 4.0 * num_sms * sm_mhz * 1e6
    kern_s = res["fov120"]["kernel_s"]
    roof = {"bound": "issue", "kernel": "k_view", "achieved": inst / kern_s if inst else None, "peak": issue_peak, "unit": "warp-inst/s",
            "frac": inst / kern_s / issue_peak if inst else None,
            "peak_kind": "4 issue slots per SM per cycle x %d SMs at the sampled median SM clock (%.0f MHz)" % (num_sms, sm_mhz),
            "lanes_active_of_32": tinst / inst if (inst and tinst) else None, "kernel_s": kern_s,
            "note": "closest-hit walk: its 2 M-triangle tree stays in L2 and most loads hit L1 (DRAM nearly idle), so instruction "
                    "issue bounds it; achieved = warp instructions of the fov 120 trace of the whole city (ncu, "
                    "profiles/k_view_views.md) / its kernels' CUDA-event time"}
    line = {"metric": "Mrays/s (closest hit)", "unit": "Mrays/s", "value": res["fov120"]["mrays_s"], "roofline": roof,
            "config": {"workload": "views city: %d facade sensors, %d triangles, 3 target groups; fov 120 / 2 deg (3600 rays), fov 360 / 2 deg "
                                   "(10800 rays, isovist volume, reach 6/20/50), jitter on" % (nc, len(city["tri"]))},
            "fov120": res["fov120"], "fov360": res["fov360"], "meshes": meshes, "bvh_build_s": build_s, "bvh": "device LBVH + treelet restructuring",
            "host_sah_tree": host_tree}
    e.close()
    return line


# ---------------------------------------------------------------------------------------------- serving: a mixed request stream
def serving_requests(pkg, scenes, rate, window, seed=5):
    """A seeded Poisson stream: 70 % daylight (sensors log-uniform 100..200k, sky density 145 / 577 / 2305 patches, time
    range log-uniform 1 h .. 1 year -> its sun-up hours as sun directions, radiation + sun hours), 30 % views (fov 120
    or 360 at 2 degree cells, sensors log-uniform 1k..50k); scenes uniform over the resident four."""
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    dirs = {mf: pkg.workloads.patch_dirs(mf) for mf in (1, 2, 4)}
    while True:
        t += rng.exponential(1.0 / rate)
        if t > window:
            break
        sc = int(rng.integers(0, len(scenes)))
        s = scenes[sc]
        if rng.random() < 0.7:
            n = int(min(len(s["P"]), np.exp(rng.uniform(np.log(100), np.log(200_000)))))
            mf = int(rng.choice([1, 2, 4]))
            hours = float(np.exp(rng.uniform(0, np.log(8760))))
            nSun = max(0, int(hours * 0.5))
            Dsky, om = dirs[mf]
            sun = pkg.workloads.hemisphere_dirs(1, nSun, int(rng.integers(1 << 30)))[2:] if nSun else np.zeros((0, 3), np.float32)
            D = np.concatenate([Dsky, -Dsky, sun]).astype(np.float32)
            W = np.zeros((2, len(D)), np.float32)
            W[0, :2 * len(Dsky)] = np.concatenate([om, om]) * 0.1
            W[0, 2 * len(Dsky):] = 0.8
            W[1, 2 * len(Dsky):] = 1.0
            first = int(rng.integers(0, len(s["P"]) - n + 1))
            out.append(dict(t=t, kind="daylight", scene=sc, P=s["P"][first:first + n], N=s["N"][first:first + n], D=D, W=W, use_cos=[True, False]))
        else:
            n = int(min(len(s["P"]), np.exp(rng.uniform(np.log(1000), np.log(50_000)))))
            fov = float(rng.choice([120.0, 360.0]))
            first = int(rng.integers(0, len(s["P"]) - n + 1))
            out.append(dict(t=t, kind="views", scene=sc, P=s["P"][first:first + n], N=s["N"][first:first + n], fov=fov))
    return out


def run_serving(args, pkg):
    import torch
    torch.cuda.set_device(0)
    lib = pkg.load()
    kgb = pkg.kgb
    sizes = [500_000, 1_000_000, 2_000_000, 5_000_000]
    scenes = [pkg.workloads.views_city(seed=10 + k, n_buildings=max(2000, n // 100), target_tris=n, n_sensors=60_000) for k, n in enumerate(sizes)]
    srv = kgb.Server(lib, 150e9)
    ids = [srv.add_scene(s["v"], s["tri"]) for s in scenes]
    srv.autotune()
    if args.old_seconds:
        srv.set_priority(args.old_seconds)
    reqs = serving_requests(pkg, scenes, args.rate, args.window)
    grids = {fov: pkg.workloads.views_grid(fov, 2.0) for fov in (120.0, 360.0)}
    t0 = time.perf_counter()
    tickets = []
    for r in reqs:
        dt = r["t"] - (time.perf_counter() - t0)
        if dt > 0:
            time.sleep(dt)
        if r["kind"] == "daylight":
            tickets.append(srv.submit(ids[r["scene"]], r["P"], r["N"], r["D"], r["W"], r["use_cos"]))
        else:
            nAz, nEl, dAz, rowSin, wRow = grids[r["fov"]]
            world = r["fov"] == 360.0
            tickets.append(srv.submit_views(ids[r["scene"]], r["P"], r["N"], nAz, nEl, 0.0 if world else -r["fov"] / 2, dAz, rowSin, wRow, 6,
                                            1000.0, reach=[6.0, 20.0, 50.0] if world else [], isoDim=3 if world else 0, label=scenes[r["scene"]]["label"],
                                            world=world, cull=world, groundZ=scenes[r["scene"]]["groundZ"]))
    for t in tickets:
        srv.wait(t, 240)
    wall = time.perf_counter() - t0
    st = srv.stats()
    tm = srv.timing()
    tuning = srv.tuning()
    srv.close()
    sensors = sum(len(r["P"]) for r in reqs)
    # the plain form: one request per launch, FIFO, through the single-request entry points (scenes parked and attached)
    e = pkg.engine()
    parked = []
    for s in scenes:
        e.build(s["v"], s["tri"])
        parked.append(e.detach())
    service = []
    cur = None
    for r in reqs:
        t1 = time.perf_counter()
        if cur != r["scene"]:
            if cur is not None:
                parked[cur] = e.detach()
            e.attach(parked[r["scene"]])
            cur = r["scene"]
        if r["kind"] == "daylight":
            e.set_scene(r["P"], r["N"], r["D"])
            e.trace(0, len(r["P"]), lib.ray_flags(False, False))
            for q, c in enumerate(r["use_cos"]):
                e.reduce(len(r["P"]), r["W"][q], c)
        else:
            nAz, nEl, dAz, rowSin, wRow = grids[r["fov"]]
            world = r["fov"] == 360.0
            e.set_labels(scenes[r["scene"]]["label"])
            e.set_scene(r["P"], r["N"], np.zeros((0, 3), np.float32))
            e.view(0, len(r["P"]), lib.bounce_flags(False), nAz, nEl, 0.0 if world else -r["fov"] / 2, dAz, rowSin, world=world, cull=world,
                   groundZ=scenes[r["scene"]]["groundZ"])
            e.reduce_view(len(r["P"]), wRow, 6, 1000.0, reach=[6.0, 20.0, 50.0] if world else [], isoDim=3 if world else 0)
        service.append(time.perf_counter() - t1)
    done, lat = 0.0, []
    for r, sv in zip(reqs, service):
        done = max(done, r["t"]) + sv
        lat.append(done - r["t"])
    base_wall = done
    e.close()
    line = {"metric": "solves/s", "unit": "sensor solves/s", "value": sensors / wall, "p50_ms": 1e3 * st["p50_s"], "p99_ms": 1e3 * st["p99_s"],
            "plain_one_request_per_launch": {"solves_s": sensors / base_wall, "p50_ms": 1e3 * float(np.percentile(lat, 50)),
                                             "p99_ms": 1e3 * float(np.percentile(lat, 99))},
            "config": {"workload": "serving: Poisson %.0f req/s for %.1f s (%d requests: %d daylight, %d views), 4 resident scenes of %s triangles, "
                                   "150 GB HBM budget" % (args.rate, args.window, len(reqs), sum(r["kind"] == "daylight" for r in reqs),
                                                         sum(r["kind"] == "views" for r in reqs), "/".join("%.1fM" % (len(s["tri"]) / 1e6) for s in scenes))},
            "server": dict({k: st[k] for k in ("completed", "items", "rays")}, **tuning), "wall_s": wall,
            "gpu": {"daylight_s": tm["day_gpu_s"], "daylight_mrays_s": tm["day_rays"] / max(tm["day_gpu_s"], 1e-9) / 1e6, "views_s": tm["views_gpu_s"],
                    "views_mrays_s": tm["views_rays"] / max(tm["views_gpu_s"], 1e-9) / 1e6, "queued_s": tm["queued_s"]}}
    return line


# ---------------------------------------------------------------------------------------------- serving: time series
def run_serving_series(args, pkg):
    """The serving form of the time series: daylight requests with hourly time series at 2305 patches + ground (the precision
    configuration's sky, opaque scene: the serving form traces visibility bits) through the server, each batch's series
    chunks of every request in it as one grouped split-BF16 tensor-core launch, against the plain FP32 form one request
    per launch (trace, the ground reduce, kgb_series in its FP32 form) on the same GPU. Requests: seeded, sensors
    log-uniform 1k..50k (contiguous ranges of the urban block), time ranges log-uniform 1 day .. 1 year, all submitted
    at once (throughput); solves = sensors x series columns."""
    import torch
    torch.cuda.set_device(0)
    kgb, lib = pkg.kgb, pkg.load()
    mf = 4
    e = pkg.engine()
    Dsky, omega = pkg.workloads.patch_dirs(mf)
    w = np.load(os.path.join(GOLDEN, "urban_sky", "weather.npy"))
    yr = pkg.workloads.urban_year_sky(e, mf, w)
    col = (w[0] + w[1]) > 1e-4
    colOf = np.cumsum(col) - 1
    sun = e.sun_noaa(np.stack([np.full(8760, 52.52), np.full(8760, 13.41), np.full(8760, 1.0), np.repeat(np.arange(1, 13), [24 * d for d in
                                [31, 28, 31, 30, 31, 30, 31, 31, 30, 31, 30, 31]]),
                               np.concatenate([np.repeat(np.arange(1, d + 1), 24) for d in [31, 28, 31, 30, 31, 30, 31, 31, 30, 31, 30, 31]]),
                               np.tile(np.arange(24) + 0.5, 365), np.zeros(8760)], axis=1))
    scene = pkg.workloads.urban_block()
    P = len(Dsky)
    rng = np.random.default_rng(args.series_seed)
    reqs = []
    for k in range(args.series_requests):
        n = int(np.exp(rng.uniform(np.log(1000), np.log(50000))))
        first = int(rng.integers(0, len(scene["P"]) - n))
        days = float(np.exp(rng.uniform(0, np.log(365))))
        h0 = int(rng.integers(0, 8760 - int(days * 24) + 1))
        hrs = np.arange(h0, h0 + max(1, int(days * 24)))
        hcols = hrs[col[hrs]]
        if not len(hcols):
            continue
        cols = colOf[hcols]
        ups = hrs[(sun[hrs, 2] > 0) & col[hrs]]
        sunVec = sun[ups, 3:6].astype(np.float32)
        D = np.concatenate([Dsky, -Dsky, sunVec]).astype(np.float32)
        Wg = np.zeros(len(D), np.float32)
        Wg[P:2 * P] = omega
        Wr = np.zeros(len(D), np.float32)
        Wr[:P] = omega * 0.1
        Wr[2 * P:] = w[0][ups].astype(np.float32)
        si = dict(nSky=P, row=np.arange(P, dtype=np.int32), wsky=omega, S=np.ascontiguousarray(yr["S"][:, cols]), g=np.ascontiguousarray(yr["g"][cols]),
                  sun0=2 * P, sunStep=(colOf[ups] - cols[0]).astype(np.int32), sunVec=sunVec, sunW=w[0][ups].astype(np.float32))
        reqs.append(dict(P=scene["P"][first:first + n], N=scene["N"][first:first + n], D=D, W=np.stack([Wg, Wr]), si=si))
    solves = sum(len(r["P"]) * r["si"]["S"].shape[1] for r in reqs)
    # the server: every request submitted at once
    srv = kgb.Server(lib, 150e9)
    sid = srv.add_scene(scene["v"], scene["tri"])
    srv.autotune()
    t0 = time.perf_counter()
    tickets = [srv.submit_series(sid, r["P"], r["N"], r["D"], r["W"], [True, True], 0, **r["si"]) for r in reqs]
    for t in tickets:
        srv.wait(t, 600)
    wall = time.perf_counter() - t0
    st, tm = srv.stats(), srv.timing()
    srv.close()
    # the plain FP32 form: one request after another through the single-request entry points
    e.build(scene["v"], scene["tri"])
    e.set_series_form(1)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for r in reqs:
        e.set_scene(r["P"], r["N"], r["D"])
        e.trace(0, len(r["P"]), lib.ray_flags(False, False))
        G = e.reduce(len(r["P"]), r["W"][0], True)
        e.reduce(len(r["P"]), r["W"][1], True)
        e.series(len(r["P"]), G=G.astype(np.float32), **r["si"])
    plain = time.perf_counter() - t0
    e.set_series_form(0)
    e.close()
    return {"metric": "radiation solves/s (time series, serving)", "unit": "sensor-steps/s", "value": solves / wall,
            "plain_fp32_one_request_per_launch": solves / plain, "speedup_vs_plain_fp32": plain / wall,
            "p50_ms": 1e3 * st["p50_s"], "p99_ms": 1e3 * st["p99_s"], "wall_s": wall, "plain_s": plain,
            "gpu": {"daylight_s": tm["day_gpu_s"], "queued_s": tm["queued_s"]}, "server": {k: st[k] for k in ("completed", "items", "chunk_sensors", "batch_rays")},
            "config": {"workload": "%d daylight requests with hourly series on the urban block (%d triangles): 2305 patches + ground, sensors "
                                   "log-uniform 1k..50k (%d in all), time ranges log-uniform 1 day..1 year (%d series columns in all), "
                                   "submitted at once" % (len(reqs), len(scene["tri"]), sum(len(r["P"]) for r in reqs),
                                                         sum(r["si"]["S"].shape[1] for r in reqs)),
                       "solves": solves},
            "dtype": "series: split-bf16 on tcgen05 (server) vs fp32 SIMT (plain form)"}


# ---------------------------------------------------------------------------------------------- .dmesh ingest
def dmesh_grid(n):
    """The reference's ingest benchmark mesh (validate/ingest.py: an n x n quad grid, (n + 1)^2 points), as a .dmesh
    image with a slot per face."""
    xs, ys = np.meshgrid(np.arange(n + 1, dtype=np.float64), np.arange(n + 1, dtype=np.float64), indexing="ij")
    P = np.stack([xs.ravel(), ys.ravel(), 0.01 * np.sin(xs.ravel()) * np.cos(ys.ravel())], 1)
    q = np.arange(n * (n + 1)).reshape(n, n + 1)[:, :n].ravel()
    I = np.stack([q, q + n + 1, q + n + 2, q + 1], 1).astype(np.int32).ravel()
    C = np.full(n * n, 4, np.int32)
    S = (np.arange(n * n) % 3).astype(np.uint16)
    head = b"DLM1" + np.array([1], np.uint32).tobytes() + np.array([len(P), len(C), len(I)], np.uint64).tobytes()
    return head + P.tobytes() + C.tobytes() + I.tobytes() + S.tobytes()


def run_ingest(args, pkg):
    """A 1000 x 1000 quad grid (2M triangles) as a .dmesh file in the page cache: read to the device and checked there
    (kgb_mesh_file), then the scene built from it on the device (kgb_build_meshes: triangulation + BVH); beside it the
    oracle's restatement of the reference's read_dmesh (whole file into host memory, arrays copied out, checked) on
    one host core. Wall-clock seconds, median of the repeats."""
    import tempfile
    img = dmesh_grid(1000)
    d = tempfile.mkdtemp(prefix="kgb_ingest_")
    path = os.path.join(d, "grid.dmesh")
    with open(path, "wb") as f:
        f.write(img)
    with open(path, "rb") as f:   # in the page cache, as a file just written or read before
        f.read()
    reps = max(3, args.steps)
    e = pkg.engine()
    try:
        for _ in range(2):
            e.mesh_free(e.mesh_file(path).id)
        t_read, t_mem, t_build = [], [], []
        for _ in range(reps):
            t0 = time.perf_counter()
            info = e.mesh_file(path)
            t_read.append(time.perf_counter() - t0)
            t0 = time.perf_counter()
            made, skipped = e.build_meshes([info.id], [(info.lo[a] + info.hi[a]) / 2 for a in range(3)])
            t_build.append(time.perf_counter() - t0)
            e.mesh_free(info.id)
            t0 = time.perf_counter()
            e.mesh_free(e.mesh_read(img, "grid").id)
            t_mem.append(time.perf_counter() - t0)
        tris = int(made.sum())
    finally:
        e.close()
    o = pkg.kgb.Engine(oracle_lib(pkg))
    try:
        t_cpu = []
        for _ in range(reps):
            t0 = time.perf_counter()
            o.mesh_free(o.mesh_file(path).id)
            t_cpu.append(time.perf_counter() - t0)
    finally:
        o.close()
    os.remove(path)
    os.rmdir(d)
    med = lambda x: float(np.median(x))
    return {"metric": "s per .dmesh read", "unit": "s", "higher_is_better": False, "value": med(t_read),
            "config": {"workload": "1000 x 1000 quad grid: 1,002,001 points, 1,000,000 quads with slots, %d bytes, page cache warm" % len(img),
                       "repeats": reps},
            "from_memory_s": med(t_mem), "build_scene_s": med(t_build), "triangles": tris, "skipped": skipped,
            "cpu_baseline": {"value": med(t_cpu), "unit": "s", "cores": 1, "kind": "port",
                             "sample": "the oracle's restatement of read_dmesh (src/mesh.cpp:480-489) on the same file"},
            "read_gb_per_s": len(img) / med(t_read) / 1e9}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-sample", type=int, default=30000)
    ap.add_argument("--ref-sample", type=int, default=20000)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--sensors", type=int, default=0, help="urban / precision / views: only the first N sensors (a small case for profiling)")
    ap.add_argument("--config", default="urban", choices=["urban", "precision", "views", "serving", "serving_series", "ingest"])
    ap.add_argument("--series-requests", type=int, default=64)
    ap.add_argument("--series-seed", type=int, default=12)
    ap.add_argument("--builder", type=int, default=1, choices=[0, 1], help="urban: 1 device LBVH with treelets (default), 0 host binned-SAH tree")
    ap.add_argument("--rate", type=float, default=200.0)
    ap.add_argument("--old-seconds", type=float, default=0.0, help="serving: the scheduler's wait past which requests go in arrival order")
    ap.add_argument("--window", type=float, default=2.0)
    ap.add_argument("--full-fp32", action="store_true")
    ap.add_argument("--accuracy-sensors", type=int, default=1024, help="precision: sensors of the FP64 accuracy check")
    ap.add_argument("--no-extras", action="store_true", help="urban: leave out the precision, views and serving keys")
    args = ap.parse_args()
    pkg = package()
    if args.config == "precision":
        print(json.dumps(run_precision(args, pkg)), flush=True)
    elif args.config == "views":
        print(json.dumps(run_views(args, pkg)), flush=True)
    elif args.config == "serving":
        print(json.dumps(run_serving(args, pkg)), flush=True)
    elif args.config == "serving_series":
        print(json.dumps(run_serving_series(args, pkg)), flush=True)
    elif args.config == "ingest":
        print(json.dumps(run_ingest(args, pkg)), flush=True)
    elif args.impl == "reference":
        run_reference(args, pkg)
    else:
        run_ours(args, pkg)


if __name__ == "__main__":
    main()
