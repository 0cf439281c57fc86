// The reference's GPU contract (kit-sim_daylight src/internal.h:125-220, the functions src/gpu.cu implements over
// OptiX) implemented over the GB300 engine's C ABI (include/kitsim_gb300.h). Compiled into the reference's
// daylightcore in place of src/gpu.cu + src/trace_dev.cu, it makes daylight::run, daylight::views::run, the C ABI
// (daylight_c.h: DL_DAYLIGHT / DL_VIEWS) and every binding run on the engine unchanged.
//
// Recorder: with KGB_RECORD=<dir> in the environment, every call is written to <dir>/calls.jsonl with its arrays
// (inputs and the results it returned) as raw little-endian files beside it, so that a run of the reference's host
// code can be replayed at this boundary (tests/golden/ holds such recordings).
#include "internal.h"
#include "kitsim_gb300.h"

#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace daylight {

static_assert(sizeof(Slot) == sizeof(kgb_slot), "Slot and kgb_slot share a layout (src/params.h:7-12)");
static_assert(sizeof(float3) == 12 && sizeof(uint3) == 12, "float3 / uint3 are three packed 32-bit values");

struct Gpu {
  kgb_engine* e = nullptr;
};

namespace {

// ------------------------------------------------------------------------------------------- recorder (KGB_RECORD)
struct Recorder {
  std::string dir;
  std::FILE* log = nullptr;
  unsigned seq = 0;
  std::string line;
  Recorder() {
    if (const char* d = std::getenv("KGB_RECORD")) {
      dir = d;
      log = std::fopen((dir + "/calls.jsonl").c_str(), "w");
    }
  }
  ~Recorder() { if (log) std::fclose(log); }
  bool on() const { return log != nullptr; }
  void begin(const char* call) { line = "{\"seq\": " + std::to_string(seq) + ", \"call\": \"" + call + "\""; }
  void num(const char* k, double v) {
    char b[64];
    std::snprintf(b, sizeof b, "%.17g", v);
    line += std::string(", \"") + k + "\": " + b;
  }
  void arr(const char* k, const char* dtype, const void* p, size_t bytes, size_t n0, size_t n1 = 0) {
    char name[64];
    std::snprintf(name, sizeof name, "%06u_%s.bin", seq, k);
    if (std::FILE* f = std::fopen((dir + "/" + name).c_str(), "wb")) {
      if (bytes) std::fwrite(p, 1, bytes, f);
      std::fclose(f);
    }
    line += std::string(", \"") + k + "\": [\"" + dtype + "\", [" + std::to_string(n0) + (n1 ? ", " + std::to_string(n1) : "") + "], \"" + name + "\"]";
  }
  void end(bool ok) {
    line += std::string(", \"ok\": ") + (ok ? "true" : "false") + "}\n";
    std::fputs(line.c_str(), log);
    std::fflush(log);
    ++seq;
  }
};
Recorder& rec() { static Recorder r; return r; }

int cancelled(void* ctx) { return static_cast<const std::atomic<bool>*>(ctx)->load() ? 1 : 0; }

bool ok(int r, std::string& err) {
  if (!r) err = kgb_last_error();
  return r != 0;
}
void dims(const Gpu& g, uint64_t d[6]) { kgb_dims(g.e, d); }

}  // namespace

Gpu* gpu_init(std::string& err) {
  kgb_engine* e = kgb_init();
  if (!e) { err = kgb_last_error(); return nullptr; }
  return new Gpu{e};
}

void gpu_destroy(Gpu* g) {
  if (!g) return;
  kgb_destroy(g->e);
  delete g;
}

bool gpu_build(Gpu& g, const Tris& t, const std::vector<Slot>& slots, std::string& err, bool perSlot) {
  Recorder& R = rec();
  const bool r = ok(kgb_build(g.e, t.v.empty() ? nullptr : &t.v[0].x, t.v.size(), t.i.empty() ? nullptr : &t.i[0].x, t.i.size(),
                              t.slot.empty() ? nullptr : t.slot.data(), reinterpret_cast<const kgb_slot*>(slots.data()), slots.size(), perSlot ? 1 : 0),
                    err);
  if (R.on()) {
    R.begin("gpu_build");
    R.arr("v", "<f4", t.v.data(), t.v.size() * 12, t.v.size(), 3);
    R.arr("tri", "<u4", t.i.data(), t.i.size() * 12, t.i.size(), 3);
    R.arr("slot", "<u4", t.slot.data(), t.slot.size() * 4, t.slot.size());
    R.arr("slots", "<f4", slots.data(), slots.size() * 16, slots.size(), 4);
    R.num("perSlot", perSlot);
    R.end(r);
  }
  return r;
}

size_t gpu_build_bytes(Gpu& g, size_t nVerts, size_t nTris, bool slotted, std::string& err) {
  const uint64_t b = kgb_build_bytes(g.e, nVerts, nTris, slotted ? 1 : 0);
  if (b == UINT64_MAX) { err = kgb_last_error(); return SIZE_MAX; }
  return size_t(b);
}

void gpu_trim(Gpu& g, bool sensors) { kgb_trim(g.e, sensors ? 1 : 0); }

bool gpu_set_slots(Gpu& g, const std::vector<Slot>& slots, std::string& err) {
  Recorder& R = rec();
  const bool r = ok(kgb_set_slots(g.e, reinterpret_cast<const kgb_slot*>(slots.data()), slots.size()), err);
  if (R.on()) { R.begin("gpu_set_slots"); R.arr("slots", "<f4", slots.data(), slots.size() * 16, slots.size(), 4); R.end(r); }
  return r;
}

GasSlot gpu_detach(Gpu& g) {
  const kgb_scene s = kgb_detach(g.e);
  return GasSlot{s.handle, 0ull, size_t(s.bytes)};
}
void gpu_attach(Gpu& g, GasSlot s) { kgb_attach(g.e, kgb_scene{s.dGas, uint64_t(s.bytes)}); }
void gpu_free(GasSlot& s) {
  kgb_scene k{s.dGas, uint64_t(s.bytes)};
  kgb_free_scene(&k);
  s = GasSlot{};
}
size_t gpu_free_bytes() { return size_t(kgb_free_bytes()); }

bool gpu_set_scene(Gpu& g, const Sensors& s, const std::vector<float3>& dirs, std::string& err) {
  Recorder& R = rec();
  const bool r = ok(kgb_set_scene(g.e, s.p.empty() ? nullptr : &s.p[0].x, s.n.empty() ? nullptr : &s.n[0].x, s.p.size(),
                                  dirs.empty() ? nullptr : &dirs[0].x, dirs.size()),
                    err);
  if (R.on()) {
    R.begin("gpu_set_scene");
    R.arr("P", "<f4", s.p.data(), s.p.size() * 12, s.p.size(), 3);
    R.arr("N", "<f4", s.n.data(), s.n.size() * 12, s.n.size(), 3);
    R.arr("D", "<f4", dirs.data(), dirs.size() * 12, dirs.size(), 3);
    R.end(r);
  }
  return r;
}

bool gpu_trace(Gpu& g, size_t i0, size_t nc, unsigned rayFlags, std::string& err) {
  Recorder& R = rec();
  const bool r = ok(kgb_trace(g.e, i0, nc, rayFlags), err);
  if (R.on()) {
    R.begin("gpu_trace");
    R.num("i0", double(i0)); R.num("nc", double(nc)); R.num("rayFlags", rayFlags);
    uint64_t d[6];
    dims(g, d);
    if (r && nc) {   // the visibility it left on the device
      if (d[5]) { std::vector<uint8_t> b(d[1] * nc); kgb_download_bytes(g.e, nc, b.data(), b.size()); R.arr("bytes", "<u1", b.data(), b.size(), d[1], nc); }
      else { std::vector<uint32_t> b(d[2] * nc); kgb_download_bits(g.e, nc, b.data(), b.size()); R.arr("bits", "<u4", b.data(), b.size() * 4, d[2], nc); }
    }
    R.end(r);
  }
  return r;
}

bool gpu_reduce(Gpu& g, size_t nc, const float* W, bool useCos, double* out, std::string& err) {
  Recorder& R = rec();
  const bool r = ok(kgb_reduce(g.e, nc, W, useCos ? 1 : 0, out), err);
  if (R.on()) {
    uint64_t d[6];
    dims(g, d);
    R.begin("gpu_reduce");
    R.num("nc", double(nc)); R.num("useCos", useCos);
    R.arr("W", "<f4", W, d[1] * 4, d[1]);
    R.arr("out", "<f8", out, nc * 8, nc);
    R.end(r);
  }
  return r;
}

bool gpu_series(Gpu& g, size_t nc, const SeriesIn& in, float* E, std::string& err) {
  kgb_series_in k;
  k.nSky = in.nSky; k.row = in.row; k.wsky = in.wsky; k.S = in.S; k.P = in.P; k.T = in.T; k.g = in.g; k.G = in.G;
  k.sun0 = in.sun0; k.nSun = in.nSun; k.sunStep = in.sunStep; k.sunVec = in.sunVec ? &in.sunVec[0].x : nullptr; k.sunW = in.sunW; k.Sdc = in.Sdc;
  Recorder& R = rec();
  const bool r = ok(kgb_series(g.e, nc, &k, E), err);
  if (R.on()) {
    uint64_t d[6];
    dims(g, d);
    const size_t T = in.T > 0 ? size_t(in.T) : 0;
    R.begin("gpu_series");
    R.num("nc", double(nc)); R.num("nSky", in.nSky); R.num("P", in.P); R.num("T", in.T); R.num("sun0", in.sun0); R.num("nSun", in.nSun);
    R.arr("row", "<i4", in.row, in.nSky * 4, in.nSky);
    R.arr("wsky", "<f4", in.wsky, in.nSky * 4, in.nSky);
    R.arr("S", "<f4", in.S, size_t(in.P) * T * 4, size_t(in.P), T);
    R.arr("g", "<f4", in.g, T * 4, T);
    R.arr("G", "<f4", in.G, nc * 4, nc);
    R.arr("sunStep", "<i4", in.sunStep, in.nSun * 4, in.nSun);
    R.arr("sunVec", "<f4", in.sunVec, in.nSun * 12, in.nSun, 3);
    R.arr("sunW", "<f4", in.sunW, in.nSun * 4, in.nSun);
    if (in.Sdc) R.arr("Sdc", "<f4", in.Sdc, d[3] * T * 4, d[3], T);
    R.arr("E", "<f4", E, nc * T * 4, nc, T);
    R.end(r);
  }
  return r;
}

bool gpu_bounce(Gpu& g, size_t i0, size_t nc, unsigned rayFlags, const Bounce& b, std::string& err) {
  kgb_bounce_in k;
  k.N = b.N; k.M = b.M; k.mf = b.mf; k.north = b.north;
  k.cancel = b.cancel ? cancelled : nullptr;
  k.cancelCtx = const_cast<std::atomic<bool>*>(b.cancel);
  Recorder& R = rec();
  const bool r = ok(kgb_bounce(g.e, i0, nc, rayFlags, &k), err);
  if (R.on()) {
    R.begin("gpu_bounce");
    R.num("i0", double(i0)); R.num("nc", double(nc)); R.num("rayFlags", rayFlags);
    R.num("N", b.N); R.num("M", b.M); R.num("mf", b.mf); R.num("north", b.north);
    uint64_t d[6];
    dims(g, d);
    if (r && nc) { std::vector<float> dc(d[3] * nc); kgb_download_dc(g.e, nc, dc.data(), dc.size()); R.arr("dc", "<f4", dc.data(), dc.size() * 4, d[3], nc); }
    R.end(r);
  }
  return r;
}

bool gpu_reduce_dc(Gpu& g, size_t nc, const float* W, double* out, std::string& err) {
  Recorder& R = rec();
  const bool r = ok(kgb_reduce_dc(g.e, nc, W, out), err);
  if (R.on()) {
    uint64_t d[6];
    dims(g, d);
    R.begin("gpu_reduce_dc");
    R.num("nc", double(nc));
    R.arr("W", "<f4", W, d[3] * 4, d[3]);
    R.arr("out", "<f8", out, nc * 8, nc);
    R.end(r);
  }
  return r;
}

bool gpu_download_dc(Gpu& g, size_t nc, std::vector<float>& out, std::string& err) {
  uint64_t d[6];
  dims(g, d);
  out.resize(d[3] * nc);
  return ok(kgb_download_dc(g.e, nc, out.data(), out.size()), err);
}

bool gpu_download_bits(Gpu& g, size_t nc, std::vector<uint32_t>& out, std::string& err) {
  uint64_t d[6];
  dims(g, d);
  if (d[5]) { err = "gpu_download_bits: the last trace wrote bytes"; return false; }
  out.resize(d[2] * nc);
  return ok(kgb_download_bits(g.e, nc, out.data(), out.size()), err);
}

bool gpu_download_bytes(Gpu& g, size_t nc, std::vector<uint8_t>& out, std::string& err) {
  uint64_t d[6];
  dims(g, d);
  if (!d[5]) { err = "gpu_download_bytes: the last trace wrote bits"; return false; }
  out.resize(d[1] * nc);
  return ok(kgb_download_bytes(g.e, nc, out.data(), out.size()), err);
}

bool gpu_set_labels(Gpu& g, const std::vector<uint8_t>& label, std::string& err) {
  Recorder& R = rec();
  const bool r = ok(kgb_set_labels(g.e, label.data(), label.size()), err);
  if (R.on()) { R.begin("gpu_set_labels"); R.arr("label", "<u1", label.data(), label.size(), label.size()); R.end(r); }
  return r;
}

bool gpu_view(Gpu& g, size_t i0, size_t nc, unsigned rayFlags, const ViewLaunch& v, size_t& launch, std::string& err) {
  kgb_view_in k;
  k.nAz = v.nAz; k.nEl = v.nEl; k.az0 = v.az0; k.dAz = v.dAz; k.rowSin = v.rowSin;
  k.world = v.world; k.cull = v.cull; k.jitter = v.jitter; k.back = v.back; k.vground = v.vground;
  k.nS = v.nS; k.groundZ = v.groundZ; k.north = v.north;
  k.cancel = v.cancel ? cancelled : nullptr;
  k.cancelCtx = const_cast<std::atomic<bool>*>(v.cancel);
  Recorder& R = rec();
  const size_t launch0 = launch;
  const bool r = ok(kgb_view(g.e, i0, nc, rayFlags, &k, &launch), err);
  if (R.on()) {
    R.begin("gpu_view");
    R.num("i0", double(i0)); R.num("nc", double(nc)); R.num("rayFlags", rayFlags); R.num("launch", double(launch0));
    R.num("nAz", v.nAz); R.num("nEl", v.nEl); R.num("az0", v.az0); R.num("dAz", v.dAz);
    R.num("world", v.world); R.num("cull", v.cull); R.num("jitter", v.jitter); R.num("back", v.back); R.num("vground", v.vground);
    R.num("nS", v.nS); R.num("groundZ", v.groundZ); R.num("north", v.north);
    R.arr("rowSin", "<f4", v.rowSin, size_t(v.nEl) * 8, v.nEl, 2);
    const size_t K = size_t(v.nAz) * v.nEl;
    if (r && nc && K) {
      std::vector<uint8_t> c(nc * K);
      std::vector<float> t(nc * K);
      kgb_download_view(g.e, nc, c.data(), t.data(), c.size());
      R.arr("cls", "<u1", c.data(), c.size(), nc, K);
      R.arr("dist", "<f4", t.data(), t.size() * 4, nc, K);
    }
    R.end(r);
  }
  return r;
}

bool gpu_reduce_view(Gpu& g, size_t nc, const std::vector<double>& wRow, unsigned nClass, double farDist, const std::vector<float>& reach,
                     bool glazing, unsigned isoDim, double* out, std::string& err) {
  Recorder& R = rec();
  const bool r = ok(kgb_reduce_view(g.e, nc, wRow.data(), wRow.size(), nClass, farDist, reach.data(), reach.size(), glazing ? 1 : 0, isoDim, out), err);
  if (R.on()) {
    const size_t NA = 3 * size_t(nClass) + 1 + reach.size() + (glazing ? 1 : 0) + (isoDim ? 1 : 0);
    R.begin("gpu_reduce_view");
    R.num("nc", double(nc)); R.num("nClass", nClass); R.num("farDist", farDist); R.num("glazing", glazing); R.num("isoDim", isoDim);
    R.arr("wRow", "<f8", wRow.data(), wRow.size() * 8, wRow.size());
    R.arr("reach", "<f4", reach.data(), reach.size() * 4, reach.size());
    R.arr("out", "<f8", out, nc * NA * 8, nc, NA);
    R.end(r);
  }
  return r;
}

bool gpu_download_view(Gpu& g, size_t nc, std::vector<uint8_t>& cls, std::vector<float>& dist, std::string& err) {
  uint64_t d[6];
  dims(g, d);
  cls.resize(nc * d[4]);
  dist.resize(nc * d[4]);
  return ok(kgb_download_view(g.e, nc, cls.data(), dist.data(), cls.size()), err);
}

GpuStats gpu_stats(const Gpu& g) {
  const kgb_stats s = kgb_get_stats(g.e);
  GpuStats o;
  o.buildMs = s.buildMs; o.traceMs = s.traceMs; o.bounceMs = s.bounceMs;
  o.rays = size_t(s.rays); o.gasBytes = size_t(s.gasBytes); o.launches = size_t(s.launches); o.paths = size_t(s.paths);
  o.bounceLaunches = size_t(s.bounceLaunches); o.buildTempBytes = size_t(s.buildTempBytes); o.buildOutputBytes = size_t(s.buildOutputBytes);
  return o;
}

unsigned gpu_ray_flags(bool cullBackfaces, bool translucent) { return kgb_ray_flags(cullBackfaces ? 1 : 0, translucent ? 1 : 0); }
unsigned gpu_bounce_flags(bool cullBackfaces) { return kgb_bounce_flags(cullBackfaces ? 1 : 0); }

}  // namespace daylight
