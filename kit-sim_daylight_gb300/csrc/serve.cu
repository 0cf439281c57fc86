// The serving loop: device-resident scenes, and daylight / views requests of any size admitted against an HBM budget
// and run with continuous batching. A request is cut into chunks of sensors. Every iteration of the server thread
// admits what the budget allows, then packs chunks of the admitted requests (round robin, so a short request is not held
// behind a long one) into one batch:
//  - daylight chunks: ONE persistent any-hit launch over every chunk of the batch (k_bits_batch: tasks of 32 sensors x
//    one 32-direction word, each task finds its chunk in the batch's segment table) and ONE reduce launch giving every
//    quantity of every chunk (k_reduce_batch). The batch's pipeline (segment table up, counter reset, the two kernels,
//    the sums down) is a CUDA graph captured once and replayed per batch: its pointers never change, the table does;
//  - views chunks: the view kernels (k_view, k_view_reduce, k_iso) on each chunk, between the daylight batches.
// A request completes when its last chunk has; its results are bit-identical to the request run alone through the
// single-request entry points (same kernels, same per-sensor arithmetic and summation order).
//
// The autotuner times calibration batches on the first scene at start-up and keeps the fastest chunk size and batch
// size (rays per batch) for the daylight pipeline.
#include "engine.h"
#include "rt.cuh"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

namespace kgb {

constexpr uint32_t kMaxSegs = 256;
constexpr uint32_t kMaxQ = 8;

struct __align__(16) Seg {
  const Node8* nodes;
  const TriRec* tris;
  const float* P;      // the chunk's first sensor
  const float* N;
  const float* D;
  const RayDir* tab;   // the directions' precomputed ray parts
  const double* W;     // [nQ x nDir], the request's float weights widened
  uint32_t nNodes, nDir, nWords, n;
  uint32_t rayFlags, nQ, useCosMask, taskBase;
  uint32_t sensBase, bitsOff, outOff, pad;
};
struct __align__(16) BatchHdr {
  uint32_t nSegs, nTasks, nSens, pad;
};

__device__ __forceinline__ uint32_t find_seg(const Seg* segs, uint32_t nSegs, uint32_t key, bool bySensor) {
  uint32_t lo = 0, hi = nSegs - 1;
  while (lo < hi) {
    const uint32_t mid = (lo + hi + 1) / 2;
    const uint32_t base = bySensor ? segs[mid].sensBase : segs[mid].taskBase;
    if (base <= key) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__global__ void __launch_bounds__(256) k_bits_batch(const BatchHdr* hdr, const Seg* segs, uint32_t* bitsPool, uint32_t* counter, uint32_t* status) {
  const uint32_t nSegs = hdr->nSegs, nTasks = hdr->nTasks;
  const uint32_t lane = threadIdx.x & 31;
  uint32_t overflow = 0, rays = 0;
  Count ctr;
  for (;;) {
    uint32_t task = 0;
    if (lane == 0) task = atomicAdd(counter, 1u);
    task = __shfl_sync(~0u, task, 0);
    if (task >= nTasks) break;
    const Seg& g = segs[find_seg(segs, nSegs, task, false)];
    const uint32_t local = task - g.taskBase, b = local / g.nWords, w = local % g.nWords, i = b * 32 + lane;
    if (i >= g.n) continue;
    const Scene s{g.nodes, g.tris, g.nNodes};
    const F3 n = ld3(g.N + 3 * i), o = offset_ray(ld3(g.P + 3 * i), n);
    const uint32_t word = trace_word<false>(s, n, o, g.D, g.tab, g.nDir, w, (g.rayFlags & KGB_RAY_CULL_BACK_FACING) != 0, overflow, ctr, rays);
    bitsPool[g.bitsOff + size_t(w) * g.n + i] = word;
  }
  if (overflow) atomicOr(status, (overflow & 1u ? kStatusStackOverflow : 0u) | (overflow & 2u ? kStatusVisitLimit : 0u));
}

// every quantity of every chunk: out[outOff + q n + i] = sum over visible d, in order, of
// double(float(useCos_q ? max(0, N_i . D_d) : 1)) x W_q[d] (the single-request reduce's arithmetic, per quantity:
// one fma per term, the float factor widened exactly, a zero factor skipped)
__global__ void __launch_bounds__(256) k_reduce_batch(const BatchHdr* hdr, const Seg* segs, const uint32_t* bitsPool, double* outPool) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= hdr->nSens) return;
  const Seg& g = segs[find_seg(segs, hdr->nSegs, t, true)];
  const uint32_t i = t - g.sensBase;
  const F3 n = ld3(g.N + 3 * i);
  double acc[kMaxQ];
#pragma unroll
  for (uint32_t q = 0; q < kMaxQ; ++q) acc[q] = 0;
  for (uint32_t w = 0; w < g.nWords; ++w) {
    uint32_t m = bitsPool[g.bitsOff + size_t(w) * g.n + i];
    while (m) {
      const uint32_t d = w * 32 + (__ffs(m) - 1);
      m &= m - 1;
      const F3 dir = ld3(g.D + 3 * d);
      const float c = fmaxf(__fadd_rn(__fadd_rn(__fmul_rn(n.x, dir.x), __fmul_rn(n.y, dir.y)), __fmul_rn(n.z, dir.z)), 0.f);
#pragma unroll
      for (uint32_t q = 0; q < kMaxQ; ++q) {
        const float x = ((g.useCosMask >> q) & 1u) ? c : 1.f;
        if (q < g.nQ && x != 0.f) acc[q] = __fma_rn(widen(x), __ldg(g.W + size_t(q) * g.nDir + d), acc[q]);
      }
    }
  }
  for (uint32_t q = 0; q < g.nQ; ++q) outPool[g.outOff + size_t(q) * g.n + i] = acc[q];
}

// ------------------------------------------------------------------------------------------------ host side
namespace {
using Clock = std::chrono::steady_clock;

struct DScene {
  void* nodes = nullptr;
  void* tris = nullptr;
  uint32_t nNodes = 0, nTris = 0;
  uint64_t bytes = 0;
  void* label = nullptr;   // views labels of the last views request on this scene (device, nTris)
};

struct Request {
  uint64_t ticket = 0;
  int kind = 0;   // 0 daylight, 1 views
  kgb_daylight_request d{};
  kgb_views_request v{};
  std::vector<float> rowSin;
  std::vector<double> wRow;
  std::vector<float> reach;
  std::vector<double> w64;    // daylight: the weights widened to double (the source of their upload)
  uint32_t nSensors = 0, nextSensor = 0, doneSensors = 0;
  void* dev = nullptr;        // P, N, D, ray table, W (daylight) | P, N, rowSin, wRow, label, cls, dist, out (views)
  uint64_t devBytes = 0;
  Clock::time_point tSubmit, tDone;
  bool done = false, failed = false;
  std::string err;
};
}  // namespace

struct Server {
  int device = 0, numSMs = 0;
  cudaStream_t st = nullptr;
  uint64_t budget = 0, used = 0;
  std::vector<DScene> scenes;
  // batch pools (fixed for the graph)
  uint32_t chunkSensors = 8192;
  uint64_t batchRays = uint64_t(1) << 30;
  size_t bitsPoolWords = 0, outPoolDoubles = 0;
  uint32_t* dBits = nullptr;
  double* dOut = nullptr;
  double* hOut = nullptr;            // pinned
  Seg* hSegs = nullptr;              // pinned [kMaxSegs]
  BatchHdr* hHdr = nullptr;          // pinned
  Seg* dSegs = nullptr;
  BatchHdr* dHdr = nullptr;
  uint32_t* dCtl = nullptr;          // counter, status
  cudaGraphExec_t graph = nullptr;
  int gridBits = 0;
  uint32_t maxSensPerBatch = 0;
  // requests
  std::mutex m;
  std::condition_variable cv, doneCv;
  std::deque<Request*> pending;
  std::vector<Request*> active;
  std::map<uint64_t, Request*> all;
  uint64_t nextTicket = 1;
  size_t rr = 0;
  bool stop = false;
  std::thread th;
  std::vector<double> latencies;   // seconds, completed requests
  uint64_t batches = 0, rays = 0;
  std::string fatal;
};

namespace {

bool cuok(cudaError_t e, std::string& err, const char* what) {
  if (e == cudaSuccess) return true;
  err = std::string(what) + ": " + cudaGetErrorString(e);
  return false;
}

// a daylight request's device arrays: P, N (12 B per sensor each), D (12 B per direction), its ray table (48 B per
// direction), its weights as doubles [nQ x nDir]; 256-byte aligned pieces
struct DayLayout { size_t offN, offD, offTab, offW, total; };
DayLayout day_layout(const kgb_daylight_request& d) {
  const auto up = [](size_t x) { return (x + 255) & ~size_t(255); };
  DayLayout L;
  L.offN = size_t(d.nSensors) * 12;
  L.offD = up(2 * L.offN);
  L.offTab = up(L.offD + size_t(d.nDir) * 12);
  L.offW = up(L.offTab + size_t(d.nDir) * 48);
  L.total = up(L.offW + size_t(d.nQ) * d.nDir * 8);
  return L;
}

uint64_t daylight_bytes(const kgb_daylight_request& r) { return day_layout(r).total; }
uint32_t views_NA(const kgb_views_request& r) { return 3 * r.nClass + 1 + r.nReach + (r.glazing ? 1 : 0) + (r.isoDim ? 1 : 0); }
uint64_t views_bytes(const kgb_views_request& r, uint32_t chunk, uint32_t nTris) {
  const uint64_t K = uint64_t(r.view.nAz) * r.view.nEl;
  return uint64_t(r.nSensors) * 24 + uint64_t(r.view.nEl) * 16 + (r.label ? nTris : 0) + uint64_t(chunk) * (5 * K + 8 * views_NA(r)) + 4096;
}

// graph of one daylight batch: table up, counter reset, trace, reduce, sums down
bool capture(Server& s, std::string& err) {
  cudaGraph_t gph;
  if (!cuok(cudaStreamBeginCapture(s.st, cudaStreamCaptureModeThreadLocal), err, "capture")) return false;
  cudaMemcpyAsync(s.dHdr, s.hHdr, sizeof(BatchHdr), cudaMemcpyHostToDevice, s.st);
  cudaMemcpyAsync(s.dSegs, s.hSegs, sizeof(Seg) * kMaxSegs, cudaMemcpyHostToDevice, s.st);
  cudaMemsetAsync(s.dCtl, 0, 8, s.st);
  k_bits_batch<<<s.gridBits, 256, 0, s.st>>>(s.dHdr, s.dSegs, s.dBits, s.dCtl, s.dCtl + 1);
  k_reduce_batch<<<(s.maxSensPerBatch + 255) / 256, 256, 0, s.st>>>(s.dHdr, s.dSegs, s.dBits, s.dOut);
  cudaMemcpyAsync(s.hOut, s.dOut, sizeof(double) * s.outPoolDoubles, cudaMemcpyDeviceToHost, s.st);
  if (!cuok(cudaStreamEndCapture(s.st, &gph), err, "capture end")) return false;
  if (s.graph) cudaGraphExecDestroy(s.graph);
  const bool ok = cuok(cudaGraphInstantiate(&s.graph, gph, 0), err, "graph instantiate");
  cudaGraphDestroy(gph);
  return ok;
}

bool make_pools(Server& s, std::string& err) {
  if (s.dBits) { cudaFree(s.dBits); cudaFree(s.dOut); s.used -= s.bitsPoolWords * 4 + s.outPoolDoubles * 8; }
  s.maxSensPerBatch = std::min<uint32_t>(kMaxSegs * s.chunkSensors, 1u << 20);
  // bits of a batch: rays / 32 words, plus a word per sensor and segment for the rounding up of each chunk's words
  s.bitsPoolWords = size_t(s.batchRays / 32) + size_t(s.maxSensPerBatch) * 2;
  s.outPoolDoubles = size_t(s.maxSensPerBatch) * kMaxQ;
  if (!cuok(cudaMalloc(&s.dBits, s.bitsPoolWords * 4), err, "batch pool") || !cuok(cudaMalloc(&s.dOut, s.outPoolDoubles * 8), err, "batch pool"))
    return false;
  s.used += s.bitsPoolWords * 4 + s.outPoolDoubles * 8;
  if (s.hOut) cudaFreeHost(s.hOut);
  if (!cuok(cudaMallocHost(&s.hOut, s.outPoolDoubles * 8), err, "pinned pool")) return false;
  return capture(s, err);
}

void finish(Server& s, Request* r, bool ok, const std::string& err) {
  if (r->dev) cudaFree(r->dev);
  s.used -= r->devBytes;
  r->dev = nullptr;
  r->tDone = Clock::now();
  r->failed = !ok;
  r->err = err;
  r->done = true;
  if (ok) s.latencies.push_back(std::chrono::duration<double>(r->tDone - r->tSubmit).count());
}

// device copies of a request's inputs
bool upload(Server& s, Request* r, std::string& err) {
  if (r->kind == 0) {
    const kgb_daylight_request& d = r->d;
    const DayLayout L = day_layout(d);
    r->devBytes = L.total;
    if (!cuok(cudaMalloc(&r->dev, r->devBytes), err, "request memory")) return false;
    char* b = static_cast<char*>(r->dev);
    r->w64.resize(size_t(d.nQ) * d.nDir);
    const float* W = static_cast<const float*>(d.W);
    for (size_t k = 0; k < r->w64.size(); ++k) r->w64[k] = double(W[k]);
    cudaMemcpyAsync(b, d.P, L.offN, cudaMemcpyHostToDevice, s.st);
    cudaMemcpyAsync(b + L.offN, d.N, L.offN, cudaMemcpyHostToDevice, s.st);
    cudaMemcpyAsync(b + L.offD, d.D, size_t(d.nDir) * 12, cudaMemcpyHostToDevice, s.st);
    cudaMemcpyAsync(b + L.offW, r->w64.data(), r->w64.size() * 8, cudaMemcpyHostToDevice, s.st);
    launch_ray_table(reinterpret_cast<const float*>(b + L.offD), d.nDir, b + L.offTab, s.st);
  } else {
    const kgb_views_request& v = r->v;
    const DScene& sc = s.scenes[size_t(v.scene)];
    const uint64_t K = uint64_t(v.view.nAz) * v.view.nEl;
    const size_t offN = size_t(v.nSensors) * 12, offRow = (offN * 2 + 255) & ~size_t(255), offW = offRow + size_t(v.view.nEl) * 8;
    const size_t offLab = (offW + size_t(v.view.nEl) * 8 + 255) & ~size_t(255), offCls = (offLab + (v.label ? sc.nTris : 0) + 255) & ~size_t(255);
    const size_t offDist = (offCls + s.chunkSensors * K + 255) & ~size_t(255), offOut = (offDist + s.chunkSensors * K * 4 + 255) & ~size_t(255);
    r->devBytes = offOut + size_t(s.chunkSensors) * views_NA(v) * 8;
    if (!cuok(cudaMalloc(&r->dev, r->devBytes), err, "request memory")) return false;
    char* b = static_cast<char*>(r->dev);
    cudaMemcpyAsync(b, v.P, offN, cudaMemcpyHostToDevice, s.st);
    cudaMemcpyAsync(b + offN, v.N, offN, cudaMemcpyHostToDevice, s.st);
    cudaMemcpyAsync(b + offRow, r->rowSin.data(), size_t(v.view.nEl) * 8, cudaMemcpyHostToDevice, s.st);
    cudaMemcpyAsync(b + offW, r->wRow.data(), size_t(v.view.nEl) * 8, cudaMemcpyHostToDevice, s.st);
    if (v.label) cudaMemcpyAsync(b + offLab, v.label, sc.nTris, cudaMemcpyHostToDevice, s.st);
  }
  s.used += r->devBytes;
  return true;
}

// one views chunk of a request: the single-request view kernels on its device arrays
bool run_views_chunk(Server& s, Request* r, uint32_t i0, uint32_t nc, std::string& err) {
  const kgb_views_request& v = r->v;
  const DScene& sc = s.scenes[size_t(v.scene)];
  const uint64_t K = uint64_t(v.view.nAz) * v.view.nEl;
  const size_t offN = size_t(v.nSensors) * 12, offRow = (offN * 2 + 255) & ~size_t(255), offW = offRow + size_t(v.view.nEl) * 8;
  const size_t offLab = (offW + size_t(v.view.nEl) * 8 + 255) & ~size_t(255), offCls = (offLab + (v.label ? sc.nTris : 0) + 255) & ~size_t(255);
  const size_t offDist = (offCls + s.chunkSensors * K + 255) & ~size_t(255), offOut = (offDist + s.chunkSensors * K * 4 + 255) & ~size_t(255);
  char* b = static_cast<char*>(r->dev);
  const double rad = v.view.north * KGB_PI_D / 180;
  ViewArgs a{};
  a.nodes = static_cast<const Node8*>(sc.nodes); a.tris = static_cast<const TriRec*>(sc.tris); a.nNodes = sc.nNodes;
  a.P = reinterpret_cast<const float*>(b); a.N = reinterpret_cast<const float*>(b + offN);
  a.first = i0; a.n = nc; a.out0 = 0; a.stride = nc; a.i0 = i0;
  a.K = uint32_t(K); a.nWords = uint32_t((K + 31) / 32); a.nAz = v.view.nAz; a.nEl = v.view.nEl; a.rayFlags = v.rayFlags;
  a.rowSin = reinterpret_cast<const float*>(b + offRow); a.az0 = v.view.az0; a.dAz = v.view.dAz; a.groundZ = v.view.groundZ;
  a.cosN = float(std::cos(rad)); a.sinN = float(std::sin(rad));
  a.world = v.view.world ? 1 : 0; a.cull = v.view.cull ? 1 : 0; a.jitter = v.view.jitter ? 1 : 0; a.nS = v.view.nS; a.back = v.view.back ? 1 : 0;
  a.vground = v.view.vground ? 1 : 0;
  a.label = v.label ? reinterpret_cast<const uint8_t*>(b + offLab) : nullptr;
  a.cls = reinterpret_cast<uint8_t*>(b + offCls); a.dist = reinterpret_cast<float*>(b + offDist);
  a.counter = s.dCtl; a.status = s.dCtl + 1;
  cudaMemsetAsync(s.dCtl, 0, 8, s.st);
  launch_view(a, s.numSMs * 4, s.st);
  ViewReduceArgs ra{};
  ra.cls = a.cls; ra.dist = a.dist; ra.nc = nc; ra.K = uint32_t(K); ra.nAz = v.view.nAz; ra.nEl = v.view.nEl; ra.nClass = v.nClass;
  ra.nReach = v.nReach; ra.glazing = v.glazing ? 1 : 0; ra.iso = v.isoDim ? 1 : 0; ra.NA = views_NA(v);
  ra.wRow = reinterpret_cast<const double*>(b + offW); ra.farDist = float(v.farDist); ra.lnFar = std::log(v.farDist);
  for (uint32_t k = 0; k < v.nReach; ++k) ra.reach[k] = v.reach[k];
  ra.isoDim = v.isoDim; ra.world = a.world; ra.jitter = a.jitter; ra.i0 = i0; ra.nS = v.view.nS; ra.back = a.back;
  ra.az0 = v.view.az0; ra.dAz = v.view.dAz; ra.rowSin = a.rowSin; ra.out = reinterpret_cast<double*>(b + offOut);
  launch_reduce_view(ra, s.st);
  cudaMemcpyAsync(v.out + size_t(i0) * ra.NA, ra.out, size_t(nc) * ra.NA * 8, cudaMemcpyDeviceToHost, s.st);
  uint32_t status = 0;
  cudaMemcpyAsync(&status, s.dCtl + 1, 4, cudaMemcpyDeviceToHost, s.st);
  if (!cuok(cudaStreamSynchronize(s.st), err, "views chunk")) return false;
  if (status) { err = "views chunk: traversal stack overflow"; return false; }
  s.rays += uint64_t(nc) * K;
  return true;
}

struct Part { Request* r; uint32_t i0, n; };

// one daylight batch through the graph; parts' results scattered into their requests' outputs
bool run_daylight_batch(Server& s, const std::vector<Part>& parts, std::string& err) {
  uint32_t tasks = 0, sens = 0;
  size_t bits = 0, out = 0;
  for (size_t k = 0; k < parts.size(); ++k) {
    const Part& p = parts[k];
    const kgb_daylight_request& d = p.r->d;
    const DScene& sc = s.scenes[size_t(d.scene)];
    const char* b = static_cast<const char*>(p.r->dev);
    const DayLayout L = day_layout(d);
    Seg& g = s.hSegs[k];
    g.nodes = static_cast<const Node8*>(sc.nodes); g.tris = static_cast<const TriRec*>(sc.tris); g.nNodes = sc.nNodes;
    g.P = reinterpret_cast<const float*>(b) + 3 * size_t(p.i0); g.N = reinterpret_cast<const float*>(b + L.offN) + 3 * size_t(p.i0);
    g.D = reinterpret_cast<const float*>(b + L.offD); g.tab = reinterpret_cast<const RayDir*>(b + L.offTab);
    g.W = reinterpret_cast<const double*>(b + L.offW);
    g.nDir = d.nDir; g.nWords = (d.nDir + 31) / 32; g.n = p.n; g.rayFlags = d.rayFlags; g.nQ = d.nQ; g.useCosMask = d.useCosMask;
    g.taskBase = tasks; g.sensBase = sens; g.bitsOff = uint32_t(bits); g.outOff = uint32_t(out);
    tasks += (p.n + 31) / 32 * g.nWords;
    sens += p.n;
    bits += size_t(g.nWords) * p.n;
    out += size_t(d.nQ) * p.n;
  }
  if (bits > s.bitsPoolWords || out > s.outPoolDoubles || sens > s.maxSensPerBatch) { err = "internal: batch beyond its pools"; return false; }
  s.hHdr->nSegs = uint32_t(parts.size()); s.hHdr->nTasks = tasks; s.hHdr->nSens = sens;
  if (!cuok(cudaGraphLaunch(s.graph, s.st), err, "batch graph") || !cuok(cudaStreamSynchronize(s.st), err, "batch")) return false;
  uint32_t status = 0;
  cudaMemcpy(&status, s.dCtl + 1, 4, cudaMemcpyDeviceToHost);
  if (status) { err = "batch: traversal stack overflow"; return false; }
  for (size_t k = 0; k < parts.size(); ++k) {
    const Part& p = parts[k];
    const Seg& g = s.hSegs[k];
    for (uint32_t q = 0; q < g.nQ; ++q)
      std::memcpy(p.r->d.out + size_t(q) * p.r->nSensors + p.i0, s.hOut + g.outOff + size_t(q) * p.n, size_t(p.n) * 8);
    s.rays += uint64_t(p.n) * g.nDir;
  }
  ++s.batches;
  return true;
}

// one iteration: admit, pack, run; false when there was nothing to do
bool step(Server& s) {
  std::vector<Request*> admitted;
  {
    std::unique_lock<std::mutex> lk(s.m);
    while (!s.pending.empty()) {
      Request* r = s.pending.front();
      const uint64_t need = r->kind == 0 ? daylight_bytes(r->d) : views_bytes(r->v, s.chunkSensors, s.scenes[size_t(r->v.scene)].nTris);
      if (s.used + need > s.budget && !s.active.empty()) break;   // wait for memory (a lone request always runs)
      s.pending.pop_front();
      admitted.push_back(r);
      s.active.push_back(r);
    }
  }
  for (Request* r : admitted) {
    std::string err;
    if (!upload(s, r, err)) { std::lock_guard<std::mutex> lk(s.m); finish(s, r, false, err); s.doneCv.notify_all(); }
  }
  std::vector<Request*> act;
  {
    std::lock_guard<std::mutex> lk(s.m);
    for (Request* r : s.active) if (!r->done) act.push_back(r);
  }
  if (act.empty()) return false;
  // pack: round robin over the active requests, a chunk each per turn, until the batch is full
  std::vector<Part> parts;
  std::vector<Part> views;
  uint64_t raysInBatch = 0;
  size_t bitsInBatch = 0, outInBatch = 0;
  uint32_t sensInBatch = 0;
  bool progress = true;
  const size_t n = act.size();
  while (progress && parts.size() < kMaxSegs && raysInBatch < s.batchRays) {
    progress = false;
    for (size_t j = 0; j < n && parts.size() < kMaxSegs && raysInBatch < s.batchRays; ++j) {
      Request* r = act[(s.rr + j) % n];
      if (r->nextSensor >= r->nSensors) continue;
      const uint32_t c = std::min(s.chunkSensors, r->nSensors - r->nextSensor);
      if (r->kind == 1) {
        if (views.empty()) { views.push_back(Part{r, r->nextSensor, c}); r->nextSensor += c; progress = true; }
        continue;
      }
      const size_t words = size_t((r->d.nDir + 31) / 32) * c;
      if (bitsInBatch + words > s.bitsPoolWords || outInBatch + size_t(r->d.nQ) * c > s.outPoolDoubles || sensInBatch + c > s.maxSensPerBatch) continue;
      parts.push_back(Part{r, r->nextSensor, c});
      r->nextSensor += c;
      raysInBatch += uint64_t(c) * r->d.nDir;
      sensInBatch += c;
      bitsInBatch += words;
      outInBatch += size_t(r->d.nQ) * c;
      progress = true;
    }
  }
  s.rr = (s.rr + 1) % std::max<size_t>(1, n);
  std::string err;
  const auto account = [&](const Part& p, bool ok) {
    std::lock_guard<std::mutex> lk(s.m);
    p.r->doneSensors += p.n;
    if (!ok && !p.r->done) finish(s, p.r, false, err);
    else if (p.r->doneSensors == p.r->nSensors && !p.r->done) finish(s, p.r, true, "");
    s.active.erase(std::remove_if(s.active.begin(), s.active.end(), [](Request* q) { return q->done; }), s.active.end());
  };
  if (!parts.empty()) {
    const bool ok = run_daylight_batch(s, parts, err);
    for (const Part& p : parts) account(p, ok);
  }
  for (const Part& p : views) account(p, run_views_chunk(s, p.r, p.i0, p.n, err));
  s.doneCv.notify_all();
  return !parts.empty() || !views.empty();
}

void loop(Server* s) {
  cudaSetDevice(s->device);
  for (;;) {
    {
      std::unique_lock<std::mutex> lk(s->m);
      s->cv.wait(lk, [&] { return s->stop || !s->pending.empty() || !s->active.empty(); });
      if (s->stop) return;
    }
    step(*s);
  }
}

// the autotuner: calibration batches of one synthetic request on scene 0 (its first sensors against a fixed
// direction table), keeping the chunk size and batch size with the most rays per second
bool autotune(Server& s, std::string& err) {
  const DScene& sc = s.scenes[0];
  if (!sc.nNodes) return true;
  const uint32_t nDir = 1024, nSens = 65536;
  std::vector<float> P(3 * nSens), N(3 * nSens), D(3 * nDir), W(nDir, 1.f);
  std::vector<double> out(nSens);
  // sensors on a horizontal grid over the middle of the scene's first node box, looking up; directions over the sky
  float p0[3];
  std::vector<uint32_t> node(20);
  cudaMemcpy(node.data(), sc.nodes, 80, cudaMemcpyDeviceToHost);
  std::memcpy(p0, node.data(), 12);
  for (uint32_t i = 0; i < nSens; ++i) {
    P[3 * i] = p0[0] * 0.5f + float(i % 256); P[3 * i + 1] = p0[1] * 0.5f + float(i / 256); P[3 * i + 2] = 1.f;
    N[3 * i] = 0; N[3 * i + 1] = 0; N[3 * i + 2] = 1;
  }
  for (uint32_t d = 0; d < nDir; ++d) {
    const double z = 0.05 + 0.9 * (d + 0.5) / nDir, a = 2.399963 * d, r = std::sqrt(1 - z * z);
    D[3 * d] = float(r * std::sin(a)); D[3 * d + 1] = float(r * std::cos(a)); D[3 * d + 2] = float(z);
  }
  double best = -1;
  uint32_t bestChunk = s.chunkSensors;
  uint64_t bestRays = s.batchRays;
  for (uint32_t chunk : {2048u, 8192u, 32768u})
    for (uint64_t br : {uint64_t(1) << 28, uint64_t(1) << 30}) {
      s.chunkSensors = chunk;
      s.batchRays = br;
      if (!make_pools(s, err)) return false;
      Request r;
      r.kind = 0;
      r.d = kgb_daylight_request{0, nSens, nDir, 1, P.data(), N.data(), D.data(), W.data(), 1u, KGB_RAY_TERMINATE_ON_FIRST_HIT | KGB_RAY_DISABLE_ANYHIT, out.data()};
      r.nSensors = nSens;
      if (!upload(s, &r, err)) return false;
      std::vector<Part> parts;
      uint64_t acc = 0;
      uint32_t sens = 0;
      for (uint32_t i = 0; i < nSens && parts.size() < kMaxSegs && acc < br && sens + chunk <= s.maxSensPerBatch; i += chunk) {
        const uint32_t c = std::min(chunk, nSens - i);
        parts.push_back(Part{&r, i, c});
        acc += uint64_t(c) * nDir;
        sens += c;
      }
      const auto t0 = Clock::now();
      const bool ok = run_daylight_batch(s, parts, err);
      const double sec = std::chrono::duration<double>(Clock::now() - t0).count();
      uint64_t rays = 0;
      for (const Part& p : parts) rays += uint64_t(p.n) * nDir;
      cudaFree(r.dev);
      s.used -= r.devBytes;
      if (!ok) return false;
      const double rate = rays / sec;
      if (rate > best) { best = rate; bestChunk = chunk; bestRays = br; }
    }
  s.chunkSensors = bestChunk;
  s.batchRays = bestRays;
  s.rays = 0;
  s.batches = 0;
  return make_pools(s, err);
}

}  // namespace
}  // namespace kgb

using namespace kgb;

extern "C" {

KGB_API kgb_server* kgb_server_create(uint64_t hbmBudgetBytes) {
  Server* s = new Server;
  std::string err;
  const auto bad = [&](const std::string& m) { set_error(m); kgb_server_destroy(reinterpret_cast<kgb_server*>(s)); return nullptr; };
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return bad("no CUDA device");
  cudaGetDevice(&s->device);
  cudaDeviceGetAttribute(&s->numSMs, cudaDevAttrMultiProcessorCount, s->device);
  s->gridBits = s->numSMs * 4;
  s->budget = hbmBudgetBytes;
  if (!cuok(cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking), err, "stream") ||
      !cuok(cudaMallocHost(&s->hSegs, sizeof(Seg) * kMaxSegs), err, "pinned") || !cuok(cudaMallocHost(&s->hHdr, sizeof(BatchHdr)), err, "pinned") ||
      !cuok(cudaMalloc(&s->dSegs, sizeof(Seg) * kMaxSegs), err, "segments") || !cuok(cudaMalloc(&s->dHdr, sizeof(BatchHdr)), err, "segments") ||
      !cuok(cudaMalloc(&s->dCtl, 64), err, "control"))
    return bad(err);
  std::memset(s->hSegs, 0, sizeof(Seg) * kMaxSegs);
  std::memset(s->hHdr, 0, sizeof(BatchHdr));
  if (!make_pools(*s, err)) return bad(err);
  s->th = std::thread(loop, s);
  return reinterpret_cast<kgb_server*>(s);
}

KGB_API void kgb_server_destroy(kgb_server* h) {
  if (!h) return;
  Server* s = reinterpret_cast<Server*>(h);
  {
    std::lock_guard<std::mutex> lk(s->m);
    s->stop = true;
  }
  s->cv.notify_all();
  if (s->th.joinable()) s->th.join();
  if (s->st) cudaStreamSynchronize(s->st);
  for (auto& kv : s->all) { if (kv.second->dev) cudaFree(kv.second->dev); delete kv.second; }
  for (DScene& d : s->scenes) { cudaFree(d.nodes); cudaFree(d.tris); }
  if (s->graph) cudaGraphExecDestroy(s->graph);
  cudaFree(s->dBits); cudaFree(s->dOut); cudaFree(s->dSegs); cudaFree(s->dHdr); cudaFree(s->dCtl);
  if (s->hOut) cudaFreeHost(s->hOut);
  if (s->hSegs) cudaFreeHost(s->hSegs);
  if (s->hHdr) cudaFreeHost(s->hHdr);
  if (s->st) cudaStreamDestroy(s->st);
  delete s;
}

KGB_API int kgb_server_add_scene(kgb_server* h, const float* v, size_t nv, const uint32_t* tri, size_t nt, int32_t* sceneId) {
  Server* s = reinterpret_cast<Server*>(h);
  for (size_t k = 0; k < 3 * nt; ++k) if (tri[k] >= nv) { set_error("kgb_server_add_scene: a triangle's vertex index exceeds the vertices"); return 0; }
  DScene d;
  std::lock_guard<std::mutex> lk(s->m);
  if (nt) {   // the device builder (bvh_gpu.cu), on the server's stream
    uint64_t temp = 0;
    const std::string why = build_bvh8_gpu(v, nv, tri, nt, nullptr, nullptr, s->st, &d.nodes, &d.tris, &d.nNodes, &temp);
    if (!why.empty()) {
      if (d.nodes) cudaFree(d.nodes);
      if (d.tris) cudaFree(d.tris);
      set_error("kgb_server_add_scene: " + why);
      return 0;
    }
  }
  d.nTris = uint32_t(nt);
  d.bytes = uint64_t(d.nNodes) * 80 + uint64_t(nt) * 48;
  s->used += d.bytes;
  s->scenes.push_back(d);
  *sceneId = int32_t(s->scenes.size() - 1);
  return 1;
}

KGB_API int kgb_server_autotune(kgb_server* h) {
  Server* s = reinterpret_cast<Server*>(h);
  std::unique_lock<std::mutex> lk(s->m);
  if (!s->active.empty() || !s->pending.empty()) { set_error("kgb_server_autotune: only while idle"); return 0; }
  std::string err;
  if (!autotune(*s, err)) { set_error(err); return 0; }
  return 1;
}

KGB_API int kgb_server_submit(kgb_server* h, const kgb_daylight_request* req, uint64_t* ticket) {
  Server* s = reinterpret_cast<Server*>(h);
  if (req->scene < 0 || size_t(req->scene) >= s->scenes.size()) { set_error("kgb_server_submit: unknown scene"); return 0; }
  if (req->nQ < 1 || req->nQ > kMaxQ) { set_error("kgb_server_submit: 1 to 8 quantities"); return 0; }
  Request* r = new Request;
  r->kind = 0;
  r->d = *req;
  r->nSensors = req->nSensors;
  r->tSubmit = Clock::now();
  std::lock_guard<std::mutex> lk(s->m);
  r->ticket = s->nextTicket++;
  if (!r->nSensors || !req->nDir) { std::fill(req->out, req->out + size_t(req->nQ) * req->nSensors, 0.0); finish(*s, r, true, ""); }
  else s->pending.push_back(r);
  s->all[r->ticket] = r;
  *ticket = r->ticket;
  s->cv.notify_all();
  return 1;
}

KGB_API int kgb_server_submit_views(kgb_server* h, const kgb_views_request* req, uint64_t* ticket) {
  Server* s = reinterpret_cast<Server*>(h);
  if (req->scene < 0 || size_t(req->scene) >= s->scenes.size()) { set_error("kgb_server_submit_views: unknown scene"); return 0; }
  if (req->nClass > KGB_VIEW_CLASSES || req->nReach > 8) { set_error("kgb_server_submit_views: at most 16 groups and 8 reach distances"); return 0; }
  Request* r = new Request;
  r->kind = 1;
  r->v = *req;
  r->rowSin.assign(req->view.rowSin, req->view.rowSin + 2 * size_t(req->view.nEl));
  r->wRow.assign(req->wRow, req->wRow + req->view.nEl);
  r->nSensors = req->nSensors;
  r->tSubmit = Clock::now();
  std::lock_guard<std::mutex> lk(s->m);
  r->ticket = s->nextTicket++;
  if (!r->nSensors) finish(*s, r, true, "");
  else s->pending.push_back(r);
  s->all[r->ticket] = r;
  *ticket = r->ticket;
  s->cv.notify_all();
  return 1;
}

KGB_API int kgb_server_wait(kgb_server* h, uint64_t ticket, double timeoutSec) {
  Server* s = reinterpret_cast<Server*>(h);
  std::unique_lock<std::mutex> lk(s->m);
  auto it = s->all.find(ticket);
  if (it == s->all.end()) { set_error("kgb_server_wait: unknown ticket"); return 0; }
  Request* r = it->second;
  if (!s->doneCv.wait_for(lk, std::chrono::duration<double>(timeoutSec), [&] { return r->done; })) { set_error("kgb_server_wait: timed out"); return 0; }
  if (r->failed) { set_error(r->err); return 0; }
  return 1;
}

// out[0..7]: completed requests, p50, p90, p99, max latency (s), rays, batches, HBM bytes in use; out[8..9]: the tuned
// chunk sensors and batch rays
KGB_API void kgb_server_stats(kgb_server* h, double* out) {
  Server* s = reinterpret_cast<Server*>(h);
  std::lock_guard<std::mutex> lk(s->m);
  std::vector<double> l = s->latencies;
  std::sort(l.begin(), l.end());
  const auto q = [&](double f) { return l.empty() ? 0.0 : l[std::min(l.size() - 1, size_t(f * (l.size() - 1) + 0.5))]; };
  out[0] = double(l.size()); out[1] = q(0.5); out[2] = q(0.9); out[3] = q(0.99); out[4] = l.empty() ? 0.0 : l.back();
  out[5] = double(s->rays); out[6] = double(s->batches); out[7] = double(s->used); out[8] = s->chunkSensors; out[9] = double(s->batchRays);
}

}  // extern "C"
