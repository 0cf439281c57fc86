// The serving loop: device-resident scenes, and daylight / views requests of any size admitted against an HBM budget
// and run with continuous batching.
//
// Requests are cut into work items that run one after another on one work stream, two of them queued at a time so that
// the GPU never waits for the host:
//  - a daylight batch: chunks of sensors of any number of admitted daylight requests, traced by ONE persistent any-hit
//    launch (k_bits_batch: tasks of 32 sensors x one 32-direction word, each task finds its chunk in the batch's
//    segment table) and reduced by ONE launch giving every quantity of every chunk (k_reduce_batch). The batch's
//    pipeline (segment table up, counter reset, the two kernels, the sums and the status down into pinned memory) is a
//    CUDA graph built once per slot and replayed per batch, its copy sizes and the reduce's grid set per batch;
//  - a views chunk: the view kernels (k_view, k_view_reduce, k_iso) on a range of one request's sensors, sized by rays.
// The scheduler picks the next item by a priority over every request with sensors not yet issued: a request that has
// waited more than 1.0 s goes first, in arrival order; the others by their remaining work (rays times a running
// estimate of seconds per ray of its kind, measured from the items' own GPU time) divided by their age plus 0.3 s.
// Short requests overtake long ones, which keeps the p50 near one item's time, and no request waits behind younger
// ones for long, which keeps the p99 at arrival order's. A daylight batch is packed in that order, a chunk at a time.
// Admitted requests' inputs go up on a separate upload stream into stream-ordered allocations from the server's own
// memory pool, so neither uploads nor frees wait for the work stream. A request completes when its last item has; its
// results are bit-identical to the request run alone through the single-request entry points (same kernels, same
// per-sensor arithmetic and summation order).
//
// A daylight request may also ask for its hourly time series (kgb_server_submit_series). Its S matrix is split into
// bf16 pieces once, at upload; in each batch, right after the batch's graph, the series chunks of every request in it
// get their V rows from the batch's visibility bits and ground sums, and all of them run as ONE grouped launch of the
// tensor-core contraction (series_tc_group: a tile table across the chunks, each with its own tensor maps, K and output
// rows), whose rows come down with the batch. A request's rows equal kgb_series' tensor-core form bit for bit.
//
// The autotuner times calibration batches on the first scene at start-up and keeps the chunk size and batch size
// (rays per batch) for the daylight pipeline: the fastest, or a smaller batch within 5 % of it.
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

// Three blocks an SM, as k_bits: left to itself the compiler gives this kernel 100 registers and two blocks an SM, and
// the batch's trace ran 13 % longer than the single-request kernel on the same rays.
__global__ void __launch_bounds__(256, 3) k_bits_batch(const BatchHdr* hdr, const Seg* segs, uint32_t* bitsPool, uint32_t* counter, uint32_t* status) {
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
// one fma per term, the float factor widened exactly, a zero factor skipped).
// NQ = the chunk's quantity count, a compile-time constant: the accumulators stay in registers and no predicated-off
// FP64 instruction takes a slot of the narrow FP64 pipe (one kernel over kMaxQ accumulators with q < nQ tests held
// them in local memory and ran 1.75 times as long as the single-request reduces of the same sums).
template <uint32_t NQ>
__device__ __forceinline__ void reduce_chunk_sensor(const Seg& g, uint32_t i, const uint32_t* bitsPool, double* outPool) {
  const F3 n = ld3(g.N + 3 * i);
  double acc[NQ];
#pragma unroll
  for (uint32_t q = 0; q < NQ; ++q) acc[q] = 0;
  for (uint32_t w = 0; w < g.nWords; ++w) {
    uint32_t m = bitsPool[g.bitsOff + size_t(w) * g.n + i];
    while (m) {
      const uint32_t d = w * 32 + (__ffs(m) - 1);
      m &= m - 1;
      const F3 dir = ld3(g.D + 3 * d);
      const float c = fmaxf(__fadd_rn(__fadd_rn(__fmul_rn(n.x, dir.x), __fmul_rn(n.y, dir.y)), __fmul_rn(n.z, dir.z)), 0.f);
#pragma unroll
      for (uint32_t q = 0; q < NQ; ++q) {
        const float x = ((g.useCosMask >> q) & 1u) ? c : 1.f;
        if (x != 0.f) acc[q] = __fma_rn(widen(x), __ldg(g.W + size_t(q) * g.nDir + d), acc[q]);
      }
    }
  }
#pragma unroll
  for (uint32_t q = 0; q < NQ; ++q) outPool[g.outOff + size_t(q) * g.n + i] = acc[q];
}
static_assert(kMaxQ == 8, "k_reduce_batch dispatches 1..8 quantities");
constexpr uint32_t kReduceBatchBlock = 128;   // as the single-request reduce: small blocks keep the SMs busy to the end
__global__ void __launch_bounds__(kReduceBatchBlock) k_reduce_batch(const BatchHdr* hdr, const Seg* segs, const uint32_t* bitsPool, double* outPool) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= hdr->nSens) return;
  const Seg& g = segs[find_seg(segs, hdr->nSegs, t, true)];
  const uint32_t i = t - g.sensBase;
  switch (g.nQ) {   // uniform across a warp but where it straddles two chunks
    case 1: reduce_chunk_sensor<1>(g, i, bitsPool, outPool); break;
    case 2: reduce_chunk_sensor<2>(g, i, bitsPool, outPool); break;
    case 3: reduce_chunk_sensor<3>(g, i, bitsPool, outPool); break;
    case 4: reduce_chunk_sensor<4>(g, i, bitsPool, outPool); break;
    case 5: reduce_chunk_sensor<5>(g, i, bitsPool, outPool); break;
    case 6: reduce_chunk_sensor<6>(g, i, bitsPool, outPool); break;
    case 7: reduce_chunk_sensor<7>(g, i, bitsPool, outPool); break;
    case 8: reduce_chunk_sensor<8>(g, i, bitsPool, outPool); break;
    default: break;
  }
}


// ------------------------------------------------------------------------------------------------ host side
namespace {
using Clock = std::chrono::steady_clock;

constexpr int kSlots = 2;                       // work items of each kind that can be in flight at once
constexpr size_t kDepth = 2;                    // work items queued on the work stream at once
constexpr uint32_t kMaxViewChunk = 65536;       // sensors in one views chunk
constexpr uint32_t kMaxNA = 3 * KGB_VIEW_CLASSES + 1 + 8 + 1 + 1;   // views columns
constexpr double kAgeSeconds = 0.3;             // the priority's age offset (default; kgb_server_set_priority)
constexpr double kOldSeconds = 1.0;             // past this wait a request goes first, in arrival order (default)
constexpr size_t kSeriesVBytes = size_t(256) << 20;   // per daylight slot: the series chunks' V pieces (bf16)
constexpr size_t kSeriesEBytes = size_t(256) << 20;   // per daylight slot: their rows of E, on the device and pinned

struct DScene {
  void* nodes = nullptr;
  void* tris = nullptr;
  uint32_t nNodes = 0, nTris = 0;
  uint64_t bytes = 0;
};

struct Request {
  uint64_t ticket = 0;
  int kind = 0;   // 0 daylight, 1 views
  kgb_daylight_request d{};
  kgb_views_request v{};
  std::vector<float> rowSin;
  std::vector<double> wRow;
  std::vector<double> w64;    // daylight: the weights widened to double (the source of their upload)
  uint32_t nSensors = 0, nextSensor = 0, doneSensors = 0;
  uint64_t raysPerSensor = 0;
  void* dev = nullptr;        // P, N, D, ray table, W (daylight) | P, N, rowSin, wRow, label (views)
  uint64_t devBytes = 0;
  // the time series of a daylight request (kgb_server_submit_series)
  bool series = false;
  kgb_series_request sq{};
  uint32_t Kp = 0;            // its K (patches + ground), padded to 64
  std::vector<int32_t> csr, sunOfCol;   // directions per patch (first [P + 1], then the directions); sun per column
  Clock::time_point tSubmit, tDone;
  bool done = false, failed = false;
  std::string err;
};

struct Part { Request* r; uint32_t i0, n; size_t eOff = 0, vOff = 0; };   // its series rows (floats) and V pieces (bytes) in the slot's pools

// a daylight batch slot: its pinned and device buffers, its graph and the nodes set per batch
struct DaySlot {
  Seg* hSegs = nullptr;         // pinned [kMaxSegs]
  BatchHdr* hHdr = nullptr;     // pinned
  uint32_t* hStatus = nullptr;  // pinned
  double* hOut = nullptr;       // pinned [outPoolDoubles]
  Seg* dSegs = nullptr;
  BatchHdr* dHdr = nullptr;
  uint32_t* dCtl = nullptr;     // counter, status
  uint32_t* dBits = nullptr;
  double* dOut = nullptr;
  cudaGraph_t graph = nullptr;      // kept: the nodes set per batch belong to it
  cudaGraphExec_t exec = nullptr;
  cudaGraphNode_t nSegs = nullptr, nReduce = nullptr, nOut = nullptr;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  std::vector<Part> parts;
  uint64_t rays = 0;
  // series: the chunks' V pieces and rows of E (device), the rows again (pinned), the series' status word (pinned)
  void* dV = nullptr;
  float* dE = nullptr;
  float* hE = nullptr;
  uint32_t* hSeriesStatus = nullptr;
  bool anySeries = false;
};
// a views chunk slot: its status and columns come back into pinned memory
struct ViewSlot {
  uint32_t* dCtl = nullptr;
  uint32_t* hStatus = nullptr;
  double* hOut = nullptr;       // pinned [kMaxViewChunk x kMaxNA]
  cudaEvent_t ev[2] = {nullptr, nullptr};
  Part part{nullptr, 0, 0};
  uint32_t NA = 0;
};
}  // namespace

struct Server {
  int device = 0, numSMs = 0, gridBits = 0, gridView = 0;
  cudaStream_t st = nullptr;    // work stream: daylight batches and views chunks in the scheduler's order
  cudaStream_t up = nullptr;    // uploads of admitted requests' inputs
  cudaEvent_t upDone = nullptr;
  bool upPending = false;       // uploads issued that the work stream has not been made to wait for
  cudaMemPool_t pool = nullptr; // requests' device memory
  uint64_t budget = 0, used = 0;
  std::vector<DScene> scenes;
  // tuning
  uint32_t chunkSensors = 8192;
  uint64_t batchRays = uint64_t(1) << 28;
  uint64_t viewRays = uint64_t(1) << 27;
  double oldSeconds = kOldSeconds, ageSeconds = kAgeSeconds;   // the scheduler's priority (kgb_server_set_priority)
  // batch pools (fixed for the graphs)
  size_t bitsPoolWords = 0, outPoolDoubles = 0;
  uint32_t maxSensPerBatch = 0;
  uint64_t poolBytes = 0;
  DaySlot day[kSlots];
  ViewSlot view[kSlots];
  uint8_t* dCls = nullptr;      // views scratch for one chunk (chunks run in stream order): classes, distances, columns
  float* dDist = nullptr;
  double* dViewOut = nullptr;
  uint64_t viewCap = 0;         // rays the scratch holds
  std::deque<std::pair<int, int>> inflight;   // (kind, slot), in launch order
  double cost[2] = {1e-10, 3e-10};            // seconds per ray of daylight and views work (running estimate)
  // requests
  std::mutex m;
  std::condition_variable cv, doneCv;
  std::deque<Request*> pending;
  std::vector<Request*> active;
  std::map<uint64_t, Request*> all;
  uint64_t nextTicket = 1;
  bool stop = false;
  std::thread th;
  std::vector<double> latencies;   // seconds, completed requests
  uint64_t items = 0, rays = 0;
  double gpuSec[2] = {0, 0}, kindRays[2] = {0, 0};   // GPU seconds and rays of daylight batches and views chunks
  double queuedSec = 0;                             // wall seconds with at least one item on the work stream
  Clock::time_point queuedSince;
};

namespace {

bool cuok(cudaError_t e, std::string& err, const char* what) {
  if (e == cudaSuccess) return true;
  err = std::string(what) + ": " + cudaGetErrorString(e);
  return false;
}
size_t up256(size_t x) { return (x + 255) & ~size_t(255); }

// a daylight request's device arrays: P, N (12 B per sensor each), D (12 B per direction), its ray table (48 B per
// direction), its weights as doubles [nQ x nDir]; 256-byte aligned pieces
struct DayLayout { size_t offN, offD, offTab, offW, total; };
DayLayout day_layout(const kgb_daylight_request& d) {
  DayLayout L;
  L.offN = size_t(d.nSensors) * 12;
  L.offD = up256(2 * L.offN);
  L.offTab = up256(L.offD + size_t(d.nDir) * 12);
  L.offW = up256(L.offTab + size_t(d.nDir) * 48);
  L.total = up256(L.offW + size_t(d.nQ) * d.nDir * 8);
  return L;
}
// a views request's device arrays: P, N, rowSin [nEl x 2], wRow [nEl], labels [scene triangles] (when given)
struct ViewLayout { size_t offN, offRow, offW, offLab, total; };
ViewLayout view_layout(const kgb_views_request& v, uint32_t nTris) {
  ViewLayout L;
  L.offN = size_t(v.nSensors) * 12;
  L.offRow = up256(2 * L.offN);
  L.offW = up256(L.offRow + size_t(v.view.nEl) * 8);
  L.offLab = up256(L.offW + size_t(v.view.nEl) * 8);
  L.total = up256(L.offLab + (v.label ? nTris : 0));
  return L;
}
// a series request's device arrays after its daylight ones: S^T in three bf16 pieces [3 x T x Kp], S [P x T] and g [T]
// (the pieces' source), the directions per patch, wsky, the sun direction of each column, sunVec, sunW
struct SeriesLayout { size_t offSt, offS, offG, offCsr, offWsky, offSunCol, offSunVec, offSunW, total; };
SeriesLayout series_layout(const Request& r, size_t base) {
  const kgb_series_in& in = r.sq.in;
  const size_t T = size_t(in.T), P = size_t(in.P);
  SeriesLayout L;
  L.offSt = base;
  L.offS = up256(L.offSt + 3 * T * r.Kp * 2);
  L.offG = up256(L.offS + P * T * 4);
  L.offCsr = up256(L.offG + T * 4);
  L.offWsky = up256(L.offCsr + (P + 1 + in.nSky) * 4);
  L.offSunCol = up256(L.offWsky + size_t(in.nSky) * 4);
  L.offSunVec = up256(L.offSunCol + T * 4);
  L.offSunW = up256(L.offSunVec + size_t(in.nSun) * 12);
  L.total = up256(L.offSunW + size_t(in.nSun) * 4);
  return L;
}
uint32_t views_NA(const kgb_views_request& r) { return 3 * r.nClass + 1 + r.nReach + (r.glazing ? 1 : 0) + (r.isoDim ? 1 : 0); }
uint64_t request_bytes(const Server& s, const Request* r) {
  if (r->kind == 1) return view_layout(r->v, s.scenes[size_t(r->v.scene)].nTris).total;
  const size_t day = day_layout(r->d).total;
  return r->series ? series_layout(*r, day).total : day;
}

// one slot's graph: table up, counter reset, trace, reduce, sums and status down
bool build_graph(Server& s, DaySlot& d, std::string& err) {
  if (d.exec) { cudaGraphExecDestroy(d.exec); d.exec = nullptr; }
  if (d.graph) { cudaGraphDestroy(d.graph); d.graph = nullptr; }
  if (!cuok(cudaGraphCreate(&d.graph, 0), err, "graph")) return false;
  cudaGraph_t g = d.graph;
  cudaGraphNode_t nHdr, nCtl, nBits, nStatus;
  uint32_t* status = d.dCtl + 1;
  void* aBits[] = {&d.dHdr, &d.dSegs, &d.dBits, &d.dCtl, &status};
  void* aRed[] = {&d.dHdr, &d.dSegs, &d.dBits, &d.dOut};
  cudaKernelNodeParams kb{};
  kb.func = reinterpret_cast<void*>(k_bits_batch); kb.gridDim = dim3(unsigned(s.gridBits)); kb.blockDim = dim3(256); kb.kernelParams = aBits;
  cudaKernelNodeParams kr{};
  kr.func = reinterpret_cast<void*>(k_reduce_batch); kr.gridDim = dim3((s.maxSensPerBatch + kReduceBatchBlock - 1) / kReduceBatchBlock); kr.blockDim = dim3(kReduceBatchBlock);
  kr.kernelParams = aRed;
  cudaMemsetParams ms{};
  ms.dst = d.dCtl; ms.value = 0; ms.elementSize = 4; ms.width = 2; ms.height = 1;
  bool ok = cuok(cudaGraphAddMemcpyNode1D(&nHdr, g, nullptr, 0, d.dHdr, d.hHdr, sizeof(BatchHdr), cudaMemcpyHostToDevice), err, "graph") &&
            cuok(cudaGraphAddMemcpyNode1D(&d.nSegs, g, &nHdr, 1, d.dSegs, d.hSegs, sizeof(Seg) * kMaxSegs, cudaMemcpyHostToDevice), err, "graph") &&
            cuok(cudaGraphAddMemsetNode(&nCtl, g, &d.nSegs, 1, &ms), err, "graph") &&
            cuok(cudaGraphAddKernelNode(&nBits, g, &nCtl, 1, &kb), err, "graph") &&
            cuok(cudaGraphAddKernelNode(&d.nReduce, g, &nBits, 1, &kr), err, "graph") &&
            cuok(cudaGraphAddMemcpyNode1D(&d.nOut, g, &d.nReduce, 1, d.hOut, d.dOut, sizeof(double) * s.outPoolDoubles, cudaMemcpyDeviceToHost), err, "graph") &&
            cuok(cudaGraphAddMemcpyNode1D(&nStatus, g, &d.nOut, 1, d.hStatus, status, 4, cudaMemcpyDeviceToHost), err, "graph") &&
            cuok(cudaGraphInstantiate(&d.exec, g, 0), err, "graph instantiate");
  return ok;
}

void free_pools(Server& s) {
  for (DaySlot& d : s.day) {
    if (d.exec) cudaGraphExecDestroy(d.exec);
    if (d.graph) cudaGraphDestroy(d.graph);
    cudaFree(d.dBits); cudaFree(d.dOut);
    if (d.hOut) cudaFreeHost(d.hOut);
    d.graph = nullptr; d.exec = nullptr; d.dBits = nullptr; d.dOut = nullptr; d.hOut = nullptr;
  }
  cudaFree(s.dCls); cudaFree(s.dDist);
  s.dCls = nullptr; s.dDist = nullptr;
  s.used -= s.poolBytes;
  s.poolBytes = 0;
}

// the pools that depend on the tuning: each day slot's bits and sums (device) and sums (pinned), and its graph; the
// views scratch
bool make_pools(Server& s, std::string& err) {
  free_pools(s);
  s.maxSensPerBatch = std::min<uint32_t>(kMaxSegs * s.chunkSensors, 1u << 20);
  // bits of a batch: rays / 32 words, plus a word per sensor and segment for the rounding up of each chunk's words
  s.bitsPoolWords = size_t(s.batchRays / 32) + size_t(s.maxSensPerBatch) * 2;
  s.outPoolDoubles = size_t(s.maxSensPerBatch) * kMaxQ;
  s.viewCap = std::max<uint64_t>(s.viewRays, uint64_t(1) << 16);
  for (DaySlot& d : s.day)
    if (!cuok(cudaMalloc(&d.dBits, s.bitsPoolWords * 4), err, "batch pool") || !cuok(cudaMalloc(&d.dOut, s.outPoolDoubles * 8), err, "batch pool") ||
        !cuok(cudaMallocHost(&d.hOut, s.outPoolDoubles * 8), err, "pinned pool") || !build_graph(s, d, err))
      return false;
  if (!cuok(cudaMalloc(&s.dCls, s.viewCap), err, "views scratch") || !cuok(cudaMalloc(&s.dDist, s.viewCap * 4), err, "views scratch"))
    return false;
  s.poolBytes = kSlots * (s.bitsPoolWords * 4 + s.outPoolDoubles * 8) + s.viewCap * 5;
  s.used += s.poolBytes;
  return true;
}

void finish(Server& s, Request* r, bool ok, const std::string& err) {
  if (r->dev) cudaFreeAsync(r->dev, s.st);   // after every item queued on the work stream, the last users of it
  s.used -= r->devBytes;
  r->dev = nullptr;
  r->devBytes = 0;
  r->tDone = Clock::now();
  r->failed = !ok;
  r->err = err;
  r->done = true;
  if (ok) s.latencies.push_back(std::chrono::duration<double>(r->tDone - r->tSubmit).count());
}

// a request's inputs up on the upload stream, into memory from the server's pool (r->devBytes, reserved at admission)
bool upload(Server& s, Request* r, std::string& err) {
  if (!cuok(cudaMallocFromPoolAsync(&r->dev, r->devBytes, s.pool, s.up), err, "request memory")) { r->dev = nullptr; return false; }
  char* b = static_cast<char*>(r->dev);
  bool ok = true;
  if (r->kind == 0) {
    const kgb_daylight_request& d = r->d;
    const DayLayout L = day_layout(d);
    r->w64.resize(size_t(d.nQ) * d.nDir);
    const float* W = static_cast<const float*>(d.W);
    for (size_t k = 0; k < r->w64.size(); ++k) r->w64[k] = double(W[k]);
    ok = cuok(cudaMemcpyAsync(b, d.P, L.offN, cudaMemcpyHostToDevice, s.up), err, "upload") &&
         cuok(cudaMemcpyAsync(b + L.offN, d.N, L.offN, cudaMemcpyHostToDevice, s.up), err, "upload") &&
         cuok(cudaMemcpyAsync(b + L.offD, d.D, size_t(d.nDir) * 12, cudaMemcpyHostToDevice, s.up), err, "upload") &&
         cuok(cudaMemcpyAsync(b + L.offW, r->w64.data(), r->w64.size() * 8, cudaMemcpyHostToDevice, s.up), err, "upload");
    if (ok) launch_ray_table(reinterpret_cast<const float*>(b + L.offD), d.nDir, b + L.offTab, s.up);
    if (ok && r->series) {   // the series inputs, and S^T split into its bf16 pieces once for every batch of the request
      const kgb_series_in& in = r->sq.in;
      const size_t T = size_t(in.T), P = size_t(in.P);
      const SeriesLayout S = series_layout(*r, L.total);
      ok = cuok(cudaMemcpyAsync(b + S.offS, in.S, P * T * 4, cudaMemcpyHostToDevice, s.up), err, "upload") &&
           cuok(cudaMemcpyAsync(b + S.offG, in.g, T * 4, cudaMemcpyHostToDevice, s.up), err, "upload") &&
           cuok(cudaMemcpyAsync(b + S.offCsr, r->csr.data(), r->csr.size() * 4, cudaMemcpyHostToDevice, s.up), err, "upload") &&
           cuok(cudaMemcpyAsync(b + S.offWsky, in.wsky, size_t(in.nSky) * 4, cudaMemcpyHostToDevice, s.up), err, "upload") &&
           cuok(cudaMemcpyAsync(b + S.offSunCol, r->sunOfCol.data(), T * 4, cudaMemcpyHostToDevice, s.up), err, "upload") &&
           (!in.nSun || (cuok(cudaMemcpyAsync(b + S.offSunVec, in.sunVec, size_t(in.nSun) * 12, cudaMemcpyHostToDevice, s.up), err, "upload") &&
                         cuok(cudaMemcpyAsync(b + S.offSunW, in.sunW, size_t(in.nSun) * 4, cudaMemcpyHostToDevice, s.up), err, "upload")));
      if (ok) {
        SeriesTcPlan p{};
        p.T = uint32_t(T); p.Kp = r->Kp; p.s = b + S.offSt;
        SeriesOperands o{};
        o.P = uint32_t(P); o.S = reinterpret_cast<const float*>(b + S.offS); o.g = reinterpret_cast<const float*>(b + S.offG);
        o.rebuildS = true; o.buildV = false;
        build_series_operands(p, o, s.up);
      }
    }
  } else {
    const kgb_views_request& v = r->v;
    const ViewLayout L = view_layout(v, s.scenes[size_t(v.scene)].nTris);
    ok = cuok(cudaMemcpyAsync(b, v.P, L.offN, cudaMemcpyHostToDevice, s.up), err, "upload") &&
         cuok(cudaMemcpyAsync(b + L.offN, v.N, L.offN, cudaMemcpyHostToDevice, s.up), err, "upload") &&
         cuok(cudaMemcpyAsync(b + L.offRow, r->rowSin.data(), size_t(v.view.nEl) * 8, cudaMemcpyHostToDevice, s.up), err, "upload") &&
         cuok(cudaMemcpyAsync(b + L.offW, r->wRow.data(), size_t(v.view.nEl) * 8, cudaMemcpyHostToDevice, s.up), err, "upload") &&
         (!v.label || cuok(cudaMemcpyAsync(b + L.offLab, v.label, s.scenes[size_t(v.scene)].nTris, cudaMemcpyHostToDevice, s.up), err, "upload"));
  }
  s.upPending = true;
  return ok && cuok(cudaGetLastError(), err, "upload");
}

// admission: pending requests in arrival order while the budget allows (a lone request always runs), inputs uploaded
void admit(Server& s) {
  std::vector<Request*> admitted;
  {
    std::lock_guard<std::mutex> lk(s.m);
    while (!s.pending.empty()) {
      Request* r = s.pending.front();
      const uint64_t need = request_bytes(s, r);
      if (s.used + need > s.budget && !s.active.empty()) break;
      s.pending.pop_front();
      r->devBytes = need;
      s.used += need;
      admitted.push_back(r);
      s.active.push_back(r);
    }
  }
  if (admitted.empty()) return;
  for (Request* r : admitted) {
    std::string err;
    if (!upload(s, r, err)) {
      cudaStreamSynchronize(s.up);   // none of its copies still in flight when its memory goes back
      std::lock_guard<std::mutex> lk(s.m);
      finish(s, r, false, err);
      s.active.erase(std::remove(s.active.begin(), s.active.end(), r), s.active.end());
    }
  }
  cudaEventRecord(s.upDone, s.up);
  s.doneCv.notify_all();
}

// the work stream waits for the uploads issued so far before its next item
bool order_after_uploads(Server& s, std::string& err) {
  if (!s.upPending) return true;
  s.upPending = false;
  return cuok(cudaStreamWaitEvent(s.st, s.upDone, 0), err, "upload wait");
}

double priority(const Server& s, const Request* r, Clock::time_point now) {
  const double age = std::chrono::duration<double>(now - r->tSubmit).count();
  if (age > s.oldSeconds) return -1e9 - age;   // the oldest first, before every younger request
  const double rem = double(r->nSensors - r->nextSensor) * double(r->raysPerSensor) * s.cost[r->kind];
  return rem / (age + s.ageSeconds);
}

// The batch's series, after its graph on the work stream: each series chunk's V pieces from the batch's visibility
// bits and its ground sums (quantity gQ), then every chunk's contraction in one grouped launch, then their rows and the
// series' status word down into pinned memory.
bool launch_series(Server& s, DaySlot& d, std::string& err) {
  std::vector<SeriesTcPlan> plans;
  for (size_t j = 0; j < d.parts.size(); ++j) {
    const Part& p = d.parts[j];
    if (!p.r->series) continue;
    const Seg& g = d.hSegs[j];
    const kgb_series_in& in = p.r->sq.in;
    const char* b = static_cast<const char*>(p.r->dev);
    const SeriesLayout L = series_layout(*p.r, day_layout(p.r->d).total);
    SeriesTcPlan pl{};
    pl.nc = p.n; pl.T = uint32_t(in.T); pl.Kp = p.r->Kp; pl.sun0 = in.sun0; pl.numSMs = s.numSMs;
    pl.v = static_cast<char*>(d.dV) + p.vOff;
    pl.s = const_cast<char*>(b) + L.offSt;
    pl.sunOfCol = reinterpret_cast<const int32_t*>(b + L.offSunCol);
    pl.sunVec = reinterpret_cast<const float*>(b + L.offSunVec);
    pl.sunW = reinterpret_cast<const float*>(b + L.offSunW);
    pl.bits = d.dBits + g.bitsOff;
    pl.N = g.N;
    pl.E = d.dE + p.eOff;
    pl.status = d.dCtl + 1;
    SeriesOperands o{};
    o.P = uint32_t(in.P); o.D = g.D;
    o.patchFirst = reinterpret_cast<const int32_t*>(b + L.offCsr); o.patchDirs = o.patchFirst + in.P + 1;
    o.wsky = reinterpret_cast<const float*>(b + L.offWsky);
    o.G64 = d.dOut + g.outOff + size_t(p.r->sq.gQ) * p.n;
    o.rebuildS = false;
    build_series_operands(pl, o, s.st);
    plans.push_back(pl);
  }
  if (!cuok(cudaGetLastError(), err, "series operands")) return false;
  if (const char* why = series_tc_group(plans.data(), uint32_t(plans.size()), s.st)) { err = why; return false; }
  size_t eEnd = 0;
  for (const Part& p : d.parts) if (p.r->series) eEnd = p.eOff + size_t(p.n) * uint32_t(p.r->sq.in.T);
  return cuok(cudaGetLastError(), err, "series launch") &&
         cuok(cudaMemcpyAsync(d.hE, d.dE, eEnd * 4, cudaMemcpyDeviceToHost, s.st), err, "series rows") &&
         cuok(cudaMemcpyAsync(d.hSeriesStatus, d.dCtl + 1, 4, cudaMemcpyDeviceToHost, s.st), err, "series status");
}

// a daylight batch of the given parts into slot k, launched on the work stream
bool launch_day(Server& s, int k, const std::vector<Part>& parts, std::string& err) {
  DaySlot& d = s.day[k];
  uint32_t tasks = 0, sens = 0;
  size_t bits = 0, out = 0;
  d.rays = 0;
  for (size_t j = 0; j < parts.size(); ++j) {
    const Part& p = parts[j];
    const kgb_daylight_request& q = p.r->d;
    const DScene& sc = s.scenes[size_t(q.scene)];
    const char* b = static_cast<const char*>(p.r->dev);
    const DayLayout L = day_layout(q);
    Seg& g = d.hSegs[j];
    g.nodes = static_cast<const Node8*>(sc.nodes); g.tris = static_cast<const TriRec*>(sc.tris); g.nNodes = sc.nNodes;
    g.P = reinterpret_cast<const float*>(b) + 3 * size_t(p.i0); g.N = reinterpret_cast<const float*>(b + L.offN) + 3 * size_t(p.i0);
    g.D = reinterpret_cast<const float*>(b + L.offD); g.tab = reinterpret_cast<const RayDir*>(b + L.offTab);
    g.W = reinterpret_cast<const double*>(b + L.offW);
    g.nDir = q.nDir; g.nWords = (q.nDir + 31) / 32; g.n = p.n; g.rayFlags = q.rayFlags; g.nQ = q.nQ; g.useCosMask = q.useCosMask;
    g.taskBase = tasks; g.sensBase = sens; g.bitsOff = uint32_t(bits); g.outOff = uint32_t(out);
    tasks += (p.n + 31) / 32 * g.nWords;
    sens += p.n;
    bits += size_t(g.nWords) * p.n;
    out += size_t(q.nQ) * p.n;
    d.rays += uint64_t(p.n) * q.nDir;
  }
  if (parts.empty() || parts.size() > kMaxSegs || bits > s.bitsPoolWords || out > s.outPoolDoubles || sens > s.maxSensPerBatch) {
    err = "internal: batch beyond its pools";
    return false;
  }
  d.hHdr->nSegs = uint32_t(parts.size()); d.hHdr->nTasks = tasks; d.hHdr->nSens = sens;
  d.parts = parts;
  // the series chunks' places in the slot's pools (the packer kept them within kSeriesVBytes / kSeriesEBytes)
  d.anySeries = false;
  size_t vUsed = 0, eUsed = 0;
  uint32_t nSeries = 0;
  for (Part& p : d.parts)
    if (p.r->series) {
      p.vOff = vUsed; p.eOff = eUsed;
      vUsed += up256(size_t(3) * p.n * p.r->Kp * 2);
      eUsed += (size_t(p.n) * uint32_t(p.r->sq.in.T) + 63) / 64 * 64;
      ++nSeries;
      d.anySeries = true;
    }
  if (vUsed > kSeriesVBytes || eUsed * 4 > kSeriesEBytes || nSeries > kMaxSeriesGroup) {
    err = "internal: batch beyond its series pools";
    d.parts.clear();
    return false;
  }
  void* aRed[] = {&d.dHdr, &d.dSegs, &d.dBits, &d.dOut};
  cudaKernelNodeParams kr{};
  kr.func = reinterpret_cast<void*>(k_reduce_batch); kr.gridDim = dim3((sens + kReduceBatchBlock - 1) / kReduceBatchBlock); kr.blockDim = dim3(kReduceBatchBlock); kr.kernelParams = aRed;
  const bool ok =
      cuok(cudaGraphExecMemcpyNodeSetParams1D(d.exec, d.nSegs, d.dSegs, d.hSegs, sizeof(Seg) * parts.size(), cudaMemcpyHostToDevice), err, "batch table") &&
      cuok(cudaGraphExecKernelNodeSetParams(d.exec, d.nReduce, &kr), err, "batch reduce") &&
      cuok(cudaGraphExecMemcpyNodeSetParams1D(d.exec, d.nOut, d.hOut, d.dOut, sizeof(double) * out, cudaMemcpyDeviceToHost), err, "batch sums") &&
      order_after_uploads(s, err) && cuok(cudaEventRecord(d.ev[0], s.st), err, "batch") && cuok(cudaGraphLaunch(d.exec, s.st), err, "batch graph") &&
      (!d.anySeries || launch_series(s, d, err)) && cuok(cudaEventRecord(d.ev[1], s.st), err, "batch");
  if (!ok) d.parts.clear();
  return ok;
}

// a views chunk of one request into slot k: the single-request view kernels on its device arrays and the views scratch
bool launch_views(Server& s, int k, const Part& p, std::string& err) {
  ViewSlot& vs = s.view[k];
  const kgb_views_request& v = p.r->v;
  const DScene& sc = s.scenes[size_t(v.scene)];
  const ViewLayout L = view_layout(v, sc.nTris);
  const uint64_t K = p.r->raysPerSensor;
  const char* b = static_cast<const char*>(p.r->dev);
  const double rad = v.view.north * KGB_PI_D / 180;
  ViewArgs a{};
  a.nodes = static_cast<const Node8*>(sc.nodes); a.tris = static_cast<const TriRec*>(sc.tris); a.nNodes = sc.nNodes;
  a.P = reinterpret_cast<const float*>(b); a.N = reinterpret_cast<const float*>(b + L.offN);
  a.first = p.i0; a.n = p.n; a.out0 = 0; a.stride = p.n; a.i0 = p.i0;
  a.K = uint32_t(K); a.nWords = uint32_t((K + 31) / 32); a.nAz = v.view.nAz; a.nEl = v.view.nEl; a.rayFlags = v.rayFlags;
  a.rowSin = reinterpret_cast<const float*>(b + L.offRow); a.az0 = v.view.az0; a.dAz = v.view.dAz; a.groundZ = v.view.groundZ;
  a.cosN = float(std::cos(rad)); a.sinN = float(std::sin(rad));
  a.world = v.view.world ? 1 : 0; a.cull = v.view.cull ? 1 : 0; a.jitter = v.view.jitter ? 1 : 0; a.nS = v.view.nS; a.back = v.view.back ? 1 : 0;
  a.vground = v.view.vground ? 1 : 0;
  a.label = v.label ? reinterpret_cast<const uint8_t*>(b + L.offLab) : nullptr;
  a.cls = s.dCls; a.dist = s.dDist;
  a.counter = vs.dCtl; a.status = vs.dCtl + 1;
  ViewReduceArgs ra{};
  ra.cls = a.cls; ra.dist = a.dist; ra.nc = p.n; ra.K = uint32_t(K); ra.nAz = v.view.nAz; ra.nEl = v.view.nEl; ra.nClass = v.nClass;
  ra.nReach = v.nReach; ra.glazing = v.glazing ? 1 : 0; ra.iso = v.isoDim ? 1 : 0; ra.NA = views_NA(v);
  ra.wRow = reinterpret_cast<const double*>(b + L.offW); ra.farDist = float(v.farDist); ra.lnFar = std::log(v.farDist);
  for (uint32_t j = 0; j < v.nReach; ++j) ra.reach[j] = v.reach[j];
  ra.isoDim = v.isoDim; ra.world = a.world; ra.jitter = a.jitter; ra.i0 = p.i0; ra.nS = v.view.nS; ra.back = a.back;
  ra.az0 = v.view.az0; ra.dAz = v.view.dAz; ra.rowSin = a.rowSin; ra.out = s.dViewOut;
  vs.part = p;
  vs.NA = ra.NA;
  const size_t tasks = (size_t(p.n) + 31) / 32 * a.nWords;
  const int grid = int(std::min<size_t>(size_t(s.gridView), (tasks + 7) / 8));
  if (!order_after_uploads(s, err) || !cuok(cudaEventRecord(vs.ev[0], s.st), err, "views") || !cuok(cudaMemsetAsync(vs.dCtl, 0, 8, s.st), err, "views"))
    return false;
  launch_view(a, grid, s.st);
  launch_reduce_view(ra, s.st);
  return cuok(cudaGetLastError(), err, "views launch") &&
         cuok(cudaMemcpyAsync(vs.hOut, s.dViewOut, size_t(p.n) * ra.NA * 8, cudaMemcpyDeviceToHost, s.st), err, "views") &&
         cuok(cudaMemcpyAsync(vs.hStatus, vs.dCtl + 1, 4, cudaMemcpyDeviceToHost, s.st), err, "views") &&
         cuok(cudaEventRecord(vs.ev[1], s.st), err, "views");
}

// sensors of a views request in one chunk: the views rays the scratch holds, at most kMaxViewChunk
uint32_t views_chunk(const Server& s, const Request* r) {
  const uint64_t n = std::min<uint64_t>(kMaxViewChunk, std::max<uint64_t>(1, s.viewRays / r->raysPerSensor));
  return uint32_t(std::min<uint64_t>(n, r->nSensors - r->nextSensor));
}

void account(Server& s, Request* r, uint32_t n, bool ok, const std::string& err) {
  std::lock_guard<std::mutex> lk(s.m);
  r->doneSensors += n;
  if (!r->done && !ok) finish(s, r, false, err);
  else if (!r->done && r->doneSensors == r->nSensors) finish(s, r, true, "");
  s.active.erase(std::remove_if(s.active.begin(), s.active.end(), [](Request* q) { return q->done; }), s.active.end());
}

bool slot_busy(const Server& s, int kind, int k) {
  for (const auto& f : s.inflight) if (f.first == kind && f.second == k) return true;
  return false;
}

// the next work item by priority; false when there is nothing to launch
bool launch_next(Server& s) {
  const Clock::time_point now = Clock::now();
  std::vector<std::pair<double, Request*>> cand;
  {
    std::lock_guard<std::mutex> lk(s.m);
    for (Request* r : s.active)
      if (!r->done && r->nextSensor < r->nSensors) cand.emplace_back(priority(s, r, now), r);
  }
  if (cand.empty()) return false;
  std::sort(cand.begin(), cand.end(), [](const auto& a, const auto& b) { return a.first < b.first || (a.first == b.first && a.second->ticket < b.second->ticket); });
  const int kind = cand.front().second->kind;
  int k = 0;
  while (k < kSlots && slot_busy(s, kind, k)) ++k;
  if (k == kSlots) return false;
  std::string err;
  if (kind == 1) {
    Request* r = cand.front().second;
    const uint32_t n = views_chunk(s, r);
    if (uint64_t(n) * r->raysPerSensor > s.viewCap) {
      r->nextSensor = r->nSensors;
      account(s, r, 0, false, "views: one sensor's rays exceed the views scratch (raise the views chunk rays)");
      return true;
    }
    const Part p{r, r->nextSensor, n};
    r->nextSensor += n;
    if (!launch_views(s, k, p, err)) { account(s, r, n, false, err); return true; }
    s.inflight.emplace_back(1, k);
    std::lock_guard<std::mutex> lk(s.m);
    ++s.items;
    return true;
  }
  // daylight: chunks of the daylight candidates in priority order until the batch is full
  std::vector<Part> parts;
  uint64_t rays = 0;
  size_t bits = 0, out = 0, vUsed = 0, eUsed = 0;
  uint32_t sens = 0, nSeries = 0;
  for (const auto& c : cand) {
    Request* r = c.second;
    if (r->kind != 0) continue;
    if (r->series && nSeries >= kMaxSeriesGroup) continue;   // the grouped launch is full: other requests may still fit
    const size_t perSensor = (r->d.nDir + 31) / 32;
    while (r->nextSensor < r->nSensors && parts.size() < kMaxSegs && rays < s.batchRays && (!r->series || nSeries < kMaxSeriesGroup)) {
      // a chunk, cut to what is left of the batch's rays and of its pools (a series chunk also to the series pools)
      uint64_t fit = std::min({uint64_t(s.chunkSensors), uint64_t(r->nSensors - r->nextSensor),
                               (s.batchRays - rays + r->d.nDir - 1) / r->d.nDir, uint64_t((s.bitsPoolWords - bits) / perSensor),
                               uint64_t((s.outPoolDoubles - out) / r->d.nQ), uint64_t(s.maxSensPerBatch - sens)});
      if (r->series) {
        const size_t vRow = size_t(6) * r->Kp, eRow = size_t(4) * uint32_t(r->sq.in.T);
        const size_t vLeft = kSeriesVBytes - vUsed > 256 ? kSeriesVBytes - vUsed - 256 : 0, eLeft = kSeriesEBytes - eUsed > 256 ? kSeriesEBytes - eUsed - 256 : 0;
        fit = std::min<uint64_t>({fit, vLeft / vRow, eLeft / eRow});
      }
      if (fit == 0) break;
      const uint32_t n = uint32_t(fit);
      const size_t words = perSensor * n;
      parts.push_back(Part{r, r->nextSensor, n});
      r->nextSensor += n;
      rays += uint64_t(n) * r->d.nDir;
      bits += words;
      out += size_t(r->d.nQ) * n;
      sens += n;
      if (r->series) {   // as launch_day places them
        vUsed += up256(size_t(3) * n * r->Kp * 2);
        eUsed += ((size_t(n) * uint32_t(r->sq.in.T) + 63) / 64 * 64) * 4;
        ++nSeries;
      }
    }
    if (parts.size() >= kMaxSegs || rays >= s.batchRays) break;
    if (parts.empty()) {   // not one sensor of the top request fits an empty batch: it can never run
      r->nextSensor = r->nSensors;
      account(s, r, 0, false, r->series ? "daylight: one sensor's series row exceeds the batch's series pools" :
                                          "daylight: one sensor's direction words exceed the batch pools (raise the batch rays)");
      return true;
    }
  }
  if (parts.empty()) return false;
  if (!launch_day(s, k, parts, err)) {
    for (const Part& p : parts) account(s, p.r, p.n, false, err);
    return true;
  }
  s.inflight.emplace_back(0, k);
  std::lock_guard<std::mutex> lk(s.m);
  ++s.items;
  return true;
}

// the oldest item, whose end event has been reached (or failed): results out to the requests, the cost estimate updated
void complete(Server& s, int kind, int k, cudaError_t q) {
  std::string err;
  bool ok = cuok(q, err, kind == 0 ? "batch" : "views chunk");
  cudaEvent_t* ev = kind == 0 ? s.day[k].ev : s.view[k].ev;
  float ms = 0;
  const uint64_t rays = kind == 0 ? s.day[k].rays : uint64_t(s.view[k].part.n) * s.view[k].part.r->raysPerSensor;
  if (ok && cudaEventElapsedTime(&ms, ev[0], ev[1]) == cudaSuccess && rays && ms > 0) {
    s.cost[kind] = 0.7 * s.cost[kind] + 0.3 * (double(ms) * 1e-3 / double(rays));
    std::lock_guard<std::mutex> lk(s.m);
    s.gpuSec[kind] += double(ms) * 1e-3;
    s.kindRays[kind] += double(rays);
  }
  if (kind == 0) {
    DaySlot& d = s.day[k];
    if (ok && *d.hStatus) { ok = false; err = "batch: traversal stack overflow or visit limit"; }
    if (ok && d.anySeries && (*d.hSeriesStatus & kStatusTimeout)) { ok = false; err = "batch: the series' tensor-core pipeline timed out waiting"; }
    for (size_t j = 0; j < d.parts.size(); ++j) {
      const Part& p = d.parts[j];
      const Seg& g = d.hSegs[j];
      if (ok && !p.r->done) {
        for (uint32_t qq = 0; qq < g.nQ; ++qq)
          std::memcpy(p.r->d.out + size_t(qq) * p.r->nSensors + p.i0, d.hOut + g.outOff + size_t(qq) * p.n, size_t(p.n) * 8);
        if (p.r->series) {
          const size_t T = size_t(p.r->sq.in.T);
          std::memcpy(p.r->sq.E + size_t(p.i0) * T, d.hE + p.eOff, size_t(p.n) * T * 4);
        }
      }
      account(s, p.r, p.n, ok, err);
    }
    d.parts.clear();
  } else {
    ViewSlot& vs = s.view[k];
    const Part& p = vs.part;
    if (ok && *vs.hStatus) { ok = false; err = "views chunk: traversal stack overflow"; }
    if (ok && !p.r->done) std::memcpy(p.r->v.out + size_t(p.i0) * vs.NA, vs.hOut, size_t(p.n) * vs.NA * 8);
    account(s, p.r, p.n, ok, err);
  }
  {
    std::lock_guard<std::mutex> lk(s.m);
    if (ok) s.rays += rays;
  }
  s.doneCv.notify_all();
}

void loop(Server* s) {
  cudaSetDevice(s->device);
  for (;;) {
    {
      std::unique_lock<std::mutex> lk(s->m);
      s->cv.wait(lk, [&] { return s->stop || !s->pending.empty() || !s->active.empty() || !s->inflight.empty(); });
      if (s->stop) return;
    }
    admit(*s);
    const bool idle = s->inflight.empty();
    while (s->inflight.size() < kDepth && launch_next(*s)) {}
    if (idle && !s->inflight.empty()) s->queuedSince = Clock::now();
    if (s->inflight.empty()) {   // admitted requests that all failed, or nothing launchable yet
      std::unique_lock<std::mutex> lk(s->m);
      s->cv.wait_for(lk, std::chrono::milliseconds(1));
      continue;
    }
    const std::pair<int, int> f = s->inflight.front();
    const cudaError_t q = cudaEventQuery(f.first == 0 ? s->day[f.second].ev[1] : s->view[f.second].ev[1]);
    if (q == cudaErrorNotReady) { std::this_thread::sleep_for(std::chrono::microseconds(100)); continue; }
    s->inflight.pop_front();
    if (s->inflight.empty()) {
      std::lock_guard<std::mutex> lk(s->m);
      s->queuedSec += std::chrono::duration<double>(Clock::now() - s->queuedSince).count();
    }
    complete(*s, f.first, f.second, q);
  }
}

// one daylight batch through slot 0, waited for (the autotuner's calibration); its parts' outputs written
bool run_batch_now(Server& s, const std::vector<Part>& parts, double& sec, std::string& err) {
  const auto t0 = Clock::now();
  if (!launch_day(s, 0, parts, err)) return false;
  const cudaError_t q = cudaEventSynchronize(s.day[0].ev[1]);
  sec = std::chrono::duration<double>(Clock::now() - t0).count();
  if (!cuok(q, err, "calibration batch")) return false;
  if (*s.day[0].hStatus) { err = "calibration batch: traversal stack overflow"; return false; }
  float ms = 0;
  if (cudaEventElapsedTime(&ms, s.day[0].ev[0], s.day[0].ev[1]) == cudaSuccess && s.day[0].rays && ms > 0) s.cost[0] = double(ms) * 1e-3 / double(s.day[0].rays);
  s.day[0].parts.clear();
  return true;
}

// a views request's chunks one after another in slot 0 at the server's views chunk size; its rays per second
bool run_views_now(Server& s, Request& r, double& rate, std::string& err) {
  const auto t0 = Clock::now();
  uint64_t rays = 0;
  for (uint32_t i0 = 0; i0 < r.nSensors;) {
    r.nextSensor = i0;
    const uint32_t n = views_chunk(s, &r);
    if (uint64_t(n) * r.raysPerSensor > s.viewCap) { err = "calibration views chunk beyond the scratch"; return false; }
    if (!launch_views(s, 0, Part{&r, i0, n}, err)) return false;
    if (!cuok(cudaEventSynchronize(s.view[0].ev[1]), err, "calibration views chunk")) return false;
    if (*s.view[0].hStatus) { err = "calibration views chunk: traversal stack overflow"; return false; }
    rays += uint64_t(n) * r.raysPerSensor;
    i0 += n;
  }
  rate = double(rays) / std::chrono::duration<double>(Clock::now() - t0).count();
  return true;
}

// the views chunk size: one synthetic fov 120 request (2-degree cells, 40,960 sensors: 147 M rays, the size of the
// larger views requests) from the same sensors, run whole at each candidate size; the size with the most rays per
// second, or a smaller one within 1 % of it. (Picking the smallest within 5 % on a 16 k-sensor request chose 2^26 rays,
// and the serving config's views then ran 5 % slower than at 2^27.)
bool tune_views(Server& s, const std::vector<float>& P, const std::vector<float>& N, uint32_t nSens, std::string& err) {
  const uint32_t nAz = 60, nEl = 60;   // 3600 rays a sensor
  std::vector<float> rowSin(2 * nEl);
  std::vector<double> wRow(nEl);
  for (uint32_t j = 0; j < nEl; ++j) {
    const double lo = (-60.0 + 2.0 * j) * KGB_PI_D / 180, hi = (-58.0 + 2.0 * j) * KGB_PI_D / 180;
    rowSin[2 * j] = float(std::sin(lo)); rowSin[2 * j + 1] = float(std::sin(hi));
    wRow[j] = std::sin(hi) - std::sin(lo);
  }
  std::vector<double> out(size_t(nSens) * (3 * 1 + 1));
  struct Trial { uint64_t rays; double rate; };
  std::vector<Trial> trials;
  const uint64_t keep = s.viewRays;
  for (uint64_t vr : {uint64_t(1) << 25, uint64_t(1) << 26, uint64_t(1) << 27, uint64_t(1) << 28}) {
    s.viewRays = vr;
    if (!make_pools(s, err)) return false;
    Request r;
    r.kind = 1;
    r.v = kgb_views_request{};
    r.v.scene = 0; r.v.nSensors = nSens; r.v.P = P.data(); r.v.N = N.data(); r.v.label = nullptr;
    r.v.view.nAz = nAz; r.v.view.nEl = nEl; r.v.view.az0 = -60.f; r.v.view.dAz = 2.f; r.v.view.rowSin = rowSin.data();
    r.v.view.jitter = 1; r.v.view.vground = 1; r.v.view.nS = 1; r.v.view.groundZ = -1e4f;
    r.v.rayFlags = KGB_RAY_DISABLE_ANYHIT; r.v.wRow = wRow.data(); r.v.nClass = 1; r.v.farDist = 1000.0; r.v.out = out.data();
    r.rowSin = rowSin; r.wRow = wRow;
    r.nSensors = nSens;
    r.raysPerSensor = uint64_t(nAz) * nEl;
    r.devBytes = request_bytes(s, &r);
    if (!upload(s, &r, err)) return false;
    cudaEventRecord(s.upDone, s.up);
    double best = 0;
    for (int rep = 0; rep < 2; ++rep) {   // the first run warms the caches
      double rate = 0;
      if (!run_views_now(s, r, rate, err)) { cudaFreeAsync(r.dev, s.st); return false; }
      best = std::max(best, rate);
    }
    cudaFreeAsync(r.dev, s.st);
    s.view[0].part = Part{nullptr, 0, 0};   // the calibration request is gone; nothing refers to it
    trials.push_back(Trial{vr, best});
  }
  double top = 0;
  for (const Trial& t : trials) top = std::max(top, t.rate);
  s.viewRays = keep;
  for (const Trial& t : trials)
    if (t.rate >= 0.99 * top) { s.viewRays = t.rays; break; }   // the candidates run smallest first
  return true;
}

// the autotuner: calibration batches of one synthetic request on scene 0 (its first sensors against a fixed
// direction table); keeps the chunk size and batch size with the most rays per second, or the smallest batch within
// 5 % of that rate (a smaller batch is a shorter wait for requests that arrive while it runs); then the views chunk
// size the same way (tune_views)
bool autotune(Server& s, std::string& err) {
  const DScene& sc = s.scenes[0];
  if (!sc.nNodes) return true;
  const uint32_t nDir = 1024, nSens = 65536;
  std::vector<float> P(3 * nSens), N(3 * nSens), D(3 * nDir), W(nDir, 1.f);
  std::vector<double> out(nSens);
  // sensors on a horizontal grid over the middle of the scene's root box (its children's lowest x and y), looking up;
  // directions over the sky
  float p0[2] = {INFINITY, INFINITY};
  std::vector<float> node(kNodeWords);
  if (!cuok(cudaMemcpy(node.data(), sc.nodes, kNodeBytes, cudaMemcpyDeviceToHost), err, "autotune")) return false;
  for (int k = 0; k < 8; ++k) { p0[0] = std::min(p0[0], node[4 + k]); p0[1] = std::min(p0[1], node[4 + 16 + k]); }
  if (!std::isfinite(p0[0]) || !std::isfinite(p0[1])) p0[0] = p0[1] = 0.f;
  for (uint32_t i = 0; i < nSens; ++i) {
    P[3 * i] = p0[0] * 0.5f + float(i % 256); P[3 * i + 1] = p0[1] * 0.5f + float(i / 256); P[3 * i + 2] = 1.f;
    N[3 * i] = 0; N[3 * i + 1] = 0; N[3 * i + 2] = 1;
  }
  for (uint32_t d = 0; d < nDir; ++d) {
    const double z = 0.05 + 0.9 * (d + 0.5) / nDir, a = 2.399963 * d, r = std::sqrt(1 - z * z);
    D[3 * d] = float(r * std::sin(a)); D[3 * d + 1] = float(r * std::cos(a)); D[3 * d + 2] = float(z);
  }
  struct Trial { uint32_t chunk; uint64_t rays; double rate; };
  std::vector<Trial> trials;
  for (uint32_t chunk : {2048u, 8192u, 32768u})
    for (uint64_t br : {uint64_t(1) << 26, uint64_t(1) << 27, uint64_t(1) << 28}) {
      s.chunkSensors = chunk;
      s.batchRays = br;
      if (!make_pools(s, err)) return false;
      Request r;
      r.kind = 0;
      r.d = kgb_daylight_request{0, nSens, nDir, 1, P.data(), N.data(), D.data(), W.data(), 1u, KGB_RAY_TERMINATE_ON_FIRST_HIT | KGB_RAY_DISABLE_ANYHIT, out.data()};
      r.nSensors = nSens;
      r.raysPerSensor = nDir;
      r.devBytes = request_bytes(s, &r);
      if (!upload(s, &r, err)) return false;
      cudaEventRecord(s.upDone, s.up);
      double best = 0;
      for (int rep = 0; rep < 2; ++rep) {   // the first run warms the caches and the graph
        std::vector<Part> parts;
        uint64_t acc = 0;
        uint32_t sens = 0;
        for (uint32_t i = 0; i < nSens && parts.size() < kMaxSegs && acc < br && sens + chunk <= s.maxSensPerBatch; i += chunk) {
          const uint32_t c = std::min(chunk, nSens - i);
          parts.push_back(Part{&r, i, c});
          acc += uint64_t(c) * nDir;
          sens += c;
        }
        double sec = 0;
        if (!run_batch_now(s, parts, sec, err)) { cudaFreeAsync(r.dev, s.st); return false; }
        best = std::max(best, double(acc) / sec);
      }
      cudaFreeAsync(r.dev, s.st);
      trials.push_back(Trial{chunk, br, best});
    }
  double top = 0;
  for (const Trial& t : trials) top = std::max(top, t.rate);
  Trial pick = trials.front();
  bool have = false;
  for (const Trial& t : trials)
    if (t.rate >= 0.95 * top && (!have || t.rays < pick.rays || (t.rays == pick.rays && t.rate > pick.rate))) { pick = t; have = true; }
  s.chunkSensors = pick.chunk;
  s.batchRays = pick.rays;
  if (!tune_views(s, P, N, 40960, err)) return false;
  s.rays = 0;
  s.items = 0;
  s.gpuSec[0] = s.gpuSec[1] = s.kindRays[0] = s.kindRays[1] = s.queuedSec = 0;
  s.cost[1] = 3 * s.cost[0];
  return make_pools(s, err) && cuok(cudaStreamSynchronize(s.st), err, "autotune");
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
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) { delete s; set_error("no CUDA device"); return nullptr; }
  cudaGetDevice(&s->device);
  cudaDeviceGetAttribute(&s->numSMs, cudaDevAttrMultiProcessorCount, s->device);
  s->gridBits = s->numSMs * 4;
  s->gridView = s->numSMs * view_blocks_per_sm();
  s->budget = hbmBudgetBytes;
  cudaMemPoolProps props{};
  props.allocType = cudaMemAllocationTypePinned;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = s->device;
  if (!cuok(cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking), err, "stream") ||
      !cuok(cudaStreamCreateWithFlags(&s->up, cudaStreamNonBlocking), err, "stream") ||
      !cuok(cudaEventCreateWithFlags(&s->upDone, cudaEventDisableTiming), err, "event") || !cuok(cudaMemPoolCreate(&s->pool, &props), err, "memory pool"))
    return bad(err);
  // the pool keeps freed memory for the next requests, and an upload never waits for the work stream to reuse memory
  uint64_t keep = ~uint64_t(0);
  int no = 0;
  if (!cuok(cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &keep), err, "memory pool") ||
      !cuok(cudaMemPoolSetAttribute(s->pool, cudaMemPoolReuseAllowInternalDependencies, &no), err, "memory pool"))
    return bad(err);
  for (DaySlot& d : s->day) {   // the series pools
    if (!cuok(cudaMalloc(&d.dV, kSeriesVBytes), err, "series pool") || !cuok(cudaMalloc(reinterpret_cast<void**>(&d.dE), kSeriesEBytes), err, "series pool") ||
        !cuok(cudaMallocHost(reinterpret_cast<void**>(&d.hE), kSeriesEBytes), err, "series pool") ||
        !cuok(cudaMallocHost(reinterpret_cast<void**>(&d.hSeriesStatus), 4), err, "pinned"))
      return bad(err);
    s->used += kSeriesVBytes + kSeriesEBytes;
  }
  for (DaySlot& d : s->day)
    if (!cuok(cudaMallocHost(&d.hSegs, sizeof(Seg) * kMaxSegs), err, "pinned") || !cuok(cudaMallocHost(&d.hHdr, sizeof(BatchHdr)), err, "pinned") ||
        !cuok(cudaMallocHost(&d.hStatus, 4), err, "pinned") || !cuok(cudaMalloc(&d.dSegs, sizeof(Seg) * kMaxSegs), err, "segments") ||
        !cuok(cudaMalloc(&d.dHdr, sizeof(BatchHdr)), err, "segments") || !cuok(cudaMalloc(&d.dCtl, 64), err, "control") ||
        !cuok(cudaEventCreate(&d.ev[0]), err, "event") || !cuok(cudaEventCreate(&d.ev[1]), err, "event")) {
      return bad(err);
    } else {
      std::memset(d.hSegs, 0, sizeof(Seg) * kMaxSegs);
      std::memset(d.hHdr, 0, sizeof(BatchHdr));
    }
  for (ViewSlot& v : s->view)
    if (!cuok(cudaMalloc(&v.dCtl, 64), err, "control") || !cuok(cudaMallocHost(&v.hStatus, 4), err, "pinned") ||
        !cuok(cudaMallocHost(&v.hOut, size_t(kMaxViewChunk) * kMaxNA * 8), err, "pinned") || !cuok(cudaEventCreate(&v.ev[0]), err, "event") ||
        !cuok(cudaEventCreate(&v.ev[1]), err, "event"))
      return bad(err);
  if (!cuok(cudaMalloc(&s->dViewOut, size_t(kMaxViewChunk) * kMaxNA * 8), err, "views columns")) return bad(err);
  s->used += size_t(kMaxViewChunk) * kMaxNA * 8;
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
  if (s->up) cudaStreamSynchronize(s->up);
  for (auto& kv : s->all) {
    if (kv.second->dev && s->st) cudaFreeAsync(kv.second->dev, s->st);
    delete kv.second;
  }
  if (s->st) cudaStreamSynchronize(s->st);
  for (DScene& d : s->scenes) { cudaFree(d.nodes); cudaFree(d.tris); }
  free_pools(*s);
  for (DaySlot& d : s->day) {
    if (d.hSegs) cudaFreeHost(d.hSegs);
    if (d.hHdr) cudaFreeHost(d.hHdr);
    if (d.hStatus) cudaFreeHost(d.hStatus);
    cudaFree(d.dSegs); cudaFree(d.dHdr); cudaFree(d.dCtl);
    cudaFree(d.dV); cudaFree(d.dE);
    if (d.hE) cudaFreeHost(d.hE);
    if (d.hSeriesStatus) cudaFreeHost(d.hSeriesStatus);
    for (cudaEvent_t e : d.ev) if (e) cudaEventDestroy(e);
  }
  for (ViewSlot& v : s->view) {
    cudaFree(v.dCtl);
    if (v.hStatus) cudaFreeHost(v.hStatus);
    if (v.hOut) cudaFreeHost(v.hOut);
    for (cudaEvent_t e : v.ev) if (e) cudaEventDestroy(e);
  }
  cudaFree(s->dViewOut);
  if (s->pool) cudaMemPoolDestroy(s->pool);
  if (s->upDone) cudaEventDestroy(s->upDone);
  if (s->up) cudaStreamDestroy(s->up);
  if (s->st) cudaStreamDestroy(s->st);
  delete s;
}

KGB_API int kgb_server_add_scene(kgb_server* h, const float* v, size_t nv, const uint32_t* tri, size_t nt, int32_t* sceneId) {
  Server* s = reinterpret_cast<Server*>(h);
  for (size_t k = 0; k < 3 * nt; ++k) if (tri[k] >= nv) { set_error("kgb_server_add_scene: a triangle's vertex index exceeds the vertices"); return 0; }
  if (nt >= (size_t(1) << 32)) { set_error("kgb_server_add_scene: at most 2^32 - 1 triangles"); return 0; }
  DScene d;
  std::lock_guard<std::mutex> lk(s->m);
  if (nt) {   // the device builder (bvh_gpu.cu), on the server's work stream
    uint64_t temp = 0;
    const std::string why = build_bvh8_gpu(v, nv, tri, nt, nullptr, nullptr, s->st, &d.nodes, &d.tris, &d.nNodes, &temp);
    if (!why.empty()) {
      if (d.nodes) cudaFree(d.nodes);
      if (d.tris) cudaFree(d.tris);
      set_error("kgb_server_add_scene: " + why);
      return 0;
    }
  }
  if (d.nNodes >= kMaxNodes) {
    cudaFree(d.nodes);
    cudaFree(d.tris);
    set_error("kgb_server_add_scene: 2^24 nodes or more (the node records' child index has 24 bits)");
    return 0;
  }
  d.nTris = uint32_t(nt);
  d.bytes = uint64_t(d.nNodes) * kNodeBytes + uint64_t(nt) * 48;
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

KGB_API int kgb_server_set_tuning(kgb_server* h, uint32_t chunkSensors, uint64_t batchRays, uint64_t viewRays) {
  Server* s = reinterpret_cast<Server*>(h);
  std::unique_lock<std::mutex> lk(s->m);
  if (!s->active.empty() || !s->pending.empty()) { set_error("kgb_server_set_tuning: only while idle"); return 0; }
  if ((chunkSensors && (chunkSensors < 32 || chunkSensors > (1u << 20))) || (batchRays && (batchRays < (1u << 16) || batchRays > (uint64_t(1) << 32))) ||
      (viewRays && (viewRays < (1u << 16) || viewRays > (uint64_t(1) << 31)))) {
    set_error("kgb_server_set_tuning: chunk 32..2^20 sensors, batch 2^16..2^32 rays, views chunk 2^16..2^31 rays");
    return 0;
  }
  if (chunkSensors) s->chunkSensors = chunkSensors;
  if (batchRays) s->batchRays = batchRays;
  if (viewRays) s->viewRays = viewRays;
  std::string err;
  if (!make_pools(*s, err) || !cuok(cudaStreamSynchronize(s->st), err, "tuning")) { set_error(err); return 0; }
  return 1;
}

KGB_API void kgb_server_tuning(kgb_server* h, uint64_t* out) {
  Server* s = reinterpret_cast<Server*>(h);
  std::unique_lock<std::mutex> lk(s->m);
  out[0] = s->chunkSensors;
  out[1] = s->batchRays;
  out[2] = s->viewRays;
}

KGB_API int kgb_server_set_priority(kgb_server* h, double oldSeconds, double ageSeconds) {
  Server* s = reinterpret_cast<Server*>(h);
  if (!(oldSeconds > 0 && oldSeconds < 1e6 && ageSeconds > 0 && ageSeconds < 1e6)) {
    set_error("kgb_server_set_priority: both times in (0, 1e6) seconds");
    return 0;
  }
  std::unique_lock<std::mutex> lk(s->m);
  s->oldSeconds = oldSeconds;
  s->ageSeconds = ageSeconds;
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
  r->raysPerSensor = req->nDir;
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

KGB_API int kgb_server_submit_series(kgb_server* h, const kgb_daylight_request* req, const kgb_series_request* q, uint64_t* ticket) {
  Server* s = reinterpret_cast<Server*>(h);
  const auto no = [](const char* m) { set_error(std::string("kgb_server_submit_series: ") + m); return 0; };
  if (!q || (!q->E && req->nSensors)) return no("no series or no E");
  const kgb_series_in& in = q->in;
  if (req->scene < 0 || size_t(req->scene) >= s->scenes.size()) return no("unknown scene");
  if (req->nQ < 1 || req->nQ > kMaxQ) return no("1 to 8 quantities");
  if (q->gQ >= req->nQ) return no("gQ is not one of the request's quantities");
  if (in.G || in.Sdc) return no("G comes from quantity gQ and there is no reflected light: G and Sdc must be NULL");
  if (in.P <= 0 || in.T <= 0 || !in.S || !in.g || (in.nSky && (!in.row || !in.wsky)) || (in.nSun && (!in.sunStep || !in.sunVec || !in.sunW)))
    return no("missing series inputs");
  if (in.nSky > req->nDir || uint64_t(in.sun0) + in.nSun > req->nDir) return no("directions beyond the request's direction table");
  Request* r = new Request;
  r->kind = 0;
  r->d = *req;
  r->series = true;
  r->sq = *q;
  r->Kp = uint32_t((uint64_t(in.P) + 1 + 63) / 64 * 64);
  const size_t P = size_t(in.P), T = size_t(in.T);
  r->csr.assign(P + 1 + in.nSky, 0);
  for (uint32_t d = 0; d < in.nSky; ++d) {
    if (in.row[d] < 0 || in.row[d] >= in.P) { delete r; return no("a sky direction's row is not a patch"); }
    r->csr[size_t(in.row[d]) + 1]++;
  }
  for (size_t p = 0; p < P; ++p) r->csr[p + 1] += r->csr[p];
  {
    std::vector<int32_t> at(r->csr.begin(), r->csr.begin() + P);
    for (uint32_t d = 0; d < in.nSky; ++d) r->csr[P + 1 + size_t(at[size_t(in.row[d])]++)] = int32_t(d);
  }
  r->sunOfCol.assign(T, -1);
  for (uint32_t j = 0; j < in.nSun; ++j) {
    if (in.sunStep[j] < 0 || size_t(in.sunStep[j]) >= T) { delete r; return no("a sun step is not a column"); }
    if (r->sunOfCol[size_t(in.sunStep[j])] >= 0) { delete r; return no("two sun directions on one step (the tensor-core form's sun term takes one)"); }
    r->sunOfCol[size_t(in.sunStep[j])] = int32_t(j);
  }
  r->nSensors = req->nSensors;
  r->raysPerSensor = req->nDir;
  r->tSubmit = Clock::now();
  std::lock_guard<std::mutex> lk(s->m);
  r->ticket = s->nextTicket++;
  if (!r->nSensors || !req->nDir) {
    std::fill(req->out, req->out + size_t(req->nQ) * req->nSensors, 0.0);
    if (q->E) std::fill(q->E, q->E + size_t(req->nSensors) * T, 0.f);
    finish(*s, r, true, "");
  } else s->pending.push_back(r);
  s->all[r->ticket] = r;
  *ticket = r->ticket;
  s->cv.notify_all();
  return 1;
}

KGB_API int kgb_server_submit_views(kgb_server* h, const kgb_views_request* req, uint64_t* ticket) {
  Server* s = reinterpret_cast<Server*>(h);
  if (req->scene < 0 || size_t(req->scene) >= s->scenes.size()) { set_error("kgb_server_submit_views: unknown scene"); return 0; }
  if (req->nClass > KGB_VIEW_CLASSES || req->nReach > 8) { set_error("kgb_server_submit_views: at most 16 groups and 8 reach distances"); return 0; }
  const uint64_t K = uint64_t(req->view.nAz) * req->view.nEl;
  Request* r = new Request;
  r->kind = 1;
  r->v = *req;
  r->rowSin.assign(req->view.rowSin, req->view.rowSin + 2 * size_t(req->view.nEl));
  r->wRow.assign(req->wRow, req->wRow + req->view.nEl);
  r->nSensors = req->nSensors;
  r->raysPerSensor = K;
  r->tSubmit = Clock::now();
  std::lock_guard<std::mutex> lk(s->m);
  r->ticket = s->nextTicket++;
  if (!r->nSensors || !K) { std::fill(req->out, req->out + size_t(views_NA(*req)) * req->nSensors, 0.0); finish(*s, r, true, ""); }
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

// out[0..7]: completed requests, p50, p90, p99, max latency (s), rays, work items (daylight batches and views chunks),
// HBM bytes in use; out[8..9]: the tuned chunk sensors and batch rays
KGB_API void kgb_server_stats(kgb_server* h, double* out) {
  Server* s = reinterpret_cast<Server*>(h);
  std::lock_guard<std::mutex> lk(s->m);
  std::vector<double> l = s->latencies;
  std::sort(l.begin(), l.end());
  const auto q = [&](double f) { return l.empty() ? 0.0 : l[std::min(l.size() - 1, size_t(f * (l.size() - 1) + 0.5))]; };
  out[0] = double(l.size()); out[1] = q(0.5); out[2] = q(0.9); out[3] = q(0.99); out[4] = l.empty() ? 0.0 : l.back();
  out[5] = double(s->rays); out[6] = double(s->items); out[7] = double(s->used); out[8] = s->chunkSensors; out[9] = double(s->batchRays);
}

// out[0..4]: GPU seconds and rays of daylight batches, of views chunks (each item timed by events around it on the
// work stream), and wall seconds with work queued on that stream
KGB_API void kgb_server_timing(kgb_server* h, double* out) {
  Server* s = reinterpret_cast<Server*>(h);
  std::lock_guard<std::mutex> lk(s->m);
  out[0] = s->gpuSec[0]; out[1] = s->kindRays[0]; out[2] = s->gpuSec[1]; out[3] = s->kindRays[1]; out[4] = s->queuedSec;
}

}  // extern "C"
