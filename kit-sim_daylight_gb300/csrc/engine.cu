// The engine's C ABI (include/kitsim_gb300.h): device state, buffers, launch policy and the calls that replace the
// reference's gpu_* contract (src/internal.h:125-220, implemented there by src/gpu.cu over OptiX).
//
// Device state per engine: one CUDA stream; the scene (8-wide BVH nodes + triangle records, a movable object so that
// scenes can be parked and re-attached); the slot table; resident sensors (P, N) and directions (D); the chunk buffers
// (visibility bits / bytes, reflected-light rows, view classes + distances), grown on demand and kept between calls;
// a control block (task counter + status word) for the persistent kernels.
// Every call returns after its work is done (as the reference's synchronous calls do), so host arrays may be reused.
#include "engine.h"
#include "rt.cuh"

#include <thrust/device_ptr.h>
#include <thrust/execution_policy.h>
#include <thrust/functional.h>
#include <thrust/reduce.h>

#include <fcntl.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

namespace kgb {
namespace {

thread_local std::string g_err;
int fail(const std::string& m) { g_err = m; return 0; }

#define CU(call)                                                                          \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess) return fail(std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

struct Buf {   // device buffer, grown as needed (contents not kept)
  void* p = nullptr;
  size_t cap = 0;
  void free() { if (p) cudaFree(p); p = nullptr; cap = 0; }
};
int grow(Buf& b, size_t bytes) {
  if (bytes <= b.cap) return 1;
  b.free();
  CU(cudaMalloc(&b.p, std::max<size_t>(bytes, 256)));
  b.cap = std::max<size_t>(bytes, 256);
  return 1;
}
// Device -> pageable host copy of a large result through two pinned staging buffers: slice k + 1 streams over the
// link while the host copies slice k into place with a few threads (a pageable cudaMemcpy moves a few tens of GB/s).
// This is the fallback of HostLock below: its host memcpy bounds it at 50-110 GB/s on a Grace host.
struct Staging {
  void* h[2] = {nullptr, nullptr};
  cudaEvent_t ev[2] = {nullptr, nullptr};
  static constexpr size_t kSlice = size_t(32) << 20;
  void free() {
    for (int k = 0; k < 2; ++k) {
      if (h[k]) cudaFreeHost(h[k]);
      if (ev[k]) cudaEventDestroy(ev[k]);
      h[k] = nullptr; ev[k] = nullptr;
    }
  }
};
// A caller's host range page-locked for one call (cudaHostRegister), so that its copies run straight between the range
// and the device: the copy engines move about 190 GB/s over NVLink-C2C to and from page-locked memory, and registering
// costs about 2 us per MB on a Grace host. Before it unregisters the range, the destructor waits for the streams whose
// copies use it. The ranges this library registers are counted in one registry for the process, so that two calls
// copying the same range at once (two engines reading one input array) share one registration, which ends with the
// last of them. Memory the caller page-locked (cudaMallocHost, cudaHostRegister) is used as it is. Where the range
// cannot be registered (a read-only mapping) or overlaps a registration of this library's without matching it,
// `direct` stays false and the staged path runs.
constexpr size_t kLockMin = size_t(16) << 20;   // below this a plain copy is as fast as registering first
static bool page_locked(const void* p) {
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) { cudaGetLastError(); return false; }
  return a.type == cudaMemoryTypeHost;
}
struct LockRegistry {
  struct Range { size_t bytes; int refs; };
  std::mutex m;
  std::map<const char*, Range> ranges;   // by start address
  // the registered range overlapping [p, p + n), if any
  std::map<const char*, Range>::iterator overlap(const char* p, size_t n) {
    auto it = ranges.upper_bound(p);
    if (it != ranges.begin()) {
      auto prev = std::prev(it);
      if (prev->first + prev->second.bytes > p) return prev;
    }
    if (it != ranges.end() && it->first < p + n) return it;
    return ranges.end();
  }
};
static LockRegistry& lock_registry() {
  static LockRegistry* r = new LockRegistry;   // never destroyed: engines may outlive static destruction order
  return *r;
}
struct HostLock {
  const char* p = nullptr;
  bool direct = false, counted = false;
  cudaStream_t st[2] = {nullptr, nullptr};
  HostLock(const void* ptr, size_t bytes, bool readOnly, cudaStream_t s0, cudaStream_t s1 = nullptr)
      : p(static_cast<const char*>(ptr)), st{s0, s1} {
    if (!ptr || bytes < kLockMin) return;
    static const unsigned roFlag = [] {
      int dev = 0, ok = 0;
      return cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetAttribute(&ok, cudaDevAttrHostRegisterReadOnlySupported, dev) == cudaSuccess && ok
                 ? unsigned(cudaHostRegisterReadOnly) : 0u;
    }();
    LockRegistry& R = lock_registry();
    std::lock_guard<std::mutex> g(R.m);
    const auto it = R.overlap(p, bytes);
    if (it != R.ranges.end()) {   // registered by another call of this library: share it if it covers this range
      if (it->first <= p && p + bytes <= it->first + it->second.bytes) { it->second.refs++; direct = counted = true; }
      p = counted ? it->first : nullptr;
      return;
    }
    const cudaError_t e = cudaHostRegister(const_cast<char*>(p), bytes, readOnly ? roFlag : unsigned(cudaHostRegisterDefault));
    if (e == cudaSuccess) { R.ranges[p] = {bytes, 1}; direct = counted = true; return; }
    cudaGetLastError();   // a refused registration leaves no error behind for the next call
    direct = e == cudaErrorHostMemoryAlreadyRegistered && page_locked(p) && page_locked(p + bytes - 1);   // the caller's
  }
  ~HostLock() {
    if (!counted) return;
    for (cudaStream_t s : st) if (s) cudaStreamSynchronize(s);
    LockRegistry& R = lock_registry();
    std::lock_guard<std::mutex> g(R.m);
    auto it = R.ranges.find(p);
    if (it != R.ranges.end() && --it->second.refs == 0) {
      cudaHostUnregister(const_cast<char*>(p));
      R.ranges.erase(it);
    }
  }
  HostLock(const HostLock&) = delete;
  HostLock& operator=(const HostLock&) = delete;
};

void host_copy(void* dst, const void* src, size_t bytes) {
  constexpr size_t kPart = size_t(4) << 20;
  const int nt = int(std::min<size_t>(8, (bytes + kPart - 1) / kPart));
  if (nt <= 1) { std::memcpy(dst, src, bytes); return; }
  std::vector<std::thread> th;
  const size_t per = (bytes + nt - 1) / nt;
  for (int t = 0; t < nt; ++t) {
    const size_t a = size_t(t) * per, b = std::min(bytes, a + per);
    if (a < b) th.emplace_back([=] { std::memcpy(static_cast<char*>(dst) + a, static_cast<const char*>(src) + a, b - a); });
  }
  for (auto& x : th) x.join();
}
// Where a download goes: host memory (dst; page-locked for the call when `pinned`), or a file (fd >= 0) at a byte
// offset, written with pwrite.
struct Sink {
  void* dst = nullptr;
  int fd = -1;
  uint64_t offset = 0;
  bool pinned = false;
};
// len bytes of pinned src to the sink at byte pos: a few threads copy (memory), or pwrite calls (file: writes to one
// file take its lock in turn, so one writer is as fast as several)
int sink_put(const Sink& k, size_t pos, const void* src, size_t len) {
  if (k.fd < 0) { host_copy(static_cast<char*>(k.dst) + pos, src, len); return 1; }
  for (size_t a = 0; a < len;) {
    const ssize_t n = pwrite(k.fd, static_cast<const char*>(src) + a, len - a, off_t(k.offset + pos + a));
    if (n < 0 && errno == EINTR) continue;
    if (n <= 0) return fail(std::string("gpu_series: writing the series file failed: ") + std::strerror(n < 0 ? errno : EIO));
    a += size_t(n);
  }
  return 1;
}
// Device -> sink copy of bytes at byte pos of the sink, through the staging slices (memory results under two slices:
// one plain copy)
int download_to(Staging& s, const Sink& sk, size_t pos, const void* src, size_t bytes, cudaStream_t st) {
  if (sk.fd < 0 && (sk.pinned || bytes < 2 * Staging::kSlice)) {
    CU(cudaMemcpyAsync(static_cast<char*>(sk.dst) + pos, src, bytes, cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    return 1;
  }
  if (!bytes) return 1;
  for (int k = 0; k < 2; ++k) {
    if (!s.h[k]) CU(cudaMallocHost(&s.h[k], Staging::kSlice));
    if (!s.ev[k]) CU(cudaEventCreateWithFlags(&s.ev[k], cudaEventDisableTiming));
  }
  const size_t n = (bytes + Staging::kSlice - 1) / Staging::kSlice;
  const auto slice = [&](size_t k) { return std::min(Staging::kSlice, bytes - k * Staging::kSlice); };
  CU(cudaMemcpyAsync(s.h[0], src, slice(0), cudaMemcpyDeviceToHost, st));
  CU(cudaEventRecord(s.ev[0], st));
  for (size_t k = 0; k < n; ++k) {
    const int b = int(k & 1);
    if (k + 1 < n) {
      CU(cudaMemcpyAsync(s.h[b ^ 1], static_cast<const char*>(src) + (k + 1) * Staging::kSlice, slice(k + 1), cudaMemcpyDeviceToHost, st));
      CU(cudaEventRecord(s.ev[b ^ 1], st));
    }
    CU(cudaEventSynchronize(s.ev[b]));
    if (!sink_put(sk, pos + k * Staging::kSlice, s.h[b], slice(k))) return 0;
  }
  return 1;
}
int download_large(Staging& s, void* dst, const void* src, size_t bytes, cudaStream_t st, bool pinned) {
  Sink k;
  k.dst = dst;
  k.pinned = pinned;
  return download_to(s, k, 0, src, bytes, st);
}

// Host -> device copy of a large input: straight from the caller's range page-locked for the copy (which then has
// ended when this returns), else through the same staging slices (the host fills slice k while slice k - 1 is in
// flight; the copies are queued on the stream, in order).
int upload_large(Staging& s, void* dst, const void* src, size_t bytes, cudaStream_t st) {
  HostLock lock(src, bytes, true, st);
  if (lock.direct || bytes < 2 * Staging::kSlice) {
    CU(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st));
    return 1;
  }
  for (int k = 0; k < 2; ++k) {
    if (!s.h[k]) CU(cudaMallocHost(&s.h[k], Staging::kSlice));
    if (!s.ev[k]) CU(cudaEventCreateWithFlags(&s.ev[k], cudaEventDisableTiming));
  }
  const size_t n = (bytes + Staging::kSlice - 1) / Staging::kSlice;
  for (size_t k = 0; k < n; ++k) {
    const int b = int(k & 1);
    const size_t len = std::min(Staging::kSlice, bytes - k * Staging::kSlice);
    CU(cudaEventSynchronize(s.ev[b]));   // the slice's previous copy has left it
    host_copy(s.h[b], static_cast<const char*>(src) + k * Staging::kSlice, len);
    CU(cudaMemcpyAsync(static_cast<char*>(dst) + k * Staging::kSlice, s.h[b], len, cudaMemcpyHostToDevice, st));
    CU(cudaEventRecord(s.ev[b], st));
  }
  return 1;
}

// A direction-major [K x nc] device buffer (elements of 1 or 4 bytes) to host rows [nc x K]: slices of sensors are
// transposed on the device into one scratch buffer (at most 64 MiB) and downloaded through the staging slices.
constexpr size_t kRowsSlice = size_t(64) << 20;
int download_rows_into(Buf& rows, Staging& staging, const void* dev, size_t esize, size_t K, size_t nc, void* host, cudaStream_t st) {
  if (!K || !nc) return 1;
  if (K > 0xffffffffu) return fail("download: more than 2^32 - 1 elements per sensor");
  const size_t per = std::min<size_t>(std::max<size_t>(1, kRowsSlice / (K * esize)), 0xffffffffu);
  if (!grow(rows, std::min(per, nc) * K * esize)) return 0;
  HostLock lock(host, nc * K * esize, false, st);
  for (size_t i0 = 0; i0 < nc; i0 += per) {
    const size_t m = std::min(per, nc - i0);
    if (!launch_rows(static_cast<const char*>(dev) + i0 * esize, nc, rows.p, esize, uint32_t(K), uint32_t(m), st))
      return fail("download: too many elements per sensor for the transpose grid");
    CU(cudaGetLastError());
    if (!download_large(staging, static_cast<char*>(host) + i0 * K * esize, rows.p, m * K * esize, st, lock.direct)) return 0;
  }
  return 1;
}

int upload(Buf& b, const void* h, size_t bytes, cudaStream_t st) {
  if (!grow(b, bytes)) return 0;
  if (bytes) CU(cudaMemcpyAsync(b.p, h, bytes, cudaMemcpyHostToDevice, st));
  return 1;
}

struct SceneObj {
  Buf nodes, tris;
  uint32_t nNodes = 0, nTris = 0;
  uint64_t bytes = 0;
  ~SceneObj() { nodes.free(); tris.free(); }
};

}  // namespace

// Bands of a chunk's series whose downloads overlap the next band's kernel; the first band's kernel and the last band's
// download are not overlapped. Precision config (29,609-sensor chunks, E returned to host memory): 4 / 6 / 8 bands gave
// 17.74 / 18.36 / 18.13e9 sensor-steps/s (at 8 the shorter launches' tails cost more kernel time than they save).
constexpr uint32_t kSeriesBands = 6;

struct Engine {
  int device = 0, numSMs = 0;
  cudaStream_t st = nullptr;
  cudaEvent_t ev[2] = {};
  SceneObj* sc = nullptr;
  Buf slots;
  uint32_t nSlots = 0;
  Buf P, N, D, rayTab;   // rayTab: 48 bytes per direction (the direction-only part of each ray)
  size_t nSensors = 0, nDir = 0, nWords = 0;
  Buf order;                          // the sensors grouped by normal orientation (TraceArgs::order), on the device
  std::vector<uint32_t> orderHost;    // and here, to find a call's runs
  uint32_t classStart[7] = {};        // class c's sensors are orderHost[classStart[c] .. classStart[c + 1])
  Buf cls, clsFlags;                  // the classes the order was built from (a byte per sensor); the class kernel's flags
  Buf vis;
  bool bytes = false;
  size_t i0 = 0, visN = 0;
  Buf dc, contrib;   // contrib: one (bin, contribution) pair per path of a bounce launch
  Buf border;        // a bounce launch's samples in tracing order
  Buf bq;            // a bounce launch's two queues of paths that go on
  int gridStep = 0;
  Buf slotLog;       // ln tn per slot as a float pair (glass transmission)
  size_t nBins = 0, dcN = 0, dcI0 = 0;
  Buf viewCls, viewDist, rowSin;
  size_t viewN = 0, viewK = 0, viewI0 = 0;
  kgb_view_in view{};
  Buf label;
  size_t nLabel = 0;
  Buf scratch, out;
  Buf w64;           // a reduce's weights as doubles
  Buf ctl;   // [0] task counter, [1] status, [2..7] three u64 counters of the instrumented kernels
  bool ownStream = true;
  int seriesForm = 0;         // 0 split-BF16 tensor cores, 1 plain FP32
  Buf vop, sop, csr, sunCol;
  Staging staging;   // pinned slices for the series download
  Buf rows;          // sensor-major rows of one slice of a direction-major buffer (download_rows)
  cudaStream_t copySt = nullptr;                  // the series' E downloads, beside the next band's kernel
  cudaEvent_t bandEv[kSeriesBands] = {};
  kgb_stats stats{};
  int gridBits = 0, gridBytes = 0, gridView = 0;
  int builder = 1;            // 1 device LBVH with treelet restructuring (default), 0 host binned SAH (kgb_set_builder)
  uint32_t nodeLimit = 0;     // kgb_set_limits: the walks see only this many of the BVH's nodes (0: all)
  uint64_t bounceLimitNs = kBounceLimitNs;   // kgb_set_limits: a bounce step kernel's time limit
  uint64_t seriesWaitNs = 0;                  // kgb_set_limits: the series pipeline's wait limit (0: its default)
  bool withholdFills = false;                 // kgb_set_limits: KGB_LIMIT_WITHHOLD_FILLS
  std::vector<DevMesh*> meshes;               // meshes read to the device, by id (null: freed)
};

namespace {

Engine* E(kgb_engine* e) { return reinterpret_cast<Engine*>(e); }
// The nodes a walk may use: all of the scene's, or the first nodeLimit (kgb_set_limits). A walk that reaches a node
// index beyond them gives up as one past its visit cap does (rt.cuh), so a small limit drives that error path.
uint32_t walk_nodes(const Engine& g) { return g.nodeLimit && g.nodeLimit < g.sc->nNodes ? g.nodeLimit : g.sc->nNodes; }
const Engine* E(const kgb_engine* e) { return reinterpret_cast<const Engine*>(e); }

// The samples [s0, s1) of a bounce launch in tracing order: sorted by the 2-D Morton key of their first direction's
// coordinates before the per-sensor rotation, (s / M, radical inverse of s), so that 32 consecutive samples of a
// sensor leave it in a narrow cone.
int bounce_order(Engine& g, uint32_t s0, uint32_t s1, uint32_t M) {
  const auto spread = [](uint32_t x) {   // 16 bits to the even bit positions
    x &= 0xffffu;
    x = (x | (x << 8)) & 0x00ff00ffu; x = (x | (x << 4)) & 0x0f0f0f0fu; x = (x | (x << 2)) & 0x33333333u; x = (x | (x << 1)) & 0x55555555u;
    return x;
  };
  const auto rev = [](uint32_t x) {
    x = (x >> 16) | (x << 16); x = ((x & 0xff00ff00u) >> 8) | ((x & 0x00ff00ffu) << 8); x = ((x & 0xf0f0f0f0u) >> 4) | ((x & 0x0f0f0f0fu) << 4);
    x = ((x & 0xccccccccu) >> 2) | ((x & 0x33333333u) << 2); x = ((x & 0xaaaaaaaau) >> 1) | ((x & 0x55555555u) << 1);
    return x;
  };
  std::vector<std::pair<uint32_t, uint32_t>> key(s1 - s0);
  for (uint32_t smp = s0; smp < s1; ++smp) {
    const uint32_t u = uint32_t(std::min(65535.0, double(smp) / double(M) * 65536.0)), v = rev(smp) >> 16;
    key[smp - s0] = {(spread(v) << 1) | spread(u), smp};
  }
  std::sort(key.begin(), key.end());
  std::vector<uint32_t> ord(key.size());
  for (size_t k = 0; k < key.size(); ++k) ord[k] = key[k].second;
  return upload(g.border, ord.data(), ord.size() * 4, g.st);
}

int download_rows(Engine& g, const void* dev, size_t esize, size_t K, size_t nc, void* host) {
  return download_rows_into(g.rows, g.staging, dev, esize, K, nc, host, g.st);
}

int sync_status(Engine& g) {   // wait for the stream, then read the kernels' status word
  uint32_t status = 0;
  CU(cudaMemcpyAsync(&status, static_cast<uint32_t*>(g.ctl.p) + 1, 4, cudaMemcpyDeviceToHost, g.st));
  CU(cudaStreamSynchronize(g.st));
  CU(cudaGetLastError());
  if (status & kStatusStackOverflow) return fail("traversal stack overflow (BVH deeper than the kernel's stack)");
  if (status & kStatusVisitLimit)
    return fail("traversal gave up: a query passed its node-visit limit (the BVH's node count + 8, at most 2^20) or met a node index beyond the BVH");
  return 1;
}
int reset_ctl(Engine& g) {
  CU(cudaMemsetAsync(g.ctl.p, 0, 128, g.st));
  return 1;
}
float elapsed(Engine& g) {
  float ms = 0;
  cudaEventElapsedTime(&ms, g.ev[0], g.ev[1]);
  return ms;
}

// ---------------------------------------------------------------------------------------------------- .dmesh ingest
// The .dmesh header (the reference's parse_dmesh, src/mesh.cpp:451): magic, flags (bit 0: the slot block), counts.
struct DmeshHeader { char magic[4]; uint32_t flags; uint64_t nPoints, nFaces, nIndices; };
static_assert(sizeof(DmeshHeader) == 32, "the .dmesh header is 32 bytes");

// parse_dmesh's header checks (src/mesh.cpp:456-461) for an image of `size` bytes, in its order and words (without
// the label); payload: the arrays' bytes after the header
std::string dmesh_header(const DmeshHeader& h, uint64_t size, uint64_t& payload) {
  if (std::memcmp(h.magic, "DLM1", 4)) return "not a .dmesh file (magic DLM1)";
  if (h.flags & ~1u) return "unsupported header flags " + std::to_string(h.flags) + " (only bit 0, the slot block, is defined)";
  if (!(h.nPoints <= size / 24 && h.nFaces <= size / 4 && h.nIndices <= size / 4 && 32 + 24 * h.nPoints + 4 * h.nFaces + 4 * h.nIndices <= size))
    return "truncated";
  const uint64_t nSlots = (h.flags & 1) ? h.nFaces : 0;
  if (32 + 24 * h.nPoints + 4 * h.nFaces + 4 * h.nIndices + 2 * nSlots > size) return "truncated slot block";
  payload = 24 * h.nPoints + 4 * h.nFaces + 4 * h.nIndices + 2 * nSlots;
  return "";
}
// The device allocation of a checked header: the payload's arrays in the image's order, then the face offsets.
int mesh_alloc(const DmeshHeader& h, uint64_t payload, const std::string& label, std::unique_ptr<DevMesh>& out) {
  if (h.nPoints > 0xffffffffull || h.nFaces > 0xffffffffull || h.nIndices > 0xffffffffull)
    return fail(label + ": more than 2^32 - 1 points, faces or indices (the engine's limit)");
  std::unique_ptr<DevMesh> m(new DevMesh);
  const uint64_t offAt = (payload + 255) / 256 * 256;
  m->bytes = std::max<uint64_t>(256, offAt + 8 * h.nFaces);
  if (cudaMalloc(&m->buf, m->bytes) != cudaSuccess) {
    m->buf = nullptr;
    cudaGetLastError();
    return fail(label + ": out of device memory (" + std::to_string(m->bytes) + " bytes for the mesh)");
  }
  char* b = static_cast<char*>(m->buf);
  MeshView& v = m->view;
  v.pts = reinterpret_cast<const double*>(b);
  v.counts = reinterpret_cast<const int32_t*>(b + 24 * h.nPoints);
  v.idx = reinterpret_cast<const int32_t*>(b + 24 * h.nPoints + 4 * h.nFaces);
  v.slot16 = (h.flags & 1) ? reinterpret_cast<const uint16_t*>(b + 24 * h.nPoints + 4 * h.nFaces + 4 * h.nIndices) : nullptr;
  v.slot32 = nullptr;
  v.idxOff = reinterpret_cast<const uint64_t*>(b + offAt);
  v.nPoints = h.nPoints; v.nFaces = h.nFaces; v.nIdx = h.nIndices;
  out = std::move(m);
  return 1;
}
// The copied image's checks on the device; then the mesh is kept (an id) or, without faces, dropped.
int mesh_keep(Engine& g, std::unique_ptr<DevMesh> m, const std::string& label, kgb_mesh_info* info) {
  const std::string why = mesh_check(*m, g.st);
  if (!why.empty()) {
    cudaStreamSynchronize(g.st);
    return fail(label + ": " + why);
  }
  m->info.id = KGB_NO_MESH;
  if (m->view.nFaces) {
    size_t id = 0;
    while (id < g.meshes.size() && g.meshes[id]) ++id;
    if (id >= KGB_NO_MESH) return fail(label + ": too many meshes held");
    if (id == g.meshes.size()) g.meshes.push_back(nullptr);
    m->info.id = uint32_t(id);
    *info = m->info;
    g.meshes[id] = m.release();
    return 1;
  }
  *info = m->info;
  return 1;
}
// `bytes` of a file from byte `off` to device memory: the file read in staging slices (several threads per slice), each
// slice's copy queued while the next is read. A short read is the reference's "truncated".
int read_to_device(Engine& g, int fd, uint64_t off, uint64_t bytes, void* dst, const std::string& label) {
  Staging& s = g.staging;
  for (int k = 0; k < 2; ++k) {
    if (!s.h[k]) CU(cudaMallocHost(&s.h[k], Staging::kSlice));
    if (!s.ev[k]) CU(cudaEventCreateWithFlags(&s.ev[k], cudaEventDisableTiming));
  }
  const size_t n = (bytes + Staging::kSlice - 1) / Staging::kSlice;
  for (size_t k = 0; k < n; ++k) {
    const int b = int(k & 1);
    const size_t len = std::min<uint64_t>(Staging::kSlice, bytes - k * Staging::kSlice);
    CU(cudaEventSynchronize(s.ev[b]));   // the slice's previous copy has left it
    constexpr size_t kPart = size_t(8) << 20;
    const int parts = int(std::max<size_t>(1, std::min<size_t>(4, len / kPart)));
    const size_t per = (len + parts - 1) / parts;
    std::vector<int> ok(parts, 1);
    const auto part = [&](int q) {
      char* h = static_cast<char*>(s.h[b]);
      const size_t a0 = size_t(q) * per, a1 = std::min(len, a0 + per);
      for (size_t a = a0; a < a1;) {
        const ssize_t r = pread(fd, h + a, a1 - a, off_t(off + k * Staging::kSlice + a));
        if (r < 0 && errno == EINTR) continue;
        if (r <= 0) { ok[q] = 0; return; }
        a += size_t(r);
      }
    };
    if (parts == 1) part(0);
    else {
      std::vector<std::thread> th;
      for (int q = 0; q < parts; ++q) th.emplace_back(part, q);
      for (auto& t : th) t.join();
    }
    for (int q = 0; q < parts; ++q)
      if (!ok[q]) {
        cudaStreamSynchronize(g.st);
        return fail(label + ": truncated");
      }
    CU(cudaMemcpyAsync(static_cast<char*>(dst) + k * Staging::kSlice, s.h[b], len, cudaMemcpyHostToDevice, g.st));
    CU(cudaEventRecord(s.ev[b], g.st));
  }
  return 1;
}
DevMesh* find_mesh(Engine& g, uint32_t id) { return id < g.meshes.size() ? g.meshes[id] : nullptr; }

// The scene's records from checked arrays (kgb_build's host arrays, or kgb_build_meshes's device arrays when onDevice):
// the device builder reads either; the host builder gets device arrays copied back first.
int build_scene(Engine& g, const float* v, size_t nv, const uint32_t* tri, size_t nt, const uint32_t* slot, const uint8_t* translucent, bool onDevice) {
  CU(cudaEventRecord(g.ev[0], g.st));
  SceneObj& s = *g.sc;
  if (g.builder == 1) {   // on the device
    void* nodes = nullptr;
    void* tris = nullptr;
    uint32_t nNodes = 0;
    uint64_t temp = 0;
    const std::string why = build_bvh8_gpu(v, nv, tri, nt, slot, translucent, g.st, &nodes, &tris, &nNodes, &temp);
    s.nodes.p = nodes; s.nodes.cap = std::max<size_t>(1, nt) * kNodeBytes;
    s.tris.p = tris; s.tris.cap = nt * 48;
    if (!why.empty()) return fail("gpu_build: " + why);
    s.nNodes = nNodes;
    s.bytes = uint64_t(nNodes) * kNodeBytes + uint64_t(nt) * 48;
    g.stats.buildTempBytes = temp;
  } else {   // on the host (binned SAH)
    std::vector<float> hv;
    std::vector<uint32_t> htri, hslot;
    std::vector<uint8_t> htr;
    if (onDevice) {
      hv.resize(3 * nv); htri.resize(3 * nt);
      if (nv) CU(cudaMemcpyAsync(hv.data(), v, nv * 12, cudaMemcpyDeviceToHost, g.st));
      CU(cudaMemcpyAsync(htri.data(), tri, nt * 12, cudaMemcpyDeviceToHost, g.st));
      if (slot) { hslot.resize(nt); CU(cudaMemcpyAsync(hslot.data(), slot, nt * 4, cudaMemcpyDeviceToHost, g.st)); }
      if (translucent) { htr.resize(nt); CU(cudaMemcpyAsync(htr.data(), translucent, nt, cudaMemcpyDeviceToHost, g.st)); }
      CU(cudaStreamSynchronize(g.st));
      v = hv.data(); tri = htri.data(); slot = slot ? hslot.data() : nullptr; translucent = translucent ? htr.data() : nullptr;
    }
    BvhOut b;
    build_bvh8(v, nv, tri, nt, slot, translucent, b);
    if (!upload(s.nodes, b.nodes.data(), b.nodes.size() * 4, g.st) || !upload(s.tris, b.tris.data(), b.tris.size() * 4, g.st)) return 0;
    s.nNodes = b.nNodes;
    s.bytes = b.nodes.size() * 4 + b.tris.size() * 4;
    g.stats.buildTempBytes = uint64_t(nt) * 64;
  }
  if (s.nNodes >= kMaxNodes) return fail("gpu_build: 2^24 nodes or more (the node records' child index has 24 bits)");
  s.nTris = uint32_t(nt);
  CU(cudaEventRecord(g.ev[1], g.st));
  CU(cudaStreamSynchronize(g.st));
  g.stats.buildMs += elapsed(g);
  g.stats.gasBytes = s.bytes;
  g.stats.buildOutputBytes = s.bytes;
  return 1;
}

}  // namespace

int set_error(const std::string& message) { return fail(message); }

void engine_reduce_inputs(kgb_engine* e, ReduceInputs& in) {
  const Engine& g = *E(e);
  in.device = g.device; in.st = g.st;
  in.visN = g.visN; in.nDir = g.nDir; in.nWords = g.nWords; in.bytes = g.bytes;
  in.bitsVis = g.bytes ? nullptr : static_cast<const uint32_t*>(g.vis.p);
  in.bytesVis = g.bytes ? static_cast<const uint8_t*>(g.vis.p) : nullptr;
  in.N = static_cast<const float*>(g.N.p) + 3 * g.i0;
  in.D = static_cast<const float*>(g.D.p);
}
}  // namespace kgb

using namespace kgb;

extern "C" {

KGB_API int32_t kgb_version(void) { return KGB_ABI_VERSION; }
KGB_API const char* kgb_last_error(void) { return g_err.c_str(); }

KGB_API kgb_engine* kgb_init(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) { fail("no CUDA device"); return nullptr; }
  Engine* g = new Engine;
  const auto bad = [&](const std::string& m) { fail(m); kgb_destroy(reinterpret_cast<kgb_engine*>(g)); return nullptr; };
  if (cudaGetDevice(&g->device) != cudaSuccess) return bad("cudaGetDevice failed");
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, g->device) != cudaSuccess) return bad("cudaGetDeviceProperties failed");
  if (prop.major < 10) return bad(std::string("the engine is built for sm_103a; device is ") + prop.name);
  g->numSMs = prop.multiProcessorCount;
  if (cudaStreamCreateWithFlags(&g->st, cudaStreamNonBlocking) != cudaSuccess) return bad("cudaStreamCreate failed");
  if (cudaEventCreate(&g->ev[0]) != cudaSuccess || cudaEventCreate(&g->ev[1]) != cudaSuccess) return bad("cudaEventCreate failed");
  if (!grow(g->ctl, 128)) return bad(g_err);
  g->sc = new SceneObj;
  const kgb_slot one{0.2f, 0.f, 0.f, 0u};
  if (!kgb_set_slots(reinterpret_cast<kgb_engine*>(g), &one, 1)) return bad(g_err);
  return reinterpret_cast<kgb_engine*>(g);
}

KGB_API void kgb_destroy(kgb_engine* e) {
  if (!e) return;
  Engine* g = E(e);
  if (g->st) cudaStreamSynchronize(g->st);
  delete g->sc;
  for (DevMesh* m : g->meshes) delete m;
  for (Buf* b : {&g->slots, &g->P, &g->N, &g->D, &g->rayTab, &g->vis, &g->dc, &g->contrib, &g->viewCls, &g->viewDist, &g->rowSin, &g->label, &g->scratch, &g->out, &g->ctl,
                 &g->vop, &g->sop, &g->csr, &g->sunCol, &g->rows, &g->border, &g->slotLog, &g->bq, &g->w64}) b->free();
  g->staging.free();
  for (cudaEvent_t ev : g->ev) if (ev) cudaEventDestroy(ev);
  for (cudaEvent_t ev : g->bandEv) if (ev) cudaEventDestroy(ev);
  if (g->copySt) { cudaStreamSynchronize(g->copySt); cudaStreamDestroy(g->copySt); }
  if (g->st && g->ownStream) cudaStreamDestroy(g->st);
  delete g;
}

// Device bytes a build of nt triangles over nv vertices peaks at: inputs stay on the host (the builder runs there),
// the device holds the triangle records (48 B each) and at most nt/2 + 2 nodes of kNodeBytes; counted twice (the new
// scene and a parked one may coexist during a swap).
KGB_API uint64_t kgb_build_bytes(kgb_engine*, size_t nv, size_t nt, int slotted) {
  if (!nt) return 0;
  const uint64_t inputs = uint64_t(nv) * 12 + uint64_t(nt) * (12 + (slotted ? 4 : 0));
  const uint64_t out = uint64_t(nt) * 64 + (uint64_t(nt) / 2 + 2) * kNodeBytes + 4096;
  return inputs + 2 * out;
}

KGB_API int kgb_build(kgb_engine* e, const float* v, size_t nv, const uint32_t* tri, size_t nt, const uint32_t* slot,
                      const kgb_slot* slots, size_t nSlots, int perSlot) {
  Engine& g = *E(e);
  delete g.sc;
  g.sc = new SceneObj;
  g.stats.gasBytes = 0;
  if (!nt) return 1;   // empty scene: every ray misses
  if (slot) for (size_t k = 0; k < nt; ++k) if (slot[k] >= nSlots) return fail("gpu_build: a triangle's slot has no Slot");
  bool anyTau = false;
  for (size_t s = 0; s < nSlots; ++s) anyTau = anyTau || slots[s].tau > 0;
  const bool slotted = perSlot || anyTau;
  if (slotted && !slot) return fail("gpu_build: per-slot records need a slot per triangle");
  if (nt > (size_t(1) << 31)) return fail("gpu_build: more than 2^31 triangles");
  for (size_t k = 0; k < 3 * nt; ++k) if (tri[k] >= nv) return fail("gpu_build: a triangle's vertex index exceeds the vertices");
  std::vector<uint8_t> translucent;
  if (slotted) {
    translucent.resize(nt);
    for (size_t k = 0; k < nt; ++k) translucent[k] = slots[slot[k]].tau > 0 ? 1 : 0;
  }
  return build_scene(g, v, nv, tri, nt, slotted ? slot : nullptr, slotted ? translucent.data() : nullptr, false);
}

KGB_API void kgb_trim(kgb_engine* e, int sensors) {
  Engine& g = *E(e);
  cudaStreamSynchronize(g.st);
  g.vis.free(); g.dc.free(); g.contrib.free(); g.scratch.free(); g.out.free(); g.w64.free(); g.viewCls.free(); g.viewDist.free();
  g.vop.free(); g.sop.free(); g.csr.free(); g.sunCol.free();
  g.viewN = 0;
  if (sensors) {
    g.P.free(); g.N.free(); g.label.free(); g.order.free(); g.cls.free(); g.nLabel = 0; g.nSensors = 0;
    std::vector<uint32_t>().swap(g.orderHost);
  }
}

KGB_API int kgb_set_slots(kgb_engine* e, const kgb_slot* slots, size_t n) {
  Engine& g = *E(e);
  const kgb_slot one{0.2f, 0.f, 0.f, 0u};
  if (!n) { slots = &one; n = 1; }
  if (!upload(g.slots, slots, n * sizeof(kgb_slot), g.st) || !grow(g.slotLog, n * 8)) return 0;
  launch_slot_logs(static_cast<const kgb_slot*>(g.slots.p), uint32_t(n), static_cast<float2*>(g.slotLog.p), g.st);
  CU(cudaGetLastError());
  g.nSlots = uint32_t(n);
  CU(cudaStreamSynchronize(g.st));
  return 1;
}

KGB_API kgb_scene kgb_detach(kgb_engine* e) {
  Engine& g = *E(e);
  kgb_scene s{g.sc, g.sc->bytes};
  g.sc = new SceneObj;
  g.stats.gasBytes = 0;
  return s;
}
KGB_API void kgb_attach(kgb_engine* e, kgb_scene s) {
  Engine& g = *E(e);
  cudaStreamSynchronize(g.st);
  delete g.sc;
  g.sc = s.handle ? static_cast<SceneObj*>(s.handle) : new SceneObj;
  g.stats.gasBytes = g.sc->bytes;
}
KGB_API void kgb_free_scene(kgb_scene* s) {
  if (!s) return;
  delete static_cast<SceneObj*>(s->handle);
  s->handle = nullptr;
  s->bytes = 0;
}
KGB_API uint64_t kgb_free_bytes(void) {
  size_t f = 0, t = 0;
  return cudaMemGetInfo(&f, &t) == cudaSuccess ? f : 0;
}

// The tracing order of the visibility kernels: the sensors stably partitioned by the dominant axis of their normal and its
// sign. A warp traces one direction for 32 consecutive sensors of that order, so a warp whose sensors straddle two faces
// of different orientation (whose lanes on the face turned away from the direction idle) becomes one straddling two
// faces of the same orientation. Urban block, the reference's direction table: trace 60.9 to 58.1 ms. The results of
// every sensor do not depend on the order: any partition of the sensors into six runs, each in index order, traces the
// same rays, so the order is rebuilt only when the classes of the sensors just uploaded differ from those it was built
// from (a kernel compares them on the device; a caller that sends the same sensors every step pays for that kernel).
static bool sensor_order(Engine& g, size_t nSensors) {
  const bool fresh = g.orderHost.size() != nSensors || !g.order.p;
  if (!grow(g.cls, nSensors) || !grow(g.clsFlags, 7 * 4)) return false;
  if (fresh && nSensors) CU(cudaMemsetAsync(g.cls.p, 0xff, nSensors, g.st));   // no class yet: every sensor differs
  CU(cudaMemsetAsync(g.clsFlags.p, 0, 7 * 4, g.st));
  launch_sensor_classes(static_cast<const float*>(g.N.p), uint32_t(nSensors), static_cast<uint8_t*>(g.cls.p),
                        static_cast<uint32_t*>(g.clsFlags.p), g.st);
  CU(cudaGetLastError());
  uint32_t f[7];
  CU(cudaMemcpyAsync(f, g.clsFlags.p, sizeof f, cudaMemcpyDeviceToHost, g.st));
  CU(cudaStreamSynchronize(g.st));
  if (!f[0] && !fresh) return true;
  std::vector<uint8_t> cls(nSensors);
  if (nSensors) {
    CU(cudaMemcpyAsync(cls.data(), g.cls.p, nSensors, cudaMemcpyDeviceToHost, g.st));
    CU(cudaStreamSynchronize(g.st));
  }
  g.classStart[0] = 0;
  for (int c = 0; c < 6; ++c) g.classStart[c + 1] = g.classStart[c] + f[1 + c];
  if (g.classStart[6] != nSensors) return fail("gpu_set_scene: the sensors' classes do not add up");
  uint32_t at[6];
  for (int c = 0; c < 6; ++c) at[c] = g.classStart[c];
  g.orderHost.resize(nSensors);
  for (size_t i = 0; i < nSensors; ++i) g.orderHost[at[cls[i]]++] = uint32_t(i);
  return upload(g.order, g.orderHost.data(), nSensors * 4, g.st);
}

KGB_API int kgb_set_scene(kgb_engine* e, const float* P, const float* N, size_t nSensors, const float* D, size_t nDir) {
  Engine& g = *E(e);
  if (nSensors > 0xffffffffull) return fail("gpu_set_scene: more sensors than 32-bit indices hold");
  g.nSensors = nSensors; g.nDir = nDir; g.nWords = (nDir + 31) / 32;
  if (!upload(g.P, P, nSensors * 12, g.st) || !upload(g.N, N, nSensors * 12, g.st) || !upload(g.D, D, nDir * 12, g.st) ||
      !grow(g.rayTab, nDir * 48)) return 0;
  launch_ray_table(static_cast<const float*>(g.D.p), uint32_t(nDir), g.rayTab.p, g.st);
  CU(cudaGetLastError());
  if (!sensor_order(g, nSensors)) return 0;
  CU(cudaStreamSynchronize(g.st));
  return 1;
}

KGB_API int kgb_set_labels(kgb_engine* e, const uint8_t* label, size_t n) {
  Engine& g = *E(e);
  if (!upload(g.label, label, n, g.st)) return 0;
  g.nLabel = n;
  CU(cudaStreamSynchronize(g.st));
  return 1;
}

// gpu.cu:499-531: sensors [i0, i0 + nc) in sub-launches sized from the previous one's time (first 4096 sensors, then
// ~150 ms; byte mode 2^13 threads first and at least, then ~30 ms, at most doubling): the reference's stats and
// cancel points. Each sub-launch is one persistent grid over its (32 sensors x word) tasks.
static int trace_impl(Engine& g, size_t i0, size_t nc, uint32_t rayFlags, uint64_t* counters) {
  if (i0 + nc > g.nSensors) return fail("gpu_trace: sensor range exceeds the scene");
  g.bytes = !(rayFlags & KGB_RAY_DISABLE_ANYHIT);
  if (!grow(g.vis, g.bytes ? g.nDir * nc : g.nWords * nc * 4)) return 0;
  g.i0 = i0; g.visN = nc;
  if (nc == 0 || g.nWords == 0) return 1;
  if (!g.gridBits) g.gridBits = g.numSMs * bits_blocks_per_sm();
  if (!g.gridBytes) g.gridBytes = g.numSMs * bytes_blocks_per_sm();
  const bool any = g.bytes;
  const double targetMs = any ? 30 : 150;
  // byte mode: the reference starts at 2^13 threads and at most doubles; here at least four tasks per resident warp
  const size_t nMin = any ? std::max<size_t>((size_t(1) << 13) / g.nWords, (size_t(4) * g.gridBytes * 8 * 32 + g.nWords - 1) / g.nWords) : 1024;
  const size_t nMax = std::max<size_t>(32, size_t(0xffffffffu) / g.nWords * 32);   // warp tasks are counted in 32 bits
  size_t done = 0, n = std::min(counters ? nc : std::min(any ? nMin : size_t(4096), nc), nMax);
  TraceArgs a{};
  a.nodes = static_cast<const Node8*>(g.sc->nodes.p); a.tris = static_cast<const TriRec*>(g.sc->tris.p); a.nNodes = walk_nodes(g);
  a.P = static_cast<const float*>(g.P.p); a.N = static_cast<const float*>(g.N.p); a.D = static_cast<const float*>(g.D.p);
  a.stride = uint32_t(nc); a.nDir = uint32_t(g.nDir); a.nWords = uint32_t(g.nWords); a.rayFlags = rayFlags;
  a.bits = any ? nullptr : static_cast<uint32_t*>(g.vis.p);
  a.bytes = any ? static_cast<uint8_t*>(g.vis.p) : nullptr;
  a.slots = static_cast<const kgb_slot*>(g.slots.p); a.nSlots = g.nSlots; a.slotLog = static_cast<const float2*>(g.slotLog.p);
  a.counter = static_cast<uint32_t*>(g.ctl.p); a.status = static_cast<uint32_t*>(g.ctl.p) + 1;
  a.rayTab = static_cast<const RayDir*>(g.rayTab.p);
  if (g.orderHost.size() == g.nSensors) {   // the call's range in tracing order: per class, its run of the order
    a.order = static_cast<const uint32_t*>(g.order.p);
    a.callI0 = uint32_t(i0);
    uint32_t end = 0;
    for (int c = 0; c < 6; ++c) {
      const uint32_t* b = g.orderHost.data() + g.classStart[c];
      const uint32_t* x = g.orderHost.data() + g.classStart[c + 1];
      const uint32_t lo = uint32_t(std::lower_bound(b, x, uint32_t(i0)) - g.orderHost.data());
      const uint32_t hi = uint32_t(std::lower_bound(b, x, uint32_t(i0 + nc)) - g.orderHost.data());
      a.pieceG[c] = lo - end;   // modulo 2^32: pieceG[c] + p = lo + (p - end) for the run's positions p
      end += hi - lo;
      a.pieceEnd[c] = end;
    }
  }
  while (done < nc) {
    a.first = uint32_t(i0 + done); a.n = uint32_t(n); a.out0 = uint32_t(done); a.p0 = uint32_t(done);
    if (!reset_ctl(g)) return 0;
    const size_t tasks = (n + 31) / 32 * g.nWords;   // warp tasks: 32 sensors x one 32-direction word
    const int grid = int(std::min<size_t>(size_t(any ? g.gridBytes : g.gridBits), (tasks + 7) / 8));
    CU(cudaEventRecord(g.ev[0], g.st));
    if (any) launch_bytes(a, grid, g.st); else launch_bits(a, grid, g.st, counters != nullptr);
    CU(cudaEventRecord(g.ev[1], g.st));
    if (!sync_status(g)) return 0;
    if (counters) {
      uint64_t c[3];
      CU(cudaMemcpy(c, static_cast<uint32_t*>(g.ctl.p) + 2, sizeof c, cudaMemcpyDeviceToHost));
      for (int k = 0; k < 3; ++k) counters[k] += c[k];
    }
    const double ms = elapsed(g);
    g.stats.traceMs += ms; g.stats.rays += n * g.nDir; g.stats.launches++;
    done += n;
    const double want = double(n) * targetMs / std::max(ms, 1e-3);
    n = std::min({std::max<size_t>(want > 1e12 ? size_t(1) << 40 : size_t(want), nMin), any ? 2 * n : nc, nc - done, nMax});
  }
  return 1;
}

KGB_API int kgb_trace(kgb_engine* e, size_t i0, size_t nc, uint32_t rayFlags) { return trace_impl(*E(e), i0, nc, rayFlags, nullptr); }

KGB_API int kgb_trace_counters(kgb_engine* e, size_t i0, size_t nc, uint32_t rayFlags, uint64_t out[4]) {
  Engine& g = *E(e);
  if (!(rayFlags & KGB_RAY_DISABLE_ANYHIT)) return fail("kgb_trace_counters: visibility bits only (KGB_RAY_DISABLE_ANYHIT)");
  out[0] = out[1] = out[2] = 0;
  out[3] = g.sc->bytes;
  return trace_impl(g, i0, nc, rayFlags, out);
}

KGB_API int kgb_set_stream(kgb_engine* e, void* stream) {
  Engine& g = *E(e);
  CU(cudaStreamSynchronize(g.st));
  if (g.ownStream) CU(cudaStreamDestroy(g.st));
  g.ownStream = stream == nullptr;
  if (stream) g.st = static_cast<cudaStream_t>(stream);
  else CU(cudaStreamCreateWithFlags(&g.st, cudaStreamNonBlocking));
  return 1;
}

KGB_API int kgb_reduce(kgb_engine* e, size_t nc, const float* W, int useCos, double* out) {
  Engine& g = *E(e);
  if (nc == 0) return 1;
  if (nc != g.visN) return fail("gpu_reduce: no trace of this chunk");
  if (!upload(g.scratch, W, g.nDir * 4, g.st) || !grow(g.out, nc * 8) || !grow(g.w64, g.nDir * 8)) return 0;
  const float* N = static_cast<const float*>(g.N.p) + 3 * g.i0;
  double* w64 = static_cast<double*>(g.w64.p);
  if (g.bytes) launch_reduce_bytes(static_cast<const uint8_t*>(g.vis.p), uint32_t(nc), uint32_t(g.nDir), N, static_cast<const float*>(g.D.p),
                                   static_cast<const float*>(g.scratch.p), useCos, static_cast<double*>(g.out.p), g.st, w64);
  else launch_reduce_bits(static_cast<const uint32_t*>(g.vis.p), uint32_t(nc), uint32_t(g.nWords), uint32_t(g.nDir), N, static_cast<const float*>(g.D.p),
                          static_cast<const float*>(g.scratch.p), useCos, static_cast<double*>(g.out.p), g.st, w64);
  CU(cudaGetLastError());
  CU(cudaMemcpyAsync(out, g.out.p, nc * 8, cudaMemcpyDeviceToHost, g.st));
  CU(cudaStreamSynchronize(g.st));
  return 1;
}

namespace kgb {
// gpu_series's body; E's rows go to the sink (the caller's memory, or a file at an offset)
static int series_impl(Engine& g, size_t nc, const kgb_series_in* in, const Sink& out) {
  if (nc == 0 || in->T <= 0) return 1;
  if (in->Sdc && nc != g.dcN) return fail("gpu_series: no gpu_bounce rows for this chunk");
  if (nc != g.visN) return fail("gpu_series: no trace of this chunk");
  const size_t T = size_t(in->T);
  for (uint32_t d = 0; d < in->nSky; ++d) if (in->row[d] < 0 || in->row[d] >= in->P) return fail("gpu_series: a sky direction's row is not a patch");
  for (uint32_t j = 0; j < in->nSun; ++j) if (in->sunStep[j] < 0 || size_t(in->sunStep[j]) >= T) return fail("gpu_series: a sun step is not a column");
  if (in->nSky > g.nDir || size_t(in->sun0) + in->nSun > g.nDir) return fail("gpu_series: directions beyond the direction table");
  // one packed upload: row | wsky | S | g | G | sunStep | sunVec | sunW | Sdc, each 256-byte aligned
  const void* src[9] = {in->row, in->wsky, in->S, in->g, in->G, in->sunStep, in->sunVec, in->sunW, in->Sdc};
  const size_t len[9] = {size_t(in->nSky) * 4, size_t(in->nSky) * 4, size_t(in->P) * T * 4, T * 4, nc * 4, size_t(in->nSun) * 4,
                         size_t(in->nSun) * 12, size_t(in->nSun) * 4, in->Sdc ? g.nBins * T * 4 : 0};
  size_t off[9], total = 0;
  for (int k = 0; k < 9; ++k) { off[k] = total; total += (len[k] + 255) & ~size_t(255); }
  if (!grow(g.scratch, total) || !grow(g.out, nc * T * 4)) return 0;
  char* b = static_cast<char*>(g.scratch.p);
  for (int k = 0; k < 9; ++k)
    if (len[k] && !upload_large(g.staging, b + off[k], src[k], len[k], g.st)) return 0;
  SeriesArgs a{};
  a.bits = g.bytes ? nullptr : static_cast<const uint32_t*>(g.vis.p);
  a.bytes = g.bytes ? static_cast<const uint8_t*>(g.vis.p) : nullptr;
  a.nc = uint32_t(nc); a.nDir = uint32_t(g.nDir); a.nSky = in->nSky; a.T = uint32_t(T); a.nSun = in->nSun; a.sun0 = in->sun0;
  a.nBins = uint32_t(g.nBins);
  a.N = static_cast<const float*>(g.N.p) + 3 * g.i0; a.D = static_cast<const float*>(g.D.p);
  a.row = reinterpret_cast<const int32_t*>(b + off[0]); a.wsky = reinterpret_cast<const float*>(b + off[1]);
  a.S = reinterpret_cast<const float*>(b + off[2]); a.g = reinterpret_cast<const float*>(b + off[3]); a.G = reinterpret_cast<const float*>(b + off[4]);
  a.sunStep = reinterpret_cast<const int32_t*>(b + off[5]); a.sunVec = reinterpret_cast<const float*>(b + off[6]);
  a.sunW = reinterpret_cast<const float*>(b + off[7]);
  a.dc = in->Sdc ? static_cast<const float*>(g.dc.p) : nullptr;
  a.Sdc = in->Sdc ? reinterpret_cast<const float*>(b + off[8]) : nullptr;
  a.E = static_cast<float*>(g.out.p);
  // the tensor-core form: each sun direction on a column of its own (the reference's: one sun per sun-up step)
  std::vector<int32_t> sunOfCol(T, -1);
  bool tc = g.seriesForm == 0;
  for (uint32_t j = 0; tc && j < in->nSun; ++j) {
    if (sunOfCol[size_t(in->sunStep[j])] >= 0) tc = false;
    else sunOfCol[size_t(in->sunStep[j])] = int32_t(j);
  }
  if (!tc) {
    launch_series_fp32(a, g.st);
    CU(cudaGetLastError());
  } else {
    const uint32_t P = uint32_t(in->P), nBins = in->Sdc ? uint32_t(g.nBins) : 0u;
    const size_t Kp = (size_t(P) + 1 + nBins + 63) / 64 * 64;
    // directions per patch (CSR, each patch's directions in order)
    std::vector<int32_t> first(P + 1, 0), dirs(in->nSky);
    for (uint32_t d = 0; d < in->nSky; ++d) first[size_t(in->row[d]) + 1]++;
    for (uint32_t p = 0; p < P; ++p) first[p + 1] += first[p];
    {
      std::vector<int32_t> at(first.begin(), first.end() - 1);
      for (uint32_t d = 0; d < in->nSky; ++d) dirs[size_t(at[size_t(in->row[d])]++)] = int32_t(d);
    }
    const size_t csrBytes = (first.size() + dirs.size()) * 4;
    if (!grow(g.vop, 3 * nc * Kp * 2) || !grow(g.sop, 3 * T * Kp * 2) ||
        !grow(g.csr, csrBytes) || !grow(g.sunCol, T * 4)) return 0;
    int32_t* dFirst = static_cast<int32_t*>(g.csr.p);
    int32_t* dDirs = dFirst + first.size();
    CU(cudaMemcpyAsync(dFirst, first.data(), first.size() * 4, cudaMemcpyHostToDevice, g.st));
    if (!dirs.empty()) CU(cudaMemcpyAsync(dDirs, dirs.data(), dirs.size() * 4, cudaMemcpyHostToDevice, g.st));
    CU(cudaMemcpyAsync(g.sunCol.p, sunOfCol.data(), T * 4, cudaMemcpyHostToDevice, g.st));
    SeriesTcPlan p{};
    p.nc = uint32_t(nc); p.T = uint32_t(T); p.Kp = uint32_t(Kp); p.sun0 = in->sun0; p.numSMs = g.numSMs;
    p.v = g.vop.p; p.s = g.sop.p;
    p.sunOfCol = static_cast<const int32_t*>(g.sunCol.p); p.sunVec = a.sunVec; p.sunW = a.sunW;
    p.bits = a.bits; p.bytes = a.bytes; p.N = a.N; p.E = a.E; p.status = static_cast<uint32_t*>(g.ctl.p) + 1;
    p.waitLimitNs = g.seriesWaitNs; p.withholdFills = g.withholdFills;
    SeriesOperands o{};
    o.P = P; o.nBins = nBins; o.D = a.D; o.patchFirst = dFirst; o.patchDirs = dDirs; o.wsky = a.wsky; o.G = a.G; o.dc = a.dc;
    o.S = a.S; o.g = a.g; o.Sdc = a.Sdc; o.rebuildS = true;
    if (!reset_ctl(g)) return 0;
    build_series_operands(p, o, g.st);
    CU(cudaGetLastError());
    // E in bands of sensor rows: every band's kernel is queued on the engine's stream, and each band's rows go down
    // on the copy stream once its kernel is done, beside the next band's kernel (the first band's event also orders
    // the copies after this call's uploads, which used the same staging slices)
    const uint32_t mAll = uint32_t((nc + 127) / 128), bands = mAll >= 8 * kSeriesBands ? kSeriesBands : 1, per = (mAll + bands - 1) / bands;
    if (!g.copySt) CU(cudaStreamCreateWithFlags(&g.copySt, cudaStreamNonBlocking));
    CU(cudaEventRecord(g.ev[0], g.st));
    for (uint32_t b = 0; b < bands; ++b) {
      if (!g.bandEv[b]) CU(cudaEventCreateWithFlags(&g.bandEv[b], cudaEventDisableTiming));
      if (const char* why = series_tc_rows(p, b * per, std::min(per, mAll - b * per), g.st)) return fail(why);
      CU(cudaGetLastError());
      CU(cudaEventRecord(g.bandEv[b], g.st));
    }
    CU(cudaEventRecord(g.ev[1], g.st));
    // E straight into the caller's rows where they can be page-locked (registered while the first band runs)
    HostLock lock(out.fd < 0 ? out.dst : nullptr, nc * T * 4, false, g.copySt, g.st);
    Sink sink = out;
    sink.pinned = lock.direct;
    for (uint32_t b = 0; b < bands; ++b) {
      const size_t r0 = size_t(b) * per * 128, r1 = std::min(nc, size_t(b + 1) * per * 128);
      CU(cudaStreamWaitEvent(g.copySt, g.bandEv[b], 0));
      if (!download_to(g.staging, sink, r0 * T * 4, static_cast<const float*>(g.out.p) + r0 * T, (r1 - r0) * T * 4, g.copySt)) return 0;
    }
    uint32_t status = 0;
    CU(cudaMemcpyAsync(&status, static_cast<uint32_t*>(g.ctl.p) + 1, 4, cudaMemcpyDeviceToHost, g.st));
    CU(cudaStreamSynchronize(g.st));
    if (status & kStatusTimeout) return fail("gpu_series: the tensor-core pipeline timed out waiting (status recorded by the kernel)");
    g.stats.seriesMs += elapsed(g);
    g.stats.seriesOutputs += uint64_t(nc) * T;
    return 1;
  }
  HostLock lock(out.fd < 0 ? out.dst : nullptr, nc * T * 4, false, g.st);
  Sink sink = out;
  sink.pinned = lock.direct;
  return download_to(g.staging, sink, 0, g.out.p, nc * T * 4, g.st);
}
}  // namespace kgb

KGB_API int kgb_series(kgb_engine* e, size_t nc, const kgb_series_in* in, float* Eh) {
  Sink k;
  k.dst = Eh;
  return series_impl(*E(e), nc, in, k);
}

// gpu_series + the reference's fwrite of E (run.cpp:683-686) in one call: the rows go from the pinned staging slices
// into the file at byte offset (the .npy header's length plus i0 x T x 4 for a chunk starting at sensor i0), written
// by a few threads while the next slice comes down
KGB_API int kgb_series_file(kgb_engine* e, size_t nc, const kgb_series_in* in, int fd, uint64_t offset) {
  if (fd < 0) return fail("gpu_series: no file");
  Sink k;
  k.fd = fd;
  k.offset = offset;
  return series_impl(*E(e), nc, in, k);
}

KGB_API int kgb_sky(kgb_engine* e, int32_t mf, const kgb_sky_step* steps, size_t T, double grefl, int32_t sun, int32_t sky,
                    int32_t visible, float* out) {
  if (const char* why = sky_steps(mf, steps, T, grefl, sun, sky, visible, out, E(e)->st)) return fail(why);
  return 1;
}
KGB_API int kgb_triangulate(kgb_engine* e, const double* points, size_t nPoints, const int32_t* counts, size_t nFaces, const int32_t* indices,
                            const uint32_t* faceSlot, const double* c, uint32_t base, uint32_t slotBase, float* v, uint32_t* tri, uint32_t* slot,
                            size_t* made, int32_t* skipped) {
  if (!c || !made || !skipped || (nPoints && !v)) return fail("kgb_triangulate: the centre, v, made and skipped are required");
  const std::string why = triangulate_mesh(points, nPoints, counts, nFaces, indices, faceSlot, c, base, slotBase, v, tri, slot, made, skipped, E(e)->st);
  return why.empty() ? 1 : fail("kgb_triangulate: " + why);
}
KGB_API int kgb_thin_solids(kgb_engine* e, const double* points, size_t nPoints, const int32_t* counts, size_t nFaces, const int32_t* indices,
                            const uint32_t* faceSlot, uint32_t nSlots, const double* c, uint32_t* flags) {
  if (!c || (nSlots && !flags)) return fail("kgb_thin_solids: the centre and the flags are required");
  const std::string why = thin_solids(points, nPoints, counts, nFaces, indices, faceSlot, nSlots, c, flags, E(e)->st);
  return why.empty() ? 1 : fail("kgb_thin_solids: " + why);
}

KGB_API int kgb_mesh_read(kgb_engine* e, const void* data, size_t size, const char* name, kgb_mesh_info* info) {
  Engine& g = *E(e);
  const std::string label = name ? name : "";
  if (!info) return fail("kgb_mesh_read: no info to write");
  if (size && !data) return fail("kgb_mesh_read: no image");
  DmeshHeader h{};
  if (size < sizeof h) return fail(label + ": truncated");
  std::memcpy(&h, data, sizeof h);
  uint64_t payload = 0;
  const std::string why = dmesh_header(h, size, payload);
  if (!why.empty()) return fail(label + ": " + why);
  std::unique_ptr<DevMesh> m;
  if (!mesh_alloc(h, payload, label, m)) return 0;
  if (payload && !upload_large(g.staging, m->buf, static_cast<const char*>(data) + sizeof h, payload, g.st)) {
    cudaStreamSynchronize(g.st);
    return 0;
  }
  return mesh_keep(g, std::move(m), label, info);
}

KGB_API int kgb_mesh_file(kgb_engine* e, const char* path, kgb_mesh_info* info) {
  Engine& g = *E(e);
  const std::string p = path ? path : "";
  if (!info) return fail("kgb_mesh_file: no info to write");
  const int fd = open(p.c_str(), O_RDONLY | O_CLOEXEC);
  if (fd < 0) return fail("cannot open " + p);
  struct Closer { int fd; ~Closer() { close(fd); } } closer{fd};
  struct stat sb{};
  if (fstat(fd, &sb) != 0 || !S_ISREG(sb.st_mode)) return fail("cannot open " + p);
  const uint64_t size = uint64_t(sb.st_size);
  DmeshHeader h{};
  if (size < sizeof h || pread(fd, &h, sizeof h, 0) != ssize_t(sizeof h)) return fail(p + ": truncated");
  uint64_t payload = 0;
  const std::string why = dmesh_header(h, size, payload);
  if (!why.empty()) return fail(p + ": " + why);
  std::unique_ptr<DevMesh> m;
  if (!mesh_alloc(h, payload, p, m)) return 0;
  if (payload && !read_to_device(g, fd, sizeof h, payload, m->buf, p)) return 0;
  return mesh_keep(g, std::move(m), p, info);
}

KGB_API int kgb_mesh_download(kgb_engine* e, uint32_t id, double* points, int32_t* counts, int32_t* indices, uint16_t* slot) {
  Engine& g = *E(e);
  const DevMesh* m = find_mesh(g, id);
  if (!m) return fail("kgb_mesh_download: no mesh " + std::to_string(id));
  const MeshView& v = m->view;
  if (points && v.nPoints) CU(cudaMemcpyAsync(points, v.pts, v.nPoints * 24, cudaMemcpyDeviceToHost, g.st));
  if (counts && v.nFaces) CU(cudaMemcpyAsync(counts, v.counts, v.nFaces * 4, cudaMemcpyDeviceToHost, g.st));
  if (indices && v.nIdx) CU(cudaMemcpyAsync(indices, v.idx, v.nIdx * 4, cudaMemcpyDeviceToHost, g.st));
  if (slot && v.slot16 && v.nFaces) CU(cudaMemcpyAsync(slot, v.slot16, v.nFaces * 2, cudaMemcpyDeviceToHost, g.st));
  CU(cudaStreamSynchronize(g.st));
  return 1;
}

KGB_API int kgb_mesh_free(kgb_engine* e, uint32_t id) {
  Engine& g = *E(e);
  DevMesh* m = find_mesh(g, id);
  if (!m) return fail("kgb_mesh_free: no mesh " + std::to_string(id));
  CU(cudaStreamSynchronize(g.st));
  delete m;
  g.meshes[id] = nullptr;
  return 1;
}

KGB_API int kgb_mesh_thin_solids(kgb_engine* e, uint32_t id, const double* c, uint32_t* flags) {
  Engine& g = *E(e);
  const DevMesh* m = find_mesh(g, id);
  if (!m) return fail("kgb_mesh_thin_solids: no mesh " + std::to_string(id));
  if (!c || !flags) return fail("kgb_mesh_thin_solids: the centre and the flags are required");
  const std::string why = thin_solids_view(m->view, m->info.slots, c, flags, g.st);
  return why.empty() ? 1 : fail("kgb_mesh_thin_solids: " + why);
}

KGB_API int kgb_build_meshes(kgb_engine* e, const uint32_t* ids, size_t nMeshes, const uint8_t* blocks, const double* c, const kgb_slot* slots,
                             size_t nSlots, int perSlot, uint64_t* made, int32_t* skipped) {
  Engine& g = *E(e);
  if (!c || (nMeshes && !ids) || !slots || !nSlots) return fail("kgb_build_meshes: the centre, the ids and a slot table are required");
  delete g.sc;
  g.sc = new SceneObj;
  g.stats.gasBytes = 0;
  if (skipped) *skipped = 0;
  std::vector<const DevMesh*> ms(nMeshes);
  // run.cpp:101-106's ranges: points and at most tri_cap triangles of each blocking mesh, slots of every mesh
  std::vector<uint64_t> vBase(nMeshes + 1, 0), tBase(nMeshes + 1, 0), sBase(nMeshes + 1, 0);
  for (size_t k = 0; k < nMeshes; ++k) {
    ms[k] = find_mesh(g, ids[k]);
    if (!ms[k]) return fail("kgb_build_meshes: no mesh " + std::to_string(ids[k]));
    const bool b = !blocks || blocks[k];
    vBase[k + 1] = vBase[k] + (b ? ms[k]->info.nPoints : 0);
    tBase[k + 1] = tBase[k] + (b ? ms[k]->info.triCap : 0);
    sBase[k + 1] = sBase[k] + ms[k]->info.slots;
    if (made) made[k] = 0;
  }
  const uint64_t nPts = vBase.back(), nCap = tBase.back();
  if (nPts > 0xffffffffull || sBase.back() > 0xffffffffull) return fail("kgb_build_meshes: more than 2^32 - 1 points or slots");
  bool anyTau = false;
  for (size_t s = 0; s < nSlots; ++s) anyTau = anyTau || slots[s].tau > 0;
  const bool slotted = perSlot || anyTau;
  Buf dv, dtri, dslot, dtr, dslots;
  struct Release {   // the assembly's arrays go on every return (the scene keeps its own records)
    Buf* b[5];
    ~Release() { for (Buf* x : b) x->free(); }
  } release{{&dv, &dtri, &dslot, &dtr, &dslots}};
  if (!grow(dv, nPts * 12) || !grow(dtri, nCap * 12) || (slotted && !grow(dslot, nCap * 4))) return 0;
  uint64_t at = 0;
  int32_t skip = 0;
  for (size_t k = 0; k < nMeshes; ++k) {
    if (blocks && !blocks[k]) continue;
    uint64_t mk = 0;
    int32_t sk = 0;
    const std::string why = triangulate_view(ms[k]->view, c, uint32_t(vBase[k]), uint32_t(sBase[k]), static_cast<float*>(dv.p) + 3 * vBase[k],
                                             static_cast<uint32_t*>(dtri.p) + 3 * at, slotted ? static_cast<uint32_t*>(dslot.p) + at : nullptr, &mk, &sk,
                                             g.st);
    if (!why.empty()) return fail("kgb_build_meshes: " + why);
    if (made) made[k] = mk;
    at += mk;
    skip += sk;
  }
  if (skipped) *skipped = skip;
  const size_t nt = size_t(at);
  if (!nt) return 1;   // empty scene: every ray misses
  if (nt > (size_t(1) << 31)) return fail("gpu_build: more than 2^31 triangles");
  if (slotted) {
    uint32_t top = 0;
    thrust::device_ptr<const uint32_t> sl(static_cast<const uint32_t*>(dslot.p));
    top = thrust::reduce(thrust::cuda::par.on(g.st), sl, sl + nt, 0u, thrust::maximum<uint32_t>());
    if (top >= nSlots) return fail("gpu_build: a triangle's slot has no Slot");
    if (!upload(dslots, slots, nSlots * sizeof(kgb_slot), g.st) || !grow(dtr, nt)) return 0;
    launch_translucent(static_cast<const uint32_t*>(dslot.p), nt, static_cast<const kgb_slot*>(dslots.p), static_cast<uint8_t*>(dtr.p), g.st);
    CU(cudaGetLastError());
  }
  return build_scene(g, static_cast<const float*>(dv.p), size_t(nPts), static_cast<const uint32_t*>(dtri.p), nt,
                     slotted ? static_cast<const uint32_t*>(dslot.p) : nullptr, slotted ? static_cast<const uint8_t*>(dtr.p) : nullptr, true);
}

KGB_API int kgb_sky_ladybug(kgb_engine* e, int32_t mf, const double* steps, size_t T, double lat, double lon, double tz, double grefl,
                            double durationHours, double* lb, float* acc, float* S, float* g) {
  if (!lb) return fail("kgb_sky_ladybug: no weights to write");
  if (const char* why = sky_ladybug(mf, steps, T, lat, lon, tz, grefl, durationHours, lb, acc, S, g, E(e)->st)) return fail(why);
  return 1;
}
KGB_API int kgb_sun_noaa(kgb_engine* e, const double* in, size_t T, double* out) {
  if (const char* why = sun_steps(in, T, out, E(e)->st)) return fail(why);
  return 1;
}

KGB_API int kgb_set_builder(kgb_engine* e, int which) {
  if (which != 0 && which != 1) return fail("kgb_set_builder: 0 (host binned SAH) or 1 (device LBVH)");
  E(e)->builder = which;
  return 1;
}

KGB_API int kgb_set_limits(kgb_engine* e, uint32_t nodeLimit, uint64_t bounceLimitNs, uint64_t seriesWaitNs, uint32_t flags) {
  Engine& g = *E(e);
  if (flags & ~KGB_LIMIT_WITHHOLD_FILLS) return fail("kgb_set_limits: unknown flags");
  g.nodeLimit = nodeLimit;
  g.bounceLimitNs = bounceLimitNs ? std::min(bounceLimitNs, kBounceLimitNs) : kBounceLimitNs;
  g.seriesWaitNs = seriesWaitNs;
  g.withholdFills = (flags & KGB_LIMIT_WITHHOLD_FILLS) != 0;
  return 1;
}

KGB_API int kgb_set_series_form(kgb_engine* e, int form) {
  if (form != 0 && form != 1) return fail("kgb_set_series_form: 0 (tensor cores) or 1 (plain FP32)");
  E(e)->seriesForm = form;
  return 1;
}

// gpu.cu:533-568: the whole chunk over sample ranges [done, done + n): n from 2^13 / nc (1..64), then ~100 ms, at most
// doubling; cancel between launches. One thread per path, then per sensor the paths' contributions are added in
// sample order: deterministic, whatever the launch boundaries.
KGB_API int kgb_bounce(kgb_engine* e, size_t i0, size_t nc, uint32_t rayFlags, const kgb_bounce_in* b) {
  Engine& g = *E(e);
  if (i0 + nc > g.nSensors) return fail("gpu_bounce: sensor range exceeds the scene");
  const uint32_t mf = uint32_t(b->mf);
  g.nBins = size_t(144 * mf * mf + 1) + 1; g.dcN = nc; g.dcI0 = i0;
  if (!grow(g.dc, g.nBins * nc * 4)) return 0;
  if (nc == 0) return 1;
  CU(cudaMemsetAsync(g.dc.p, 0, g.nBins * nc * 4, g.st));
  const double rad = b->north * KGB_PI_D / 180;
  BounceArgs a{};
  a.nodes = static_cast<const Node8*>(g.sc->nodes.p); a.tris = static_cast<const TriRec*>(g.sc->tris.p); a.nNodes = walk_nodes(g);
  a.P = static_cast<const float*>(g.P.p); a.N = static_cast<const float*>(g.N.p);
  a.i0 = uint32_t(i0); a.n = uint32_t(nc); a.nc = uint32_t(nc);
  a.M = b->M; a.nBounce = b->N; a.mf = mf; a.nBins = uint32_t(g.nBins);
  a.alpha = float((KGB_PI_D / 2.) / (7 * mf + .5)); a.cosN = float(std::cos(rad)); a.sinN = float(std::sin(rad));
  a.rayFlags = rayFlags; a.slots = static_cast<const kgb_slot*>(g.slots.p); a.nSlots = g.nSlots;
  a.slotLog = static_cast<const float2*>(g.slotLog.p);
  a.dc = static_cast<float*>(g.dc.p); a.status = static_cast<uint32_t*>(g.ctl.p) + 1;
  a.limitNs = g.bounceLimitNs;
  // paths of a launch: at most 2^23 (their results 64 MiB, the two queues of paths that go on 768 MiB)
  const size_t nCap = std::max<size_t>(1, (size_t(1) << 23) / nc);
  if (!g.gridStep) g.gridStep = g.numSMs * bounce_step_blocks_per_sm();
  // the reference starts at 2^13 / nc samples (1..64); here also at least ~4 paths per resident thread (a path a thread)
  const size_t fill = (size_t(4) * size_t(g.numSMs) * 2048 + nc - 1) / nc;
  for (size_t done = 0, n = std::max(std::clamp<size_t>((size_t(1) << 13) / nc, 1, 64), fill); done < b->M;) {
    if (b->cancel && b->cancel(b->cancelCtx)) return fail("cancelled");
    n = std::min({n, size_t(b->M) - done, nCap});
    if (!grow(g.contrib, n * nc * 8) || !grow(g.bq, 2 * n * nc * bounce_state_bytes())) return 0;
    a.contrib = static_cast<uint2*>(g.contrib.p);
    a.s0 = uint32_t(done); a.s1 = uint32_t(done + n);
    if (!bounce_order(g, a.s0, a.s1, b->M)) return 0;
    a.order = static_cast<const uint32_t*>(g.border.p);
    if (!reset_ctl(g)) return 0;
    CU(cudaEventRecord(g.ev[0], g.st));
    launch_bounce(a, static_cast<PathState*>(g.bq.p), static_cast<uint32_t*>(g.ctl.p) + 28, g.gridStep, g.st);
    CU(cudaEventRecord(g.ev[1], g.st));
    uint32_t ctl[32] = {};
    CU(cudaMemcpyAsync(ctl, g.ctl.p, 128, cudaMemcpyDeviceToHost, g.st));
    CU(cudaStreamSynchronize(g.st));
    CU(cudaGetLastError());
    const unsigned long long segments = (unsigned long long)ctl[2] | ((unsigned long long)ctl[3] << 32);
    std::string where;
    if (ctl[16]) {   // the first path whose walk gave up
      const auto f = [&](int k) { float x; std::memcpy(&x, &ctl[k], 4); char b[32]; std::snprintf(b, sizeof b, "%.9g", x); return std::string(b); };
      where = "; first walk that gave up: sensor " + std::to_string(ctl[17]) + " sample " + std::to_string(ctl[18]) + " segment " +
              std::to_string(ctl[19]) + ", origin (" + f(20) + ", " + f(21) + ", " + f(22) + "), direction (" + f(23) + ", " + f(24) + ", " +
              f(25) + ")";
    }
    if (ctl[1] & kStatusTimeout) {
      char lim[32];
      std::snprintf(lim, sizeof lim, "%.9g s", double(g.bounceLimitNs) * 1e-9);
      return fail("gpu_bounce: a launch of " + std::to_string(n) + " samples x " + std::to_string(nc) + " sensors passed its " + lim +
                  " limit after " + std::to_string(segments) + " path segments" + where);
    }
    if (ctl[1] & kStatusVisitLimit)
      return fail("gpu_bounce: traversal gave up (a walk passed its node-visit limit, or met a node index beyond the BVH)" + where);
    if (!sync_status(g)) return 0;
    const double ms = elapsed(g);
    g.stats.bounceMs += ms; g.stats.paths += n * nc; g.stats.bounceLaunches++;
    done += n;
    const double want = double(n) * 100 / std::max(ms, 1e-3);
    n = std::max<size_t>(1, std::min<size_t>(2 * n, want > 1e9 ? size_t(1e9) : size_t(want)));
  }
  return 1;
}

KGB_API int kgb_reduce_dc(kgb_engine* e, size_t nc, const float* W, double* out) {
  Engine& g = *E(e);
  if (nc == 0) return 1;
  if (nc != g.dcN) return fail("gpu_reduce_dc: no gpu_bounce rows for this chunk");
  if (!upload(g.scratch, W, g.nBins * 4, g.st) || !grow(g.out, nc * 8)) return 0;
  launch_reduce_dc(static_cast<const float*>(g.dc.p), uint32_t(nc), uint32_t(g.nBins), static_cast<const float*>(g.scratch.p), static_cast<double*>(g.out.p), g.st);
  CU(cudaGetLastError());
  CU(cudaMemcpyAsync(out, g.out.p, nc * 8, cudaMemcpyDeviceToHost, g.st));
  CU(cudaStreamSynchronize(g.st));
  return 1;
}

KGB_API int kgb_download_dc(kgb_engine* e, size_t nc, float* out, size_t count) {
  Engine& g = *E(e);
  if (nc != g.dcN) return fail("gpu_download_dc: no gpu_bounce rows for this chunk");
  if (count != g.nBins * nc) return fail("gpu_download_dc: wrong element count");
  if (count) CU(cudaMemcpyAsync(out, g.dc.p, count * 4, cudaMemcpyDeviceToHost, g.st));
  CU(cudaStreamSynchronize(g.st));
  return 1;
}
KGB_API int kgb_download_bits(kgb_engine* e, size_t nc, uint32_t* out, size_t count) {
  Engine& g = *E(e);
  if (g.bytes) return fail("gpu_download_bits: the last trace wrote bytes");
  if (count != g.nWords * nc || nc != g.visN) return fail("gpu_download_bits: wrong element count");
  if (count) CU(cudaMemcpyAsync(out, g.vis.p, count * 4, cudaMemcpyDeviceToHost, g.st));
  CU(cudaStreamSynchronize(g.st));
  return 1;
}
KGB_API int kgb_download_bytes(kgb_engine* e, size_t nc, uint8_t* out, size_t count) {
  Engine& g = *E(e);
  if (!g.bytes) return fail("gpu_download_bytes: the last trace wrote bits");
  if (count != g.nDir * nc || nc != g.visN) return fail("gpu_download_bytes: wrong element count");
  if (count) CU(cudaMemcpyAsync(out, g.vis.p, count, cudaMemcpyDeviceToHost, g.st));
  CU(cudaStreamSynchronize(g.st));
  return 1;
}

// gpu.cu:572-610: sub-launches of 2^13 threads first and at least, then ~40 ms, at most doubling, the size carried
// from chunk to chunk in *launch; cancel between them.
KGB_API int kgb_view(kgb_engine* e, size_t i0, size_t nc, uint32_t rayFlags, const kgb_view_in* v, size_t* launch) {
  Engine& g = *E(e);
  if (i0 + nc > g.nSensors) return fail("gpu_view: sensor range exceeds the scene");
  const size_t K = size_t(v->nAz) * v->nEl, nWords = (K + 31) / 32;
  if (g.nLabel && g.nLabel < g.sc->nTris) return fail("gpu_view: fewer labels than the scene's triangles");
  if (!grow(g.viewCls, K * nc) || !grow(g.viewDist, K * nc * 4) || !upload(g.rowSin, v->rowSin, size_t(v->nEl) * 8, g.st)) return 0;
  g.viewN = nc; g.viewK = K; g.viewI0 = i0; g.view = *v; g.view.rowSin = nullptr;
  if (nc == 0 || K == 0) { CU(cudaStreamSynchronize(g.st)); return 1; }
  if (!g.gridView) g.gridView = g.numSMs * view_blocks_per_sm();
  const double rad = v->north * KGB_PI_D / 180;
  ViewArgs a{};
  a.nodes = static_cast<const Node8*>(g.sc->nodes.p); a.tris = static_cast<const TriRec*>(g.sc->tris.p); a.nNodes = walk_nodes(g);
  a.P = static_cast<const float*>(g.P.p); a.N = static_cast<const float*>(g.N.p);
  a.stride = uint32_t(nc); a.i0 = uint32_t(i0); a.K = uint32_t(K); a.nWords = uint32_t(nWords); a.nAz = v->nAz; a.nEl = v->nEl;
  a.rayFlags = rayFlags; a.rowSin = static_cast<const float*>(g.rowSin.p); a.az0 = v->az0; a.dAz = v->dAz; a.groundZ = v->groundZ;
  a.cosN = float(std::cos(rad)); a.sinN = float(std::sin(rad));
  a.world = v->world ? 1 : 0; a.cull = v->cull ? 1 : 0; a.jitter = v->jitter ? 1 : 0; a.nS = v->nS; a.back = v->back ? 1 : 0;
  a.vground = v->vground ? 1 : 0;
  a.label = g.nLabel ? static_cast<const uint8_t*>(g.label.p) : nullptr;
  a.cls = static_cast<uint8_t*>(g.viewCls.p); a.dist = static_cast<float*>(g.viewDist.p);
  a.counter = static_cast<uint32_t*>(g.ctl.p); a.status = static_cast<uint32_t*>(g.ctl.p) + 1;
  // gpu.cu:590: sub-launches of at least 2^13 threads there; here at least four (32 sensors x word) tasks for each
  // resident warp, so that no launch leaves the GPU idle; then ~40 ms, at most doubling, as the reference
  const size_t nMin = std::max<size_t>((size_t(1) << 13) / nWords, (size_t(4) * g.gridView * 8 * 32 + nWords - 1) / nWords);
  size_t n = std::max(*launch, nMin);
  for (size_t done = 0; done < nc;) {
    if (v->cancel && v->cancel(v->cancelCtx)) return fail("cancelled");
    const size_t m = std::min(n, nc - done);
    a.first = uint32_t(i0 + done); a.n = uint32_t(m); a.out0 = uint32_t(done);
    if (!reset_ctl(g)) return 0;
    const size_t tasks = (m + 31) / 32 * nWords;
    const int grid = int(std::min<size_t>(size_t(g.gridView), (tasks + 7) / 8));
    CU(cudaEventRecord(g.ev[0], g.st));
    launch_view(a, grid, g.st);
    CU(cudaEventRecord(g.ev[1], g.st));
    if (!sync_status(g)) return 0;
    const double ms = elapsed(g);
    g.stats.traceMs += ms; g.stats.rays += m * K; g.stats.launches++;
    done += m;
    const double want = double(m) * 40 / std::max(ms, 1e-3);
    n = std::max(nMin, std::min(2 * n, want > 1e12 ? size_t(1) << 40 : size_t(want)));
  }
  *launch = n;   // the caller passes it to the next chunk
  return 1;
}

KGB_API int kgb_reduce_view(kgb_engine* e, size_t nc, const double* wRow, size_t nRow, uint32_t nClass, double farDist,
                            const float* reach, size_t nReach, int glazing, uint32_t isoDim, double* out) {
  Engine& g = *E(e);
  if (nc == 0) return 1;
  if (nc != g.viewN) return fail("gpu_reduce_view: no gpu_view for this chunk");
  if (nClass > KGB_VIEW_CLASSES || nReach > 8) return fail("gpu_reduce_view: at most 16 groups and 8 reach distances");
  const size_t NA = 3 * size_t(nClass) + 1 + nReach + (glazing ? 1 : 0) + (isoDim ? 1 : 0);
  if (nRow < g.view.nEl) return fail("gpu_reduce_view: fewer row weights than rows");
  if (!upload(g.scratch, wRow, nRow * 8, g.st) || !grow(g.out, nc * NA * 8)) return 0;
  ViewReduceArgs a{};
  a.cls = static_cast<const uint8_t*>(g.viewCls.p); a.dist = static_cast<const float*>(g.viewDist.p);
  a.nc = uint32_t(nc); a.K = uint32_t(g.viewK); a.nAz = g.view.nAz; a.nEl = g.view.nEl; a.nClass = nClass; a.nReach = uint32_t(nReach);
  a.glazing = glazing ? 1 : 0; a.iso = isoDim ? 1 : 0; a.NA = uint32_t(NA);
  a.wRow = static_cast<const double*>(g.scratch.p); a.farDist = float(farDist); a.lnFar = std::log(farDist);
  for (size_t r = 0; r < nReach; ++r) a.reach[r] = reach[r];
  a.isoDim = isoDim; a.world = g.view.world ? 1 : 0; a.jitter = g.view.jitter ? 1 : 0; a.i0 = uint32_t(g.viewI0); a.nS = g.view.nS;
  a.back = g.view.back ? 1 : 0; a.az0 = g.view.az0; a.dAz = g.view.dAz; a.rowSin = static_cast<const float*>(g.rowSin.p);
  a.out = static_cast<double*>(g.out.p);
  launch_reduce_view(a, g.st);
  CU(cudaGetLastError());
  CU(cudaMemcpyAsync(out, g.out.p, nc * NA * 8, cudaMemcpyDeviceToHost, g.st));
  CU(cudaStreamSynchronize(g.st));
  return 1;
}

// gpu.cu:720-734 transposes the device's [K x nc] on the host; here the transpose runs on the device (rows.cu), in
// sensor slices of at most 64 MiB of rows, each downloaded through the pinned staging slices.
KGB_API int kgb_download_view(kgb_engine* e, size_t nc, uint8_t* cls, float* dist, size_t count) {
  Engine& g = *E(e);
  if (nc != g.viewN) return fail("gpu_download_view: no gpu_view for this chunk");
  const size_t K = g.viewK;
  if (count != nc * K) return fail("gpu_download_view: wrong element count");
  return download_rows(g, g.viewCls.p, 1, K, nc, cls) && download_rows(g, g.viewDist.p, 4, K, nc, dist);
}

// The last trace's visibility as one row per sensor: [nc x nWords] words or [nc x nDir] bytes (run.cpp:659-671, the
// --dump-bits rows, transposed on the device instead of the host).
KGB_API int kgb_download_bits_rows(kgb_engine* e, size_t nc, uint32_t* out, size_t count) {
  Engine& g = *E(e);
  if (g.bytes) return fail("gpu_download_bits: the last trace wrote bytes");
  if (count != g.nWords * nc || nc != g.visN) return fail("gpu_download_bits: wrong element count");
  return download_rows(g, g.vis.p, 4, g.nWords, nc, out);
}
KGB_API int kgb_download_bytes_rows(kgb_engine* e, size_t nc, uint8_t* out, size_t count) {
  Engine& g = *E(e);
  if (!g.bytes) return fail("gpu_download_bytes: the last trace wrote bits");
  if (count != g.nDir * nc || nc != g.visN) return fail("gpu_download_bytes: wrong element count");
  return download_rows(g, g.vis.p, 1, g.nDir, nc, out);
}

KGB_API kgb_stats kgb_get_stats(const kgb_engine* e) { return E(e)->stats; }
KGB_API uint32_t kgb_ray_flags(int cullBackfaces, int translucent) {
  return KGB_RAY_TERMINATE_ON_FIRST_HIT | (translucent ? 0u : KGB_RAY_DISABLE_ANYHIT) | (cullBackfaces ? KGB_RAY_CULL_BACK_FACING : 0u);
}
KGB_API uint32_t kgb_bounce_flags(int cullBackfaces) { return KGB_RAY_DISABLE_ANYHIT | (cullBackfaces ? KGB_RAY_CULL_BACK_FACING : 0u); }
KGB_API void kgb_dims(const kgb_engine* e, uint64_t out[6]) {
  const Engine& g = *E(e);
  out[0] = g.nSensors; out[1] = g.nDir; out[2] = g.nWords; out[3] = g.nBins; out[4] = g.viewK; out[5] = g.bytes ? 1 : 0;
}

}  // extern "C"
