// Internal interface between the engine's translation units: launch argument blocks of the kernels and the host
// BVH builder. Not part of the public ABI (include/kitsim_gb300.h is).
#pragma once
#include <cuda_runtime.h>
#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>
#include "kitsim_gb300.h"

namespace kgb {

// BVH8 node record (rt.cuh): 52 words = 208 bytes; a node's childBase field holds 24 bits, so a tree has fewer than
// 2^24 nodes (a scene of nt triangles has at most nt / 2 + 2).
constexpr uint32_t kNodeWords = 52;
constexpr uint32_t kNodeBytes = 4 * kNodeWords;
constexpr uint32_t kMaxNodes = 1u << 24;

struct Node8;
struct TriRec;
struct RayDir;

enum : uint32_t { kStatusStackOverflow = 1u, kStatusTimeout = 2u, kStatusVisitLimit = 4u };

// the calling thread's message for kgb_last_error (engine.cu); returns 0 for the C ABI's failure status
int set_error(const std::string& message);

// k_bits / k_bytes: sensors [first, first + n) of the engine's arrays, written to columns [out0, out0 + n) of a chunk
// whose row stride is `stride` sensors.
struct TraceArgs {
  const Node8* nodes;
  const TriRec* tris;
  uint32_t nNodes;
  const float* P;
  const float* N;
  const float* D;
  uint32_t first, n, out0, stride;
  uint32_t nDir, nWords, rayFlags;
  uint32_t* bits;
  uint8_t* bytes;
  const kgb_slot* slots;
  uint32_t nSlots;
  uint32_t* counter;
  uint32_t* status;
  const RayDir* rayTab;   // the directions' precomputed ray parts (k_bits), or null
  const float2* slotLog;  // [nSlots]: ln tn per slot as a float pair (k_slot_logs)
  // Tracing order. Null: sensors first .. first + n - 1, output columns out0 .. out0 + n - 1. Otherwise the call's sensors
  // grouped by normal orientation: order lists every sensor of the scene, stably partitioned into six classes (the
  // dominant axis of the normal and its sign); the call's range is, per class, a contiguous run of it. Position p of the
  // call (p0 + i for lane position i of this launch) is sensor order[pieceG[c] + p] for the class c whose run holds it
  // (pieceEnd[c - 1] <= p < pieceEnd[c]), written to output column sensor - callI0.
  const uint32_t* order;
  uint32_t p0, callI0;
  uint32_t pieceG[6], pieceEnd[6];
};

struct ViewArgs {
  const Node8* nodes;
  const TriRec* tris;
  uint32_t nNodes;
  const float* P;
  const float* N;
  uint32_t first, n, out0, stride, i0;
  uint32_t K, nWords, nAz, nEl, rayFlags;
  const float* rowSin;   // device [2 nEl]
  float az0, dAz, groundZ, cosN, sinN;
  uint32_t world, cull, jitter, nS, back, vground;
  const uint8_t* label;  // device, null: every hit an obstruction
  uint8_t* cls;
  float* dist;
  uint32_t* counter;
  uint32_t* status;
};

// The bounce's step kernels end their remaining paths and fail the call once a step has run this long.
constexpr uint64_t kBounceLimitNs = 10000000000ull;   // 10 s

struct PathState;   // a path between segments (trace.cu)
struct BounceArgs {
  const Node8* nodes;
  const TriRec* tris;
  uint32_t nNodes;
  const float* P;
  const float* N;
  uint32_t i0, n, nc;
  uint32_t s0, s1, M, nBounce, mf, nBins;
  float alpha, cosN, sinN;
  uint32_t rayFlags;
  const kgb_slot* slots;
  uint32_t nSlots;
  float* dc;
  uint2* contrib;     // [(s1 - s0) x n]: each path's sky bin (or none) and contribution
  uint32_t* status;
  const uint32_t* order;   // [s1 - s0]: the launch's samples in tracing order (sensor-major), or null (sample-major)
  const float2* slotLog;   // [nSlots]: ln tn per slot as a float pair (k_slot_logs)
  const PathState* qIn;    // the paths a step continues, and their count
  const uint32_t* qInCount;
  PathState* qOut;         // the paths that go on after it, appended
  uint32_t* qOutCount;
  uint64_t limitNs;        // a step kernel's time limit (kBounceLimitNs unless lowered by kgb_set_limits)
};

void launch_ray_table(const float* D, uint32_t nDir, void* tab, cudaStream_t st);   // 48 bytes per direction
// The sensors' orientation classes (TraceArgs::order) against the classes in cls: cls updated, flags[0] = 1 where one
// differs, flags[1 + c] += the sensors of class c (flags zeroed by the caller).
void launch_sensor_classes(const float* N, uint32_t n, uint8_t* cls, uint32_t* flags, cudaStream_t st);
void launch_slot_logs(const kgb_slot* slots, uint32_t n, float2* out, cudaStream_t st);   // ln tn per slot, a float pair
// rows.cu: out[i K + d] = in[d ld + i] for d < K, i < m, elements of 1 or 4 bytes; false if the grid cannot hold K
bool launch_rows(const void* in, size_t ld, void* out, size_t esize, uint32_t K, uint32_t m, cudaStream_t st);
int bytes_blocks_per_sm();
int view_blocks_per_sm();
int bits_blocks_per_sm();
void launch_bits(const TraceArgs& a, int grid, cudaStream_t st, bool count = false);
void launch_bytes(const TraceArgs& a, int grid, cudaStream_t st);
void launch_view(const ViewArgs& a, int grid, cudaStream_t st);
void launch_bounce(const BounceArgs& a, PathState* queues, uint32_t* qCount, int stepGrid, cudaStream_t st);
size_t bounce_state_bytes();   // one queued path
int bounce_step_blocks_per_sm();

// reductions (reduce.cu)
// w64: a device array of nDir doubles for the weights (the fast form), or null (the weights staged per block in
// shared memory: for callers with no room for the array)
void launch_reduce_bits(const uint32_t* bits, uint32_t nc, uint32_t nWords, uint32_t nDir, const float* N, const float* D, const float* W,
                        int useCos, double* out, cudaStream_t st, double* w64 = nullptr);
void launch_reduce_bytes(const uint8_t* bytes, uint32_t nc, uint32_t nDir, const float* N, const float* D, const float* W, int useCos,
                         double* out, cudaStream_t st, double* w64 = nullptr);
void launch_reduce_dc(const float* dc, uint32_t nc, uint32_t nBins, const float* W, double* out, cudaStream_t st);
struct ViewReduceArgs {
  const uint8_t* cls;
  const float* dist;
  uint32_t nc, K, nAz, nEl, nClass, nReach, glazing, iso, NA;
  const double* wRow;
  float farDist;
  double lnFar;
  float reach[8];
  // isovist
  uint32_t isoDim, world, jitter, i0, nS, back;
  float az0, dAz;
  const float* rowSin;
  double* out;
};
void launch_reduce_view(const ViewReduceArgs& a, cudaStream_t st);

// time series (series.cu): the plain FP32 form, visibility bits or bytes
struct SeriesArgs {
  const uint32_t* bits;
  const uint8_t* bytes;
  uint32_t nc, nDir, nSky, T, nSun, sun0, nBins;
  const float* N;
  const float* D;
  const int32_t* row;
  const float* wsky;
  const float* S;
  const float* g;
  const float* G;
  const int32_t* sunStep;
  const float* sunVec;
  const float* sunW;
  const float* dc;     // null: no reflected light
  const float* Sdc;
  float* E;
};
void launch_series_fp32(const SeriesArgs& a, cudaStream_t st);

// time series on the tensor cores (series_tc.cu): split-BF16 operands, tcgen05 MMA, then the sun term in a pass over E
struct SeriesTcPlan {
  uint32_t nc, T, Kp, sun0;
  int numSMs;
  void* v;                 // [3 x nc x Kp] bf16: the pieces hi, mid, lo of V, one after the other
  void* s;                 // [3 x T x Kp] bf16: the same of S^T
  const int32_t* sunOfCol; // [T]: the sun direction of column t, or -1
  const float* sunVec;
  const float* sunW;
  const uint32_t* bits;
  const uint8_t* bytes;
  const float* N;          // the chunk's normals
  float* E;                // [nc x T]
  uint32_t* status;
  uint64_t waitLimitNs = 0;   // the pipeline's waits give up past this (0: the default, 4 s)
  bool withholdFills = false; // the producer issues no fills (kgb_set_limits' test of the bounded waits)
};
struct SeriesOperands {
  uint32_t P, nBins;
  const float* D;
  const int32_t* patchFirst;
  const int32_t* patchDirs;
  const float* wsky;
  const float* G;
  const double* G64;   // when G is null: the ground sums as doubles, rounded to float here (a serving batch's reduce)
  const float* dc;
  const float* S;
  const float* g;
  const float* Sdc;
  bool rebuildS;
  bool buildV = true;  // false: S^T only (a serving request's pieces, built once at its upload)
};
void build_series_operands(const SeriesTcPlan& p, const SeriesOperands& o, cudaStream_t st);
const char* series_tc(const SeriesTcPlan& p, cudaStream_t st);   // null, or what failed
// the rows of 128-sensor tiles mBase .. mBase + mCount - 1 only (E's rows mBase * 128 .. , the others untouched)
const char* series_tc_rows(const SeriesTcPlan& p, uint32_t mBase, uint32_t mCount, cudaStream_t st);
// n whole contractions (each its own operands, K and output) in one launch of the same kernel (at most
// kMaxSeriesGroup); each output is the one series_tc would give it, bit for bit
constexpr uint32_t kMaxSeriesGroup = 48;
const char* series_tc_group(const SeriesTcPlan* plans, uint32_t n, cudaStream_t st);

// What a reduce of the last trace reads, for the reduce entry points outside engine.cu (reduce_noalloc.cu).
struct ReduceInputs {
  int device;
  cudaStream_t st;
  size_t visN, nDir, nWords;   // sensors of the last trace, directions, 32-direction words
  bool bytes;                  // the last trace wrote transmittance bytes (else bits)
  const uint32_t* bitsVis;
  const uint8_t* bytesVis;
  const float* N;              // the traced chunk's normals
  const float* D;
};
void engine_reduce_inputs(kgb_engine* e, ReduceInputs& in);

// sky (sky.cu): Perez sky of T steps, NOAA sun positions; null or what failed
const char* sky_steps(int mf, const kgb_sky_step* steps, size_t T, double grefl, int sun, int sky, int visible, float* out, cudaStream_t st);
const char* sun_steps(const double* in, size_t T, double* out, cudaStream_t st);
// A mesh's arrays on the device, as the .dmesh format lays them out, and each face's first index.
struct MeshView {
  const double* pts;         // [nPoints x 3]
  const int32_t* counts;     // [nFaces]
  const int32_t* idx;        // [nIdx]
  const uint64_t* idxOff;    // [nFaces]
  const uint16_t* slot16;    // [nFaces] the faces' slots as the image holds them, or null
  const uint32_t* slot32;    // [nFaces] the same as a caller's 32-bit array, or null (neither: slot 0)
  uint64_t nPoints, nFaces, nIdx;
};
// A mesh the engine keeps (kgb_mesh_read / kgb_mesh_file): one allocation holding points, counts, indices and slots in
// the image's order (the image's payload copied as it is), then the face offsets at a 256-byte boundary.
struct DevMesh {
  void* buf = nullptr;
  size_t bytes = 0;
  MeshView view{};
  kgb_mesh_info info{};
  DevMesh() = default;
  DevMesh(const DevMesh&) = delete;
  DevMesh& operator=(const DevMesh&) = delete;
  ~DevMesh() { if (buf) cudaFree(buf); }
};
// mesh.cu: the reference's array checks on a copied image (mesh_ok), then the face offsets, bounds, largest face,
// largest slot and tri_cap into m.info; "" or the rule that failed, as the reference words it (without the label)
std::string mesh_check(DevMesh& m, cudaStream_t st);
// mesh.cu: the faces of a mesh on the device as triangles into device arrays: v [nPoints x 3] (recentred on c), tri at
// most tri_cap triangles (vertex indices + base), slot (slotBase + the face's slot) or null; *made and *skipped as
// kgb_triangulate's. "" or what failed.
std::string triangulate_view(const MeshView& m, const double* c, uint32_t base, uint32_t slotBase, float* v, uint32_t* tri, uint32_t* slot,
                             uint64_t* made, int32_t* skipped, cudaStream_t st);
// mesh.cu: kgb_thin_solids over a mesh on the device; flags in host memory [nSlots] (every face's slot below nSlots)
std::string thin_solids_view(const MeshView& m, uint32_t nSlots, const double* c, uint32_t* flags, cudaStream_t st);
// mesh.cu: translucent[k] = slots[slot[k]].tau > 0 for device arrays (slots [nSlots] in device memory)
void launch_translucent(const uint32_t* slot, size_t nt, const kgb_slot* slots, uint8_t* translucent, cudaStream_t st);
// the scene's preparation on the GPU (mesh.cu): "" or what failed
std::string triangulate_mesh(const double* points, size_t nPoints, const int32_t* counts, size_t nFaces, const int32_t* indices, const uint32_t* faceSlot,
                             const double* c, uint32_t base, uint32_t slotBase, float* v, uint32_t* tri, uint32_t* slot, size_t* made, int32_t* skipped,
                             cudaStream_t st);
std::string thin_solids(const double* points, size_t nPoints, const int32_t* counts, size_t nFaces, const int32_t* indices, const uint32_t* faceSlot,
                        uint32_t nSlots, const double* c, uint32_t* flags, cudaStream_t st);
// ladybug mode's sky (kgb_sky_ladybug); null or what failed
const char* sky_ladybug(int mf, const double* steps, size_t T, double lat, double lon, double tz, double grefl, double durationHours,
                        double* lb, float* acc, float* S, float* g, cudaStream_t st);

// host BVH builder (bvh_build.cpp): binned-SAH binary BVH, collapsed to the 8-wide float-plane layout of rt.cuh
struct BvhOut {
  std::vector<uint32_t> nodes;   // kNodeWords words per node
  std::vector<float> tris;       // 12 words per triangle record
  uint32_t nNodes = 0;
};
void build_bvh8(const float* v, size_t nv, const uint32_t* tri, size_t nt, const uint32_t* slot, const uint8_t* translucent, BvhOut& out);
// device builder (bvh_gpu.cu): the same records, built on the GPU from a Morton-ordered radix tree; the input arrays
// in host or device memory (copied by kind cudaMemcpyDefault); "" or what failed
std::string build_bvh8_gpu(const float* v, size_t nv, const uint32_t* tri, size_t nt, const uint32_t* slot, const uint8_t* translucent,
                           cudaStream_t st, void** nodesOut, void** trisOut, uint32_t* nNodesOut, uint64_t* tempBytes);

}  // namespace kgb
