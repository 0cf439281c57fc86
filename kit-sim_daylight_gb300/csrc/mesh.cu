// The scene's preparation on the GPU (compiled with -fmad=false: the double arithmetic restates the reference's host
// code operation by operation, so the float vertices and the chosen triangles equal its own):
//  - mesh_check: the array rules the reference applies to a .dmesh image (mesh_ok, src/mesh.cpp:436-445) on the
//    device copy of the image, with the face offsets and the facts kgb_mesh_info reports (bounds, tri_cap, ...);
//  - kgb_triangulate / triangulate_view: a mesh's faces as triangles, the reference's triangulate_into
//    (src/mesh.cpp:137-168): vertices recentred to float, a triangle as given, a quad as 0-1-2 / 0-2-3, five or more
//    corners by ear clipping on the face's Newell plane (include/kgb_earcut.h, earcut's published algorithm),
//    triangles in face order;
//  - kgb_thin_solids / thin_solids_view: per slot, whether its faces form a closed thin solid (the reference's
//    thin_solid, src/mesh.cpp:275-304): welded corners (0.01 mm grid), every directed edge matched by its reverse,
//    twice the volume over the area under 0.1 m; the inward and volume-less (twin) variants.
// One thread per face for the triangulation (an n-gon's ear clipping runs on its own thread over scratch sized 2n + 16);
// scans, sorts and searches by thrust on the engine's stream. Every function takes a MeshView: the arrays of a mesh the
// engine keeps, or a caller's host arrays uploaded for the call (triangulate_mesh, thin_solids).
#include "engine.h"
#include "kgb_earcut.h"

#include <thrust/binary_search.h>
#include <thrust/device_ptr.h>
#include <thrust/execution_policy.h>
#include <thrust/functional.h>
#include <thrust/iterator/transform_iterator.h>
#include <thrust/reduce.h>
#include <thrust/scan.h>
#include <thrust/sort.h>
#include <thrust/transform_reduce.h>
#include <thrust/transform_scan.h>
#include <thrust/unique.h>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

namespace kgb {
namespace {

struct D3 { double x, y, z; };
__device__ __forceinline__ D3 d3sub(D3 a, D3 b) { return D3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ D3 d3cross(D3 a, D3 b) { return D3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
__device__ __forceinline__ double d3dot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ D3 d3unit(D3 a) {   // mesh.cpp's unit: a * (1 / |a|), or 0
  const double l = sqrt(d3dot(a, a));
  if (!(l > 0)) return D3{0, 0, 0};
  const double s = 1 / l;
  return D3{a.x * s, a.y * s, a.z * s};
}
__device__ __forceinline__ D3 point(const double* p, int i) { return D3{p[3 * size_t(i)], p[3 * size_t(i) + 1], p[3 * size_t(i) + 2]}; }
// mesh.cpp's newell: |N| = 2 area, direction by winding
__device__ __forceinline__ D3 newell(const double* pts, const int32_t* ix, int n) {
  D3 N{0, 0, 0};
  for (int i = 0; i < n; ++i) {
    const D3 a = point(pts, ix[i]), b = point(pts, ix[(i + 1) % n]);
    N.x += (a.y - b.y) * (a.z + b.z); N.y += (a.z - b.z) * (a.x + b.x); N.z += (a.x - b.x) * (a.y + b.y);
  }
  return N;
}
__device__ __forceinline__ uint32_t face_slot(const MeshView& m, uint64_t f) {
  return m.slot32 ? m.slot32[f] : m.slot16 ? uint32_t(m.slot16[f]) : 0u;
}

// per-face counts of the layout: triangles at most (tri_cap's term), ear-clipping scratch, the corners as u64
struct CapOf { __host__ __device__ uint64_t operator()(int32_t n) const { return n >= 3 ? uint64_t(n - 2) : 0ull; } };
struct ScrOf { __host__ __device__ uint64_t operator()(int32_t n) const { return n >= 5 ? 2 * uint64_t(n) + 16 : 0ull; } };
struct AsU64 { __host__ __device__ uint64_t operator()(int32_t n) const { return uint64_t(int64_t(n)); } };

struct DevBuf {   // a call's device buffer
  void* p = nullptr;
  ~DevBuf() { if (p) cudaFree(p); }
  template <class T> T* as() const { return static_cast<T*>(p); }
};
bool dev(DevBuf& u, size_t bytes, std::string& err) {
  if (cudaMalloc(&u.p, std::max<size_t>(bytes, 16)) != cudaSuccess) { cudaGetLastError(); err = "device memory"; return false; }
  return true;
}

// ---------------------------------------------------------------------------------------------------- image checks
// A double's bits mapped to an unsigned key in the order of the values (negatives flipped), for atomic min / max.
__device__ __forceinline__ unsigned long long order_key(double d) {
  const unsigned long long u = static_cast<unsigned long long>(__double_as_longlong(d));
  return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}
double from_key(unsigned long long k) {
  const unsigned long long u = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
  double d;
  std::memcpy(&d, &u, 8);
  return d;
}
struct CheckOut {
  unsigned long long sum;        // the counts' sum (faces of 3 or more corners only)
  unsigned long long lo[3], hi[3];   // order keys of the bounds
  uint32_t shortFace;            // a face with fewer than 3 corners
  uint32_t badIndex;             // an index outside the points
  uint32_t maxCount, maxSlot;
};

__global__ void k_check_faces(const int32_t* counts, uint64_t nF, const uint16_t* slot16, CheckOut* o) {
  unsigned long long sum = 0;
  uint32_t shortFace = 0, maxCount = 0, maxSlot = 0;
  for (uint64_t f = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; f < nF; f += uint64_t(gridDim.x) * blockDim.x) {
    const int32_t c = counts[f];
    if (c < 3) shortFace = 1;
    else { sum += uint64_t(c); maxCount = max(maxCount, uint32_t(c)); }
    if (slot16) maxSlot = max(maxSlot, uint32_t(slot16[f]));
  }
  for (int s = 16; s; s >>= 1) {
    sum += __shfl_xor_sync(0xffffffffu, sum, s);
    shortFace |= __shfl_xor_sync(0xffffffffu, shortFace, s);
    maxCount = max(maxCount, __shfl_xor_sync(0xffffffffu, maxCount, s));
    maxSlot = max(maxSlot, __shfl_xor_sync(0xffffffffu, maxSlot, s));
  }
  if ((threadIdx.x & 31) == 0) {
    if (sum) atomicAdd(&o->sum, sum);
    if (shortFace) atomicOr(&o->shortFace, 1u);
    if (maxCount) atomicMax(&o->maxCount, maxCount);
    if (maxSlot) atomicMax(&o->maxSlot, maxSlot);
  }
}
__global__ void k_check_indices(const int32_t* idx, uint64_t nI, uint64_t nP, CheckOut* o) {
  uint32_t bad = 0;
  for (uint64_t k = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; k < nI; k += uint64_t(gridDim.x) * blockDim.x) {
    const int32_t i = idx[k];
    if (i < 0 || uint64_t(i) >= nP) bad = 1;
  }
  if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(&o->badIndex, 1u);
}
// fmin / fmax per axis over the coordinates (a NaN coordinate is passed over, as fmin and fmax pass it over)
__global__ void k_bounds(const double* pts, uint64_t nP, CheckOut* o) {
  unsigned long long lo[3] = {~0ull, ~0ull, ~0ull}, hi[3] = {0ull, 0ull, 0ull};
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < nP; i += uint64_t(gridDim.x) * blockDim.x)
    for (int a = 0; a < 3; ++a) {
      const double d = pts[3 * i + a];
      if (d != d) continue;
      const unsigned long long k = order_key(d);
      lo[a] = min(lo[a], k);
      hi[a] = max(hi[a], k);
    }
  for (int a = 0; a < 3; ++a) {
    for (int s = 16; s; s >>= 1) {
      lo[a] = min(lo[a], __shfl_xor_sync(0xffffffffu, lo[a], s));
      hi[a] = max(hi[a], __shfl_xor_sync(0xffffffffu, hi[a], s));
    }
    if ((threadIdx.x & 31) == 0) {
      if (lo[a] != ~0ull) atomicMin(&o->lo[a], lo[a]);
      if (hi[a]) atomicMax(&o->hi[a], hi[a]);
    }
  }
}

// ---------------------------------------------------------------------------------------------------- triangulation
__global__ void k_recentre(const double* pts, uint32_t n, double cx, double cy, double cz, float* v) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  v[3 * size_t(i)] = __double2float_rn(pts[3 * size_t(i)] - cx);
  v[3 * size_t(i) + 1] = __double2float_rn(pts[3 * size_t(i) + 1] - cy);
  v[3 * size_t(i) + 2] = __double2float_rn(pts[3 * size_t(i) + 2] - cz);
}

struct FaceArgs {
  MeshView m;
  const uint64_t* capOff;    // [nFaces] the face's first triangle at most-triangles spacing (n - 2 each)
  const uint64_t* scrOff;    // [nFaces] its ear-clipping scratch (n-gons: 2 n + 16 nodes, stack words, xy pairs)
  kgb_earcut::Node* pool;
  int32_t* stack;
  double* xy;
  uint32_t* triTmp;          // [cap x 3]: each face's triangles at capOff (mesh indices)
  uint32_t* made;            // [nFaces]: triangles each face gave
  uint32_t* skipped;         // [nFaces]: 1 where the face gave none (fewer than 3 corners, no area, ear clipping failed)
};

__global__ void k_faces(FaceArgs a) {
  const uint64_t f = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (f >= a.m.nFaces) return;
  const int n = a.m.counts[f];
  const int32_t* ix = a.m.idx + a.m.idxOff[f];
  uint32_t* out = a.triTmp + 3 * a.capOff[f];
  uint32_t made = 0, skip = 0;
  if (n == 3) { out[0] = uint32_t(ix[0]); out[1] = uint32_t(ix[1]); out[2] = uint32_t(ix[2]); made = 1; }
  else if (n == 4) {
    out[0] = uint32_t(ix[0]); out[1] = uint32_t(ix[1]); out[2] = uint32_t(ix[2]);
    out[3] = uint32_t(ix[0]); out[4] = uint32_t(ix[2]); out[5] = uint32_t(ix[3]);
    made = 2;
  } else if (n >= 5) {
    D3 N = newell(a.m.pts, ix, n);
    if (sqrt(d3dot(N, N)) == 0) skip = 1;
    else {
      N = d3unit(N);
      const D3 ax = fabs(N.x) <= fabs(N.y) && fabs(N.x) <= fabs(N.z) ? D3{1, 0, 0} : fabs(N.y) <= fabs(N.z) ? D3{0, 1, 0} : D3{0, 0, 1};
      const D3 u = d3unit(d3cross(N, ax)), v = d3cross(N, u);   // (u, v, N) right-handed
      const uint64_t s = a.scrOff[f];
      double* xy = a.xy + 2 * s;
      for (int k = 0; k < n; ++k) { const D3 p = point(a.m.pts, ix[k]); xy[2 * k] = d3dot(p, u); xy[2 * k + 1] = d3dot(p, v); }
      const int t = kgb_earcut::earcut_ring(xy, n, a.pool + s, 2 * n + 16, a.stack + s, 2 * n + 16, out, n - 2);
      if (t <= 0) skip = 1;
      else {
        for (int k = 0; k < 3 * t; ++k) out[k] = uint32_t(ix[out[k]]);   // ring indices to the mesh's
        made = uint32_t(t);
      }
    }
  } else skip = 1;
  a.made[f] = made;
  a.skipped[f] = skip;
}

// each face's triangles from its capacity slot to its place in face order; indices offset by base, slots set
__global__ void k_compact(const uint32_t* triTmp, const uint64_t* capOff, const uint32_t* made, const uint64_t* outOff, MeshView m, uint32_t base,
                          uint32_t slotBase, uint32_t* tri, uint32_t* slot) {
  const uint64_t f = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (f >= m.nFaces) return;
  const uint32_t n = made[f];
  const uint32_t s = slotBase + face_slot(m, f);
  for (uint32_t k = 0; k < n; ++k) {
    for (int c = 0; c < 3; ++c) tri[3 * (outOff[f] + k) + c] = base + triTmp[3 * (capOff[f] + k) + c];
    if (slot) slot[outOff[f] + k] = s;
  }
}

__global__ void k_translucent(const uint32_t* slot, size_t nt, const kgb_slot* slots, uint8_t* out) {
  const size_t k = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k < nt) out[k] = slots[slot[k]].tau > 0 ? 1 : 0;
}

// ---------------------------------------------------------------------------------------------------- thin solids
struct Corner { int64_t x, y, z; uint32_t slot; uint32_t pad; };   // a welded corner of a slot's face
struct CornerLess {
  __host__ __device__ bool operator()(const Corner& a, const Corner& b) const {
    if (a.slot != b.slot) return a.slot < b.slot;
    if (a.x != b.x) return a.x < b.x;
    if (a.y != b.y) return a.y < b.y;
    return a.z < b.z;
  }
};
struct CornerEq {
  __host__ __device__ bool operator()(const Corner& a, const Corner& b) const { return a.slot == b.slot && a.x == b.x && a.y == b.y && a.z == b.z; }
};
struct Edge { uint32_t slot, a, b, pad; };
struct EdgeLess {
  __host__ __device__ bool operator()(const Edge& p, const Edge& q) const {
    if (p.slot != q.slot) return p.slot < q.slot;
    if (p.a != q.a) return p.a < q.a;
    return p.b < q.b;
  }
};

// every corner of every face: its weld key (llround of the recentred coordinate x 1e5) and its face's slot
__global__ void k_corners(MeshView m, double cx, double cy, double cz, Corner* out) {
  const uint64_t f = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (f >= m.nFaces) return;
  const int n = m.counts[f];
  const uint64_t o = m.idxOff[f];
  const uint32_t s = face_slot(m, f);
  for (int j = 0; j < n; ++j) {
    const D3 p = d3sub(point(m.pts, m.idx[o + j]), D3{cx, cy, cz});
    out[o + j] = Corner{llround(p.x * 1e5), llround(p.y * 1e5), llround(p.z * 1e5), s, 0u};
  }
}
// per face: the Newell area and the volume term (N . (p0 - c) / 6), summed per slot later in face order
__global__ void k_face_terms(MeshView m, double cx, double cy, double cz, double* area, double* vol) {
  const uint64_t f = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (f >= m.nFaces) return;
  const int n = m.counts[f];
  const int32_t* ix = m.idx + m.idxOff[f];
  const D3 N = newell(m.pts, ix, n);
  area[f] = sqrt(d3dot(N, N)) / 2;
  vol[f] = d3dot(N, d3sub(point(m.pts, ix[0]), D3{cx, cy, cz})) / 6;
}
// per slot, one thread: area and volume summed over its faces in face order (the reference's sequential sums), and its
// face count
__global__ void k_slot_sums(MeshView m, const double* area, const double* vol, uint32_t nSlots, double* sArea, double* sVol, uint32_t* sFaces) {
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nSlots) return;
  double A = 0, Vv = 0;
  uint32_t faces = 0;
  for (uint64_t f = 0; f < m.nFaces; ++f)
    if (face_slot(m, f) == s) { A += area[f]; Vv += vol[f]; ++faces; }
  sArea[s] = A;
  sVol[s] = Vv;
  sFaces[s] = faces;
}
// directed edges between welded corners, forward and reversed; an edge whose ends weld together is none
__global__ void k_edges(MeshView m, const uint32_t* ids, Edge* fwd, Edge* rev, uint32_t none) {
  const uint64_t f = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (f >= m.nFaces) return;
  const int n = m.counts[f];
  const uint64_t o = m.idxOff[f];
  const uint32_t s = face_slot(m, f);
  for (int j = 0; j < n; ++j) {
    const uint32_t a = ids[o + j], b = ids[o + (j + 1) % n];
    fwd[o + j] = a != b ? Edge{s, a, b, 0u} : Edge{none, 0u, 0u, 0u};
    rev[o + j] = a != b ? Edge{s, b, a, 0u} : Edge{none, 0u, 0u, 0u};
  }
}
// a slot is open when any of its sorted forward edges differs from the sorted reversed edge at the same place (the
// two lists hold the same number of edges per slot, so their slot ranges line up)
__global__ void k_edge_diff(const Edge* fwd, const Edge* rev, uint64_t n, uint32_t* open) {
  const uint64_t k = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const Edge p = fwd[k], q = rev[k];
  if (p.slot != q.slot || p.a != q.a || p.b != q.b) {
    if (p.slot < 0xffffffffu) atomicOr(open + p.slot, 1u);
    if (q.slot < 0xffffffffu) atomicOr(open + q.slot, 1u);
  }
}

uint32_t blocks_for(uint64_t n, uint32_t per) { return uint32_t((n + per - 1) / per); }

// A caller's host arrays on the device for one call: points, counts, indices, 32-bit slots and the face offsets
// (computed here on the host, where the caller's arrays are checked).
struct HostUpload {
  DevBuf pts, counts, idx, off, slot;
  MeshView view{};
};
std::string upload_host_mesh(const double* points, size_t nPoints, const int32_t* counts, size_t nFaces, const int32_t* indices, const uint32_t* faceSlot,
                             uint32_t nSlots, HostUpload& u, cudaStream_t st) {
  std::vector<uint64_t> idxOff(nFaces);
  uint64_t nIdx = 0;
  for (size_t f = 0; f < nFaces; ++f) {
    if (counts[f] < 0) return "a face with a negative corner count";
    if (faceSlot && nSlots && faceSlot[f] >= nSlots) return "a face's slot is not below nSlots";
    idxOff[f] = nIdx;
    nIdx += uint64_t(counts[f]);
  }
  for (uint64_t k = 0; k < nIdx; ++k)
    if (indices[k] < 0 || uint64_t(indices[k]) >= nPoints) return "a face's corner index exceeds the points";
  if (nPoints > 0xffffffffull || nFaces > 0xffffffffull || nIdx >= 0xffffffffull) return "more than 2^32 - 1 points, faces or face corners";
  std::string err;
  if (!dev(u.pts, nPoints * 24, err) || !dev(u.counts, nFaces * 4, err) || !dev(u.idx, nIdx * 4, err) || !dev(u.off, nFaces * 8, err) ||
      !dev(u.slot, faceSlot ? nFaces * 4 : 0, err))
    return err;
  if ((nPoints && cudaMemcpyAsync(u.pts.p, points, nPoints * 24, cudaMemcpyHostToDevice, st) != cudaSuccess) ||
      (nFaces && cudaMemcpyAsync(u.counts.p, counts, nFaces * 4, cudaMemcpyHostToDevice, st) != cudaSuccess) ||
      (nIdx && cudaMemcpyAsync(u.idx.p, indices, nIdx * 4, cudaMemcpyHostToDevice, st) != cudaSuccess) ||
      (nFaces && cudaMemcpyAsync(u.off.p, idxOff.data(), nFaces * 8, cudaMemcpyHostToDevice, st) != cudaSuccess) ||
      (faceSlot && nFaces && cudaMemcpyAsync(u.slot.p, faceSlot, nFaces * 4, cudaMemcpyHostToDevice, st) != cudaSuccess))
    return "the upload failed";
  // the copies read pageable host memory: complete them before the caller's arrays may change
  if (cudaStreamSynchronize(st) != cudaSuccess) return "the upload failed";
  u.view = MeshView{u.pts.as<double>(), u.counts.as<int32_t>(), u.idx.as<int32_t>(), u.off.as<uint64_t>(), nullptr,
                    faceSlot ? u.slot.as<uint32_t>() : nullptr, nPoints, nFaces, nIdx};
  return "";
}

}  // namespace

// The checks of parse_dmesh / mesh_ok on the device copy of an image, in the reference's order: a face with fewer than
// 3 corners, then the counts' sum against nIndices, then an index outside the points. Then the face offsets (an
// exclusive scan of the counts), the bounds, tri_cap and the largest face and slot.
std::string mesh_check(DevMesh& m, cudaStream_t st) {
  MeshView& v = m.view;
  DevBuf out;
  std::string err;
  if (!dev(out, sizeof(CheckOut), err)) return err;
  CheckOut init{};
  for (int a = 0; a < 3; ++a) { init.lo[a] = ~0ull; init.hi[a] = 0ull; }
  if (cudaMemcpyAsync(out.p, &init, sizeof init, cudaMemcpyHostToDevice, st) != cudaSuccess) return "the check failed";
  const uint32_t grid = 4 * 152;
  if (v.nFaces) k_check_faces<<<std::min(grid, blocks_for(v.nFaces, 256)), 256, 0, st>>>(v.counts, v.nFaces, v.slot16, out.as<CheckOut>());
  if (v.nIdx) k_check_indices<<<std::min(grid, blocks_for(v.nIdx, 256)), 256, 0, st>>>(v.idx, v.nIdx, v.nPoints, out.as<CheckOut>());
  if (v.nPoints) k_bounds<<<std::min(grid, blocks_for(v.nPoints, 256)), 256, 0, st>>>(v.pts, v.nPoints, out.as<CheckOut>());
  if (cudaGetLastError() != cudaSuccess) return "a kernel launch failed";
  CheckOut r{};
  if (cudaMemcpyAsync(&r, out.p, sizeof r, cudaMemcpyDeviceToHost, st) != cudaSuccess || cudaStreamSynchronize(st) != cudaSuccess)
    return "the check failed on the device";
  if (r.shortFace) return "face with fewer than 3 vertices";
  if (r.sum != v.nIdx) return "sum(counts) != n_indices";
  if (r.badIndex) return "vertex index out of range";
  kgb_mesh_info& in = m.info;
  in.nPoints = v.nPoints; in.nFaces = v.nFaces; in.nIndices = v.nIdx;
  in.hasSlots = v.slot16 ? 1u : 0u;
  in.slots = v.slot16 ? r.maxSlot + 1 : 1u;
  in.maxCorners = r.maxCount;
  in.triCap = r.sum - 2 * v.nFaces;   // every face has 3 or more corners here
  for (int a = 0; a < 3; ++a) {
    in.lo[a] = r.lo[a] == ~0ull ? INFINITY : from_key(r.lo[a]);
    in.hi[a] = r.hi[a] == 0ull ? -INFINITY : from_key(r.hi[a]);
  }
  if (v.nFaces) {
    thrust::device_ptr<const int32_t> c(v.counts);
    thrust::device_ptr<uint64_t> o(const_cast<uint64_t*>(v.idxOff));
    thrust::exclusive_scan(thrust::cuda::par.on(st), thrust::make_transform_iterator(c, AsU64()), thrust::make_transform_iterator(c + v.nFaces, AsU64()),
                           o, uint64_t(0), thrust::plus<uint64_t>());
  }
  if (cudaGetLastError() != cudaSuccess) return "the face offsets failed";
  return "";
}

std::string triangulate_view(const MeshView& m, const double* c, uint32_t base, uint32_t slotBase, float* v, uint32_t* tri, uint32_t* slot,
                             uint64_t* madeOut, int32_t* skippedOut, cudaStream_t st) {
  *madeOut = 0;
  *skippedOut = 0;
  if (m.nPoints) k_recentre<<<blocks_for(m.nPoints, 256), 256, 0, st>>>(m.pts, uint32_t(m.nPoints), c[0], c[1], c[2], v);
  if (!m.nFaces) return cudaGetLastError() == cudaSuccess ? "" : "a kernel launch failed";
  const auto pol = thrust::cuda::par.on(st);
  thrust::device_ptr<const int32_t> cnt(m.counts);
  const uint64_t cap = thrust::transform_reduce(pol, cnt, cnt + m.nFaces, CapOf(), uint64_t(0), thrust::plus<uint64_t>());
  const uint64_t scr = thrust::transform_reduce(pol, cnt, cnt + m.nFaces, ScrOf(), uint64_t(0), thrust::plus<uint64_t>());
  if (cap > 0xffffffffull) return "more than 2^32 - 1 triangles";
  DevBuf dOff, dScrN, dScrS, dScrXY, dTmp, dMade, dSkip;
  std::string err;
  if (!dev(dOff, m.nFaces * 8 * 3, err) || !dev(dScrN, scr * sizeof(kgb_earcut::Node), err) || !dev(dScrS, scr * 4, err) || !dev(dScrXY, scr * 16, err) ||
      !dev(dTmp, cap * 12, err) || !dev(dMade, m.nFaces * 4, err) || !dev(dSkip, m.nFaces * 4, err))
    return err;
  uint64_t* off = dOff.as<uint64_t>();   // capOff | scrOff | outOff
  thrust::device_ptr<uint64_t> capOff(off), scrOff(off + m.nFaces), outOff(off + 2 * m.nFaces);
  thrust::transform_exclusive_scan(pol, cnt, cnt + m.nFaces, capOff, CapOf(), uint64_t(0), thrust::plus<uint64_t>());
  thrust::transform_exclusive_scan(pol, cnt, cnt + m.nFaces, scrOff, ScrOf(), uint64_t(0), thrust::plus<uint64_t>());
  FaceArgs a{};
  a.m = m;
  a.capOff = off; a.scrOff = off + m.nFaces;
  a.pool = dScrN.as<kgb_earcut::Node>(); a.stack = dScrS.as<int32_t>(); a.xy = dScrXY.as<double>();
  a.triTmp = dTmp.as<uint32_t>(); a.made = dMade.as<uint32_t>(); a.skipped = dSkip.as<uint32_t>();
  k_faces<<<blocks_for(m.nFaces, 128), 128, 0, st>>>(a);
  // the triangles' places in face order
  thrust::device_ptr<uint32_t> made(dMade.as<uint32_t>()), skip(dSkip.as<uint32_t>());
  thrust::exclusive_scan(pol, made, made + m.nFaces, outOff, uint64_t(0), thrust::plus<uint64_t>());
  k_compact<<<blocks_for(m.nFaces, 128), 128, 0, st>>>(dTmp.as<uint32_t>(), off, dMade.as<uint32_t>(), off + 2 * m.nFaces, m, base, slotBase, tri, slot);
  if (cudaGetLastError() != cudaSuccess) return "a kernel launch failed";
  const uint64_t total = thrust::reduce(pol, made, made + m.nFaces, uint64_t(0), thrust::plus<uint64_t>());
  const uint64_t skipped = thrust::reduce(pol, skip, skip + m.nFaces, uint64_t(0), thrust::plus<uint64_t>());
  if (cudaStreamSynchronize(st) != cudaSuccess) return "the triangulation failed on the device";
  *madeOut = total;
  *skippedOut = int32_t(skipped);
  return "";
}

void launch_translucent(const uint32_t* slot, size_t nt, const kgb_slot* slots, uint8_t* translucent, cudaStream_t st) {
  if (nt) k_translucent<<<uint32_t((nt + 255) / 256), 256, 0, st>>>(slot, nt, slots, translucent);
}

// Host side of kgb_triangulate: the caller's arrays checked and uploaded, the faces on the device, the results back.
std::string triangulate_mesh(const double* points, size_t nPoints, const int32_t* counts, size_t nFaces, const int32_t* indices, const uint32_t* faceSlot,
                             const double* c, uint32_t base, uint32_t slotBase, float* vOut, uint32_t* triOut, uint32_t* slotOut, size_t* madeOut,
                             int32_t* skippedOut, cudaStream_t st) {
  HostUpload u;
  std::string err = upload_host_mesh(points, nPoints, counts, nFaces, indices, faceSlot, 0, u, st);
  if (!err.empty()) return err;
  uint64_t cap = 0;
  for (size_t f = 0; f < nFaces; ++f) cap += counts[f] >= 3 ? uint64_t(counts[f] - 2) : 0;
  if (cap > 0xffffffffull) return "more than 2^32 - 1 triangles";
  DevBuf dV, dTri, dTriSlot;
  if (!dev(dV, nPoints * 12, err) || !dev(dTri, cap * 12, err) || !dev(dTriSlot, cap * 4, err)) return err;
  uint64_t total = 0;
  int32_t skipped = 0;
  err = triangulate_view(u.view, c, base, slotBase, dV.as<float>(), dTri.as<uint32_t>(), slotOut ? dTriSlot.as<uint32_t>() : nullptr, &total, &skipped, st);
  if (!err.empty()) return err;
  if (nPoints) cudaMemcpyAsync(vOut, dV.p, nPoints * 12, cudaMemcpyDeviceToHost, st);
  if (total) {
    cudaMemcpyAsync(triOut, dTri.p, total * 12, cudaMemcpyDeviceToHost, st);
    if (slotOut) cudaMemcpyAsync(slotOut, dTriSlot.p, total * 4, cudaMemcpyDeviceToHost, st);
  }
  if (cudaStreamSynchronize(st) != cudaSuccess) return "the download failed";
  *madeOut = size_t(total);
  *skippedOut = skipped;
  return "";
}

std::string thin_solids_view(const MeshView& m, uint32_t nSlots, const double* c, uint32_t* flags, cudaStream_t st) {
  for (uint32_t s = 0; s < nSlots; ++s) flags[s] = 0;
  if (!m.nFaces || !nSlots) return "";
  const uint64_t nIdx = m.nIdx;
  if (nIdx >= 0xffffffffull) return "more than 2^32 - 1 face corners";
  DevBuf dCorner, dSorted, dIds, dFwd, dRev, dArea, dVol, dSArea, dSVol, dSFaces, dOpen;
  std::string err;
  if (!dev(dCorner, nIdx * sizeof(Corner), err) || !dev(dSorted, nIdx * sizeof(Corner), err) || !dev(dIds, nIdx * 4, err) ||
      !dev(dFwd, nIdx * sizeof(Edge), err) || !dev(dRev, nIdx * sizeof(Edge), err) || !dev(dArea, m.nFaces * 8, err) || !dev(dVol, m.nFaces * 8, err) ||
      !dev(dSArea, nSlots * 8, err) || !dev(dSVol, nSlots * 8, err) || !dev(dSFaces, nSlots * 4, err) || !dev(dOpen, nSlots * 4, err))
    return err;
  cudaMemsetAsync(dOpen.p, 0, nSlots * 4, st);
  const uint32_t fb = blocks_for(m.nFaces, 128);
  k_corners<<<fb, 128, 0, st>>>(m, c[0], c[1], c[2], dCorner.as<Corner>());
  k_face_terms<<<fb, 128, 0, st>>>(m, c[0], c[1], c[2], dArea.as<double>(), dVol.as<double>());
  k_slot_sums<<<(nSlots + 127) / 128, 128, 0, st>>>(m, dArea.as<double>(), dVol.as<double>(), nSlots, dSArea.as<double>(), dSVol.as<double>(),
                                                    dSFaces.as<uint32_t>());
  // the welded points: the corners sorted and made unique; each corner's id its place among them (lower bound)
  const auto pol = thrust::cuda::par.on(st);
  thrust::device_ptr<Corner> corner(dCorner.as<Corner>()), sorted(dSorted.as<Corner>());
  cudaMemcpyAsync(dSorted.p, dCorner.p, nIdx * sizeof(Corner), cudaMemcpyDeviceToDevice, st);
  thrust::sort(pol, sorted, sorted + nIdx, CornerLess());
  const auto uEnd = thrust::unique(pol, sorted, sorted + nIdx, CornerEq());
  thrust::device_ptr<uint32_t> ids(dIds.as<uint32_t>());
  thrust::lower_bound(pol, sorted, uEnd, corner, corner + nIdx, ids, CornerLess());
  // the directed edges, forward and reversed, each list sorted; a slot whose two lists differ is open
  Edge* fwd = dFwd.as<Edge>();
  Edge* rev = dRev.as<Edge>();
  k_edges<<<fb, 128, 0, st>>>(m, dIds.as<uint32_t>(), fwd, rev, 0xffffffffu);
  thrust::sort(pol, thrust::device_ptr<Edge>(fwd), thrust::device_ptr<Edge>(fwd) + nIdx, EdgeLess());
  thrust::sort(pol, thrust::device_ptr<Edge>(rev), thrust::device_ptr<Edge>(rev) + nIdx, EdgeLess());
  k_edge_diff<<<blocks_for(nIdx, 256), 256, 0, st>>>(fwd, rev, nIdx, dOpen.as<uint32_t>());
  if (cudaGetLastError() != cudaSuccess) return "a kernel launch failed";
  std::vector<double> A(nSlots), Vv(nSlots);
  std::vector<uint32_t> open(nSlots), faces(nSlots);
  cudaMemcpyAsync(A.data(), dSArea.p, nSlots * 8, cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(Vv.data(), dSVol.p, nSlots * 8, cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(open.data(), dOpen.p, nSlots * 4, cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(faces.data(), dSFaces.p, nSlots * 4, cudaMemcpyDeviceToHost, st);
  if (cudaStreamSynchronize(st) != cudaSuccess) return "the thin-solid test failed on the device";
  for (uint32_t s = 0; s < nSlots; ++s) {   // mesh.cpp:291-303's verdict
    if (!faces[s] || !(A[s] > 0) || 2 * std::fabs(Vv[s]) / A[s] >= 0.1 || open[s]) continue;
    flags[s] = KGB_SLOT_THIN | (2 * std::fabs(Vv[s]) / A[s] < 1e-5 ? KGB_SLOT_TWIN : Vv[s] < 0 ? KGB_SLOT_INWARD : 0u);
  }
  return "";
}

// Host side of kgb_thin_solids: flags[s] for every slot s < nSlots.
std::string thin_solids(const double* points, size_t nPoints, const int32_t* counts, size_t nFaces, const int32_t* indices, const uint32_t* faceSlot,
                        uint32_t nSlots, const double* c, uint32_t* flags, cudaStream_t st) {
  for (uint32_t s = 0; s < nSlots; ++s) flags[s] = 0;
  for (size_t f = 0; f < nFaces; ++f)
    if (faceSlot && faceSlot[f] >= nSlots) return "a face's slot is not below nSlots";
  if (!nFaces || !nSlots) {
    for (size_t f = 0; f < nFaces; ++f) if (counts[f] < 0) return "a face with a negative corner count";
    return "";
  }
  HostUpload u;
  const std::string err = upload_host_mesh(points, nPoints, counts, nFaces, indices, faceSlot, nSlots, u, st);
  if (!err.empty()) return err;
  return thin_solids_view(u.view, nSlots, c, flags, st);
}

}  // namespace kgb
