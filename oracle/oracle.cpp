// TEST INFRASTRUCTURE ONLY - the oracle. Not part of the engine: nothing under kit-sim_daylight_gb300/ links, loads or
// calls it. Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it, as the checker.
//
// A CPU restatement of the reference's ray-cast-and-accumulate path (src/trace_dev.cu + src/gpu.cu of
// kit-sim_daylight), behind the same C ABI as the engine (include/kitsim_gb300.h), so that
//  - the reference's own host code and tests (run.cpp, views.cpp, tests/check_gpu.cpp, tests/check_views.cpp) run on
//    it through the engine's C++ shim (oracle/Makefile, target `ref`): that pins the restatement to the reference;
//  - the engine's CUDA results are compared with it bit for bit (visibility bits / bytes, classes, distances, bins,
//    reductions) or, for the FP32 / split-BF16 time series, against its FP64 contraction within a stated tolerance.
//
// Visibility is defined by one watertight ray/triangle test (Woop, Benthin, Wald 2013, JCGT 2(1)) in IEEE float with
// no contraction: a hit of triangle k at t exists iff that test says so. Acceleration structures only filter
// conservatively (boxes expanded by 2^-16 x the scene's largest coordinate, slab tests widened), so any of them gives
// the brute-force result; here a binned-SAH binary BVH. Every decision the reference takes on "the hit OptiX reports"
// is restated over the full, ordered hit set of the ray (order-independent); the places where that differs from the
// reference in degenerate cases are listed at each function.
//
// Compile with -ffp-contract=off (oracle/Makefile does).
#include "kitsim_gb300.h"
#include "kgb_detmath.h"

#include <unistd.h>
#include <cerrno>

#include <algorithm>
#include <cfloat>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <limits>
#include <memory>
#include <string>
#include <thread>
#include <vector>

namespace {

thread_local std::string g_err;
int fail(const std::string& m) { g_err = m; return 0; }

struct F3 { float x, y, z; };
inline F3 f3(float x, float y, float z) { return F3{x, y, z}; }
inline F3 add(F3 a, F3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline F3 sub(F3 a, F3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline F3 mul(float s, F3 a) { return f3(s * a.x, s * a.y, s * a.z); }
inline float dot(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float comp(F3 a, int k) { return k == 0 ? a.x : k == 1 ? a.y : a.z; }

inline float as_float(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }
inline uint32_t as_uint(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }
inline float next_up(float t) { return as_float(as_uint(t) + 1); }   // trace_dev.cu:85, 224: the next float past t (t > 0)

// trace_dev.cu:16-25 (offset_ray): the origin nudged along the normal by 256 int-ulps, or 2^-16 m near 0.
F3 offset_ray(F3 p, F3 n) {
  const float origin = 1.f / 32.f, floatScale = 1.f / 65536.f, intScale = 256.f;
  const int ox = int(intScale * n.x), oy = int(intScale * n.y), oz = int(intScale * n.z);
  const auto nudge = [](float v, int o) { return as_float(uint32_t(int32_t(as_uint(v)) + (v < 0.f ? -o : o))); };
  return f3(std::fabs(p.x) < origin ? p.x + floatScale * n.x : nudge(p.x, ox),
            std::fabs(p.y) < origin ? p.y + floatScale * n.y : nudge(p.y, oy),
            std::fabs(p.z) < origin ? p.z + floatScale * n.z : nudge(p.z, oz));
}

// params.h:64-71 (pcg3d, Jarzynski & Olano 2020) and u01.
struct U3 { uint32_t x, y, z; };
U3 pcg3d(uint32_t x, uint32_t y, uint32_t z) {
  x = x * 1664525u + 1013904223u; y = y * 1664525u + 1013904223u; z = z * 1664525u + 1013904223u;
  x += y * z; y += z * x; z += x * y;
  x ^= x >> 16; y ^= y >> 16; z ^= z >> 16;
  x += y * z; y += z * x; z += x * y;
  return U3{x, y, z};
}
inline float u01(uint32_t v) { return float(v >> 8) * (1.f / 16777216.f); }
inline uint32_t brev(uint32_t v) {
  uint32_t r = 0;
  for (int k = 0; k < 32; ++k) { r = (r << 1) | (v & 1u); v >>= 1; }
  return r;
}

// glass.h:17-25 (glass_TR, the Radiance m_glass.c pane), powf as kgb_powf.
void glass_TR(float c, float tn, float& T, float& R) {
  const float n = 1.52f;
  const float c2 = std::sqrt((1.f - 1.f / (n * n)) + c * c / (n * n));
  const float d = kgb_powf(tn, 1.f / c2), d2 = d * d;
  float rs = (c - n * c2) / (c + n * c2), rp = (c2 - n * c) / (c2 + n * c);
  rs *= rs; rp *= rp;
  T = .5f * (1.f - rs) * (1.f - rs) * d / (1.f - rs * rs * d2) + .5f * (1.f - rp) * (1.f - rp) * d / (1.f - rp * rp * d2);
  R = .5f * rs * (1.f + (1.f - 2.f * rs) * d2) / (1.f - rs * rs * d2) + .5f * rp * (1.f + (1.f - 2.f * rp) * d2) / (1.f - rp * rp * d2);
}

// ---------------------------------------------------------------------------------------------------- the hit test
// Woop, Benthin, Wald 2013: the ray's dominant axis kz, shear constants; per triangle the 2D edge functions U V W of the
// sheared vertices (double recomputation when one is exactly 0: watertight), hit when all share a sign, t = T / det.
// front: det > 0 <=> the ray meets the side (v1-v0) x (v2-v0) points to (dot(d, ng) < 0): OptiX's front face.
struct Ray {
  F3 o, d;
  int kx, ky, kz;
  float Sx, Sy, Sz;
};
Ray make_ray(F3 o, F3 d) {
  Ray r;
  r.o = o; r.d = d;
  const float ax = std::fabs(d.x), ay = std::fabs(d.y), az = std::fabs(d.z);
  r.kz = ax >= ay ? (ax >= az ? 0 : 2) : (ay >= az ? 1 : 2);
  r.kx = r.kz == 2 ? 0 : r.kz + 1;
  r.ky = r.kx == 2 ? 0 : r.kx + 1;
  if (comp(d, r.kz) < 0.f) std::swap(r.kx, r.ky);
  const float dz = comp(d, r.kz);
  r.Sx = comp(d, r.kx) / dz;
  r.Sy = comp(d, r.ky) / dz;
  r.Sz = 1.f / dz;
  return r;
}
struct Hit { float t = 0, u = 0, v = 0; uint32_t prim = 0; bool front = false; };
// true with h (t, barycentrics of v1 / v2, front) when the triangle is hit at t in [tmin, tmax]
bool hit_tri(const Ray& r, F3 v0, F3 v1, F3 v2, float tmin, float tmax, bool cullBack, Hit& h) {
  const F3 A = sub(v0, r.o), B = sub(v1, r.o), C = sub(v2, r.o);
  const float Ax = comp(A, r.kx) - r.Sx * comp(A, r.kz), Ay = comp(A, r.ky) - r.Sy * comp(A, r.kz);
  const float Bx = comp(B, r.kx) - r.Sx * comp(B, r.kz), By = comp(B, r.ky) - r.Sy * comp(B, r.kz);
  const float Cx = comp(C, r.kx) - r.Sx * comp(C, r.kz), Cy = comp(C, r.ky) - r.Sy * comp(C, r.kz);
  float U = Cx * By - Cy * Bx, V = Ax * Cy - Ay * Cx, W = Bx * Ay - By * Ax;
  if (U == 0.f || V == 0.f || W == 0.f) {
    U = float(double(Cx) * double(By) - double(Cy) * double(Bx));
    V = float(double(Ax) * double(Cy) - double(Ay) * double(Cx));
    W = float(double(Bx) * double(Ay) - double(By) * double(Ax));
  }
  if ((U < 0.f || V < 0.f || W < 0.f) && (U > 0.f || V > 0.f || W > 0.f)) return false;
  const float det = U + V + W;
  if (det == 0.f) return false;
  if (cullBack && det < 0.f) return false;
  if (U == 0.f || V == 0.f || W == 0.f) {   // the ray meets an edge's line: one of the two triangles sharing it takes it
    const float s = det > 0.f ? 1.f : -1.f;
    const auto owns = [](float ex, float ey) { return ey > 0.f || (ey == 0.f && ex > 0.f); };
    if (U == 0.f && !owns(s * (Cx - Bx), s * (Cy - By))) return false;
    if (V == 0.f && !owns(s * (Ax - Cx), s * (Ay - Cy))) return false;
    if (W == 0.f && !owns(s * (Bx - Ax), s * (By - Ay))) return false;
  }
  const float Az = r.Sz * comp(A, r.kz), Bz = r.Sz * comp(B, r.kz), Cz = r.Sz * comp(C, r.kz);
  const float T = U * Az + V * Bz + W * Cz;
  const float t = T / det;
  if (!(t >= tmin && t <= tmax)) return false;
  h.t = t; h.u = V / det; h.v = W / det; h.front = det > 0.f;
  return true;
}

// ---------------------------------------------------------------------------------------------------- scene + BVH
struct Node { float lo[3], hi[3]; uint32_t left, right, first, count; };   // count > 0: leaf of order[first..)
struct Scene {
  std::vector<F3> v;            // vertices
  std::vector<uint32_t> tri;    // 3 per triangle
  std::vector<uint32_t> slot;   // per triangle: its hit record (0 when the build is not slotted)
  std::vector<uint8_t> translucent;   // per triangle: its slot transmitted at build (any-hit)
  bool slotted = false;
  std::vector<Node> nodes;
  std::vector<uint32_t> order;
  uint64_t bytes = 0;
};

void build_bvh(Scene& s) {
  const size_t nt = s.tri.size() / 3;
  s.nodes.clear(); s.order.resize(nt);
  if (!nt) return;
  float M = 1.f;
  for (const F3& p : s.v) M = std::max({M, std::fabs(p.x), std::fabs(p.y), std::fabs(p.z)});
  const float eps = M * (1.f / 65536.f);
  std::vector<float> blo(3 * nt), bhi(3 * nt), cen(3 * nt);
  for (size_t k = 0; k < nt; ++k) {
    s.order[k] = uint32_t(k);
    const F3 a = s.v[s.tri[3 * k]], b = s.v[s.tri[3 * k + 1]], c = s.v[s.tri[3 * k + 2]];
    for (int ax = 0; ax < 3; ++ax) {
      const float lo = std::min({comp(a, ax), comp(b, ax), comp(c, ax)}), hi = std::max({comp(a, ax), comp(b, ax), comp(c, ax)});
      blo[3 * k + ax] = lo - eps; bhi[3 * k + ax] = hi + eps; cen[3 * k + ax] = 0.5f * (lo + hi);
    }
  }
  struct Item { uint32_t node, first, count; };
  std::vector<Item> stack;
  s.nodes.push_back(Node{});
  stack.push_back({0, 0, uint32_t(nt)});
  while (!stack.empty()) {
    const Item it = stack.back(); stack.pop_back();
    Node nd{};
    for (int ax = 0; ax < 3; ++ax) { nd.lo[ax] = INFINITY; nd.hi[ax] = -INFINITY; }
    float clo[3] = {INFINITY, INFINITY, INFINITY}, chi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint32_t j = it.first; j < it.first + it.count; ++j) {
      const uint32_t k = s.order[j];
      for (int ax = 0; ax < 3; ++ax) {
        nd.lo[ax] = std::min(nd.lo[ax], blo[3 * k + ax]); nd.hi[ax] = std::max(nd.hi[ax], bhi[3 * k + ax]);
        clo[ax] = std::min(clo[ax], cen[3 * k + ax]); chi[ax] = std::max(chi[ax], cen[3 * k + ax]);
      }
    }
    int axis = 0;
    for (int ax = 1; ax < 3; ++ax) if (chi[ax] - clo[ax] > chi[axis] - clo[axis]) axis = ax;
    uint32_t split = 0;
    if (it.count > 4 && chi[axis] > clo[axis]) {   // binned SAH over 16 bins of the centroids on the widest axis
      const int NB = 16;
      float cnt[NB] = {}, bl[NB][3], bh[NB][3];
      for (int b = 0; b < NB; ++b) for (int ax = 0; ax < 3; ++ax) { bl[b][ax] = INFINITY; bh[b][ax] = -INFINITY; }
      const float scale = NB / (chi[axis] - clo[axis]);
      auto bin = [&](uint32_t k) { return std::min(NB - 1, int((cen[3 * k + axis] - clo[axis]) * scale)); };
      for (uint32_t j = it.first; j < it.first + it.count; ++j) {
        const uint32_t k = s.order[j];
        const int b = bin(k);
        cnt[b] += 1;
        for (int ax = 0; ax < 3; ++ax) { bl[b][ax] = std::min(bl[b][ax], blo[3 * k + ax]); bh[b][ax] = std::max(bh[b][ax], bhi[3 * k + ax]); }
      }
      auto area = [](const float* lo, const float* hi) {
        const float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
        return dx < 0 ? 0.f : dx * dy + dy * dz + dz * dx;
      };
      float best = INFINITY; int bestB = -1;
      for (int b = 1; b < NB; ++b) {
        float l[3] = {INFINITY, INFINITY, INFINITY}, h[3] = {-INFINITY, -INFINITY, -INFINITY}, nl = 0, nr = 0;
        float l2[3] = {INFINITY, INFINITY, INFINITY}, h2[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (int q = 0; q < NB; ++q) {
          float* lo = q < b ? l : l2; float* hi = q < b ? h : h2;
          if (cnt[q] == 0) continue;
          (q < b ? nl : nr) += cnt[q];
          for (int ax = 0; ax < 3; ++ax) { lo[ax] = std::min(lo[ax], bl[q][ax]); hi[ax] = std::max(hi[ax], bh[q][ax]); }
        }
        if (nl == 0 || nr == 0) continue;
        const float c = nl * area(l, h) + nr * area(l2, h2);
        if (c < best) { best = c; bestB = b; }
      }
      if (bestB > 0) {
        auto mid = std::partition(s.order.begin() + it.first, s.order.begin() + it.first + it.count, [&](uint32_t k) { return bin(k) < bestB; });
        split = uint32_t(mid - s.order.begin()) - it.first;
      }
    }
    if (it.count > 4 && (split == 0 || split == it.count)) {   // no SAH split: median of the widest axis
      split = it.count / 2;
      std::nth_element(s.order.begin() + it.first, s.order.begin() + it.first + split, s.order.begin() + it.first + it.count,
                       [&](uint32_t a, uint32_t b) { return cen[3 * a + axis] < cen[3 * b + axis]; });
    }
    if (it.count <= 4) { nd.first = it.first; nd.count = it.count; s.nodes[it.node] = nd; continue; }
    nd.left = uint32_t(s.nodes.size()); nd.right = nd.left + 1; nd.count = 0;
    s.nodes[it.node] = nd;
    s.nodes.push_back(Node{}); s.nodes.push_back(Node{});
    stack.push_back({nd.left, it.first, split});
    stack.push_back({nd.right, it.first + split, it.count - split});
  }
}

// Conservative slab test: the interval is widened by 2^-20 relative so that float rounding never drops a box the
// exact ray meets; a zero direction component keeps the slab when the origin lies in it.
bool box_hit(const Node& nd, const Ray& r, float tmin, float tmax) {
  float tn = -INFINITY, tf = INFINITY;
  for (int ax = 0; ax < 3; ++ax) {
    const float o = comp(r.o, ax), d = comp(r.d, ax);
    if (d == 0.f) { if (o < nd.lo[ax] || o > nd.hi[ax]) return false; continue; }
    float t0 = (nd.lo[ax] - o) / d, t1 = (nd.hi[ax] - o) / d;
    if (t0 > t1) std::swap(t0, t1);
    tn = std::max(tn, t0); tf = std::min(tf, t1);
  }
  tn -= std::fabs(tn) * 9.5367431640625e-7f;
  tf += std::fabs(tf) * 9.5367431640625e-7f;
  return std::max(tn, tmin) <= std::min(tf, tmax);
}

// Every hit of the ray in [tmin, tmax] (culling as asked) to f(hit); f returns true to stop.
template <class Fn>
void for_hits(const Scene& s, const Ray& r, float tmin, float tmax, bool cull, Fn&& f) {
  if (s.nodes.empty()) return;
  uint32_t stack[128];
  int sp = 0;
  stack[sp++] = 0;
  while (sp) {
    const Node& nd = s.nodes[stack[--sp]];
    if (!box_hit(nd, r, tmin, tmax)) continue;
    if (nd.count) {
      for (uint32_t j = nd.first; j < nd.first + nd.count; ++j) {
        const uint32_t k = s.order[j];
        Hit h;
        if (hit_tri(r, s.v[s.tri[3 * k]], s.v[s.tri[3 * k + 1]], s.v[s.tri[3 * k + 2]], tmin, tmax, cull, h)) {
          h.prim = k;
          if (f(h)) return;
        }
      }
    } else {
      stack[sp++] = nd.left;
      stack[sp++] = nd.right;
    }
  }
}
// The closest hit in [tmin, tmax]: smallest t, then smallest primitive index (a fixed tie-break).
bool closest(const Scene& s, const Ray& r, float tmin, float tmax, bool cull, Hit& best) {
  bool any = false;
  for_hits(s, r, tmin, tmax, cull, [&](const Hit& h) {
    if (!any || h.t < best.t || (h.t == best.t && h.prim < best.prim)) { best = h; any = true; }
    return false;
  });
  return any;
}

// trace_dev.cu:37-52 (Hit / hit_triangle): the hit triangle's point, unit normal on the side the ray came from
// (1/sqrt instead of rsqrtf), largest edge coordinate ext and lift 2^-20 ext along n; false when degenerate.
struct TriHit { F3 p, n, lift; float ext; bool front; };
bool hit_triangle(const Scene& s, const Hit& hh, TriHit& h) {
  const F3 v0 = s.v[s.tri[3 * hh.prim]], v1 = s.v[s.tri[3 * hh.prim + 1]], v2 = s.v[s.tri[3 * hh.prim + 2]];
  const F3 e1 = sub(v1, v0), e2 = sub(v2, v0);
  const F3 ng = f3(e1.y * e2.z - e1.z * e2.y, e1.z * e2.x - e1.x * e2.z, e1.x * e2.y - e1.y * e2.x);
  const float l2 = dot(ng, ng);
  if (!(l2 > 0.f)) return false;
  const float inv = 1.f / std::sqrt(l2);
  h.front = hh.front;
  h.n = mul(h.front ? inv : -inv, ng);
  h.p = add(add(v0, mul(hh.u, e1)), mul(hh.v, e2));
  h.ext = std::max(std::max(std::max(std::fabs(e1.x), std::fabs(e1.y)), std::max(std::fabs(e1.z), std::fabs(e2.x))), std::max(std::fabs(e2.y), std::fabs(e2.z)));
  h.lift = mul(h.ext * 9.5367432e-7f, h.n);
  return true;
}
// trace_dev.cu:60-62 (own_plane)
bool own_plane(const TriHit& h, float t, F3 d, F3 n) { return t * std::fabs(dot(d, h.n)) < h.ext * 2.3841858e-7f && dot(n, h.n) <= 0.f; }
// trace_dev.cu:68-72 (own_hit)
bool own_hit(const Scene& s, const Hit& hh, F3 d, F3 n) {
  TriHit h;
  return hh.t * dot(n, d) < 1.f / 32.f && hit_triangle(s, hh, h) && own_plane(h, hh.t, d, n);
}
// trace_dev.cu:63 (through): the origin past the hit triangle
F3 through(const TriHit& h) { return sub(offset_ray(h.p, mul(-1.f, h.n)), h.lift); }

// ---------------------------------------------------------------------------------------------------- engine
struct Engine {
  Scene* sc = nullptr;
  std::vector<kgb_slot> slots{kgb_slot{0.2f, 0.f, 0.f, 0u}};
  std::vector<F3> P, N, D;
  size_t nSensors = 0, nDir = 0, nWords = 0;
  bool bytes = false; size_t i0 = 0;
  std::vector<uint32_t> bits; std::vector<uint8_t> byt;
  std::vector<float> dc; size_t nBins = 0, dcN = 0, dcI0 = 0;
  std::vector<uint8_t> cls; std::vector<float> dist; size_t viewN = 0, viewK = 0, viewI0 = 0;
  kgb_view_in view{}; std::vector<float> rowSin;
  std::vector<uint8_t> label;
  kgb_stats stats{};
  std::vector<std::unique_ptr<struct HostMesh>> meshes;   // kgb_mesh_read / kgb_mesh_file, by id
};

// ---------------------------------------------------------------------------------------------------- .dmesh
// The reference's .dmesh reader restated on the host (parse_dmesh, src/mesh.cpp:450-474, with mesh_ok at 436-445 and
// the file variant at 480-489): the header's checks in its order and words, the arrays copied out, then the array
// rules. The engine's kgb_mesh_* do the same with the arrays on the device; tests/golden/dmesh holds the reference's
// own answers on the same images.
struct HostMesh {
  std::vector<double> points;
  std::vector<int32_t> counts, indices;
  std::vector<uint16_t> slot;
  kgb_mesh_info info{};
};

int dmesh_parse(Engine& g, const char* data, size_t size, const std::string& label, kgb_mesh_info* info) {
  struct Header { char magic[4]; uint32_t flags; uint64_t nPoints, nFaces, nIndices; };
  static_assert(sizeof(Header) == 32, "the .dmesh header is 32 bytes");
  Header h{};
  if (size < sizeof h) return fail(label + ": truncated");
  std::memcpy(&h, data, sizeof h);
  if (std::memcmp(h.magic, "DLM1", 4)) return fail(label + ": not a .dmesh file (magic DLM1)");
  if (h.flags & ~1u) return fail(label + ": unsupported header flags " + std::to_string(h.flags) + " (only bit 0, the slot block, is defined)");
  if (!(h.nPoints <= size / 24 && h.nFaces <= size / 4 && h.nIndices <= size / 4 && 32 + 24 * h.nPoints + 4 * h.nFaces + 4 * h.nIndices <= size))
    return fail(label + ": truncated");
  const uint64_t nSlots = (h.flags & 1) ? h.nFaces : 0;
  if (32 + 24 * h.nPoints + 4 * h.nFaces + 4 * h.nIndices + 2 * nSlots > size) return fail(label + ": truncated slot block");
  std::unique_ptr<HostMesh> m(new HostMesh);
  m->points.resize(3 * h.nPoints); m->counts.resize(h.nFaces); m->indices.resize(h.nIndices); m->slot.resize(nSlots);
  const char* p = data + sizeof h;
  if (h.nPoints) std::memcpy(m->points.data(), p, 24 * h.nPoints);
  p += 24 * h.nPoints;
  if (h.nFaces) std::memcpy(m->counts.data(), p, 4 * h.nFaces);
  p += 4 * h.nFaces;
  if (h.nIndices) std::memcpy(m->indices.data(), p, 4 * h.nIndices);
  p += 4 * h.nIndices;
  if (nSlots) std::memcpy(m->slot.data(), p, 2 * nSlots);
  // mesh_ok
  uint64_t sum = 0;
  uint32_t maxCorners = 0;
  for (int32_t c : m->counts) {
    if (c < 3) return fail(label + ": face with fewer than 3 vertices");
    sum += uint64_t(c);
    maxCorners = std::max(maxCorners, uint32_t(c));
  }
  if (sum != m->indices.size()) return fail(label + ": sum(counts) != n_indices");
  for (int32_t i : m->indices) if (i < 0 || uint64_t(i) >= h.nPoints) return fail(label + ": vertex index out of range");
  kgb_mesh_info& in = m->info;
  in.id = KGB_NO_MESH;
  in.nPoints = h.nPoints; in.nFaces = h.nFaces; in.nIndices = h.nIndices;
  in.hasSlots = nSlots ? 1u : 0u;
  uint32_t top = 0;
  for (uint16_t s : m->slot) top = std::max<uint32_t>(top, s);
  in.slots = (h.flags & 1) ? top + 1 : 1u;   // slot_count (src/mesh.cpp:170)
  in.maxCorners = maxCorners;
  in.triCap = sum - 2 * h.nFaces;
  for (int a = 0; a < 3; ++a) { in.lo[a] = INFINITY; in.hi[a] = -INFINITY; }
  for (size_t i = 0; i < m->points.size(); ++i) {   // bbox_centre's per-mesh box (src/mesh.cpp:110-112)
    in.lo[i % 3] = std::fmin(in.lo[i % 3], m->points[i]);
    in.hi[i % 3] = std::fmax(in.hi[i % 3], m->points[i]);
  }
  if (h.nFaces) {   // an empty mesh is dropped (src/mesh.cpp:472)
    in.id = uint32_t(g.meshes.size());
    *info = in;
    g.meshes.push_back(std::move(m));
    return 1;
  }
  *info = in;
  return 1;
}
HostMesh* host_mesh(Engine& g, uint32_t id) { return id < g.meshes.size() ? g.meshes[id].get() : nullptr; }

unsigned n_threads() {
  if (const char* e = std::getenv("KGB_ORACLE_THREADS")) { const int k = std::atoi(e); if (k > 0) return unsigned(k); }
  return std::max(1u, std::thread::hardware_concurrency());
}
// f(k) for k in [0, n) on the host's threads; callers write disjoint outputs
void par_for(size_t n, const std::function<void(size_t)>& f) {
  const unsigned T = std::min<size_t>(n_threads(), std::max<size_t>(1, n));
  if (T <= 1 || n < 2) { for (size_t k = 0; k < n; ++k) f(k); return; }
  std::atomic<size_t> next{0};
  std::vector<std::thread> th;
  for (unsigned q = 0; q < T; ++q)
    th.emplace_back([&] { for (size_t k; (k = next.fetch_add(1)) < n;) f(k); });
  for (auto& t : th) t.join();
}
using Clk = std::chrono::steady_clock;
double ms_since(Clk::time_point t0) { return std::chrono::duration<double, std::milli>(Clk::now() - t0).count(); }

const kgb_slot& record(const Engine& g, uint32_t prim) {   // the hit record of a triangle (gpu.cu:459-476)
  const uint32_t s = g.sc->slotted ? g.sc->slot[prim] : 0u;
  static const kgb_slot opaque{0.2f, 0.f, 0.f, 0u};
  return s < g.slots.size() ? g.slots[s] : opaque;
}

// trace_dev.cu:147-165 (__anyhit__tr): what a translucent crossing passes.
float crossing(const Engine& g, const Hit& h, F3 d) {
  const kgb_slot& s = record(g, h.prim);
  float T = s.tau;
  if ((s.flags & KGB_SLOT_THIN) && h.front == ((s.flags & KGB_SLOT_INWARD) != 0)) T = 1.f;
  else if (s.flags & KGB_SLOT_GLASS) {
    const Scene& sc = *g.sc;
    const F3 v0 = sc.v[sc.tri[3 * h.prim]], v1 = sc.v[sc.tri[3 * h.prim + 1]], v2 = sc.v[sc.tri[3 * h.prim + 2]];
    const float ax = v1.x - v0.x, ay = v1.y - v0.y, az = v1.z - v0.z;
    const float bx = v2.x - v0.x, by = v2.y - v0.y, bz = v2.z - v0.z;
    const float nx = ay * bz - az * by, ny = az * bx - ax * bz, nz = ax * by - ay * bx;
    float R;
    glass_TR(std::fabs(nx * d.x + ny * d.y + nz * d.z) * (1.f / std::sqrt(nx * nx + ny * ny + nz * nz)), s.tn, T, R);
  }
  return T;
}

// trace_dev.cu:91-108 (__raygen__bits) restated over the ray's hit set: direction d of a sensor (normal n, origin o
// = offset_ray) is visible when it is in the hemisphere (n.d > 0) and every hit from tmin 1e-5 on is an own-plane hit
// (own_hit), at most 3 of them (past_own_plane's 4 segments). Reference difference, degenerate cases only: hits at the
// same t each count; a hit that passes own_plane but not own_hit's 1/32 m test (triangles over 2^17 m) blocks.
bool visible_bit(const Engine& g, F3 o, F3 n, F3 dir, bool cull) {
  if (!(n.x * dir.x + n.y * dir.y + n.z * dir.z > 0.f)) return false;
  const Ray r = make_ray(o, dir);
  bool blocked = false;
  int own = 0;
  for_hits(*g.sc, r, 1e-5f, INFINITY, cull, [&](const Hit& h) {
    if (own_hit(*g.sc, h, dir, n) && ++own <= 3) return false;
    blocked = true;
    return true;
  });
  return !blocked;
}
// trace_dev.cu:115-143 (__raygen__bytes) + :147-165 (__anyhit__tr): the transmittance along the ray, x255. Own-plane
// hits pass (at most 3); an opaque hit blocks; translucent crossings multiply in the order of (t, primitive) from
// T = 1, the ray blocked once T < 1/510 (it would round to byte 0). Reference difference: a translucent own plane
// passes untouched (the reference multiplies its tau where float error meets it: its ponytail, trace_dev.cu:112-114).
uint8_t visible_byte(const Engine& g, F3 o, F3 n, F3 dir, bool cull) {
  if (!(n.x * dir.x + n.y * dir.y + n.z * dir.z > 0.f)) return 0;
  const Ray r = make_ray(o, dir);
  bool blocked = false;
  int own = 0;
  std::vector<Hit> tr;
  for_hits(*g.sc, r, 1e-5f, INFINITY, cull, [&](const Hit& h) {
    if (own_hit(*g.sc, h, dir, n)) { if (++own <= 3) return false; blocked = true; return true; }
    if (!g.sc->translucent[h.prim]) { blocked = true; return true; }
    tr.push_back(h);
    return false;
  });
  if (blocked) return 0;
  std::sort(tr.begin(), tr.end(), [](const Hit& a, const Hit& b) { return a.t < b.t || (a.t == b.t && a.prim < b.prim); });
  float T = 1.f;
  for (const Hit& h : tr) {
    T *= crossing(g, h, dir);
    if (!(T >= 1.f / 510.f)) return 0;
  }
  return (uint8_t)std::nearbyint(T * 255.f);
}

// gpu.cu:505-529: the adaptive sub-launch policy, kept for its stats (launches) and cancel points.
template <class Fn>
void sub_launches(Engine& g, size_t nc, bool any, size_t nWords, Fn&& run) {
  const double targetMs = any ? 30 : 150;
  const size_t nMin = any ? std::max<size_t>(1, (size_t(1) << 13) / std::max<size_t>(1, nWords)) : 1024;
  size_t done = 0, n = std::min(any ? nMin : size_t(4096), nc);
  while (done < nc) {
    const auto t0 = Clk::now();
    run(done, n);
    const double ms = ms_since(t0);
    g.stats.traceMs += ms; g.stats.rays += n * g.nDir; g.stats.launches++;
    done += n;
    const double want = double(n) * targetMs / std::max(ms, 1e-3);
    n = std::min({std::max<size_t>(want > 1e12 ? size_t(1) << 40 : size_t(want), nMin), any ? 2 * n : nc, nc - done});
  }
}

// trace_dev.cu:235-242 (cosine_dir), sincospif as kgb_sincospi
F3 cosine_dir(F3 n, float u, float v) {
  const float sg = std::copysign(1.f, n.z), a = -1.f / (sg + n.z), b = n.x * n.y * a;
  const F3 t = f3(1.f + sg * n.x * n.x * a, sg * b, -sg * n.x), w = f3(b, sg + n.y * n.y * a, -n.y);
  float s, c;
  kgb_sincospi(2.f * v, &s, &c);
  const float r = std::sqrt(u);
  return add(add(mul(r * c, t), mul(r * s, w)), mul(std::sqrt(std::max(0.f, 1.f - u)), n));
}
// trace_dev.cu:244-258 (sky_bin), asinf / atan2f as kgb_asin / kgb_atan2
const unsigned kTnaz[7] = {30, 30, 24, 24, 18, 12, 6};
unsigned sky_bin(F3 d, unsigned mf, unsigned nBins, float alpha, float cosN, float sinN) {
  if (!(d.z >= 0.f)) return 0;
  const unsigned r = std::min(unsigned(kgb_asin(std::min(d.z, 1.f)) / alpha), 7 * mf);
  if (r == 7 * mf) return nBins - 1;
  const unsigned n = kTnaz[r / mf] * mf;
  unsigned b = 1 + (r % mf) * n;
  for (unsigned q = 0; q < r / mf; ++q) b += kTnaz[q] * mf * mf;
  float az = kgb_atan2(d.x * cosN + d.y * sinN, d.y * cosN - d.x * sinN);
  if (az < 0.f) az += 6.28318531f;
  return b + unsigned(az * (float(n) / 6.28318531f) + .5f) % n;
}

// The reported distance of the hit that decided a view ray. The watertight test's t = T / det rounds with the vertices'
// coordinates relative to the origin, so a triangle whose vertices lie far beyond the hit (a kilometre-long ground quad
// seen from 100 m) gives t off by up to 1e-3 relative. Where a vertex lies more than 4 t from the origin along an axis
// (in float), t is recomputed from the triangle's plane in double: float(dot(v0 - o, ng)) / float(dot(d, ng)) with
// ng = (v1 - v0) x (v2 - v0), whose differences and products of float coordinates are exact or within 2^-52 in double;
// the result lies within 2 ulps of the exact distance. Measured against a double-precision walk on the 2 M-triangle views
// city: 9 % of the hits are recomputed, and every distance lies within 3.2e-6 of the double one (7e-4 without). The walk
// itself (which hits, their order, the own-plane rules) keeps the float t.
bool g_refine = true;   // kgbo_set_refine: a test switches the refinement off to plant the error it removes
float refine_t(F3 o, F3 d, F3 v0, F3 v1, F3 v2, float t) {
  if (!g_refine) return t;
  const float reach = std::max({std::fabs(v0.x - o.x), std::fabs(v0.y - o.y), std::fabs(v0.z - o.z), std::fabs(v1.x - o.x), std::fabs(v1.y - o.y),
                                std::fabs(v1.z - o.z), std::fabs(v2.x - o.x), std::fabs(v2.y - o.y), std::fabs(v2.z - o.z)});
  if (!(reach > 4.f * t)) return t;
  const double ex = double(v1.x) - double(v0.x), ey = double(v1.y) - double(v0.y), ez = double(v1.z) - double(v0.z);
  const double fx = double(v2.x) - double(v0.x), fy = double(v2.y) - double(v0.y), fz = double(v2.z) - double(v0.z);
  const double nx = ey * fz - ez * fy, ny = ez * fx - ex * fz, nz = ex * fy - ey * fx;
  const double num = ((double(v0.x) - double(o.x)) * nx + (double(v0.y) - double(o.y)) * ny) + (double(v0.z) - double(o.z)) * nz;
  const double den = (double(d.x) * nx + double(d.y) * ny) + double(d.z) * nz;
  const float r = float(num) / float(den);
  return r > 0.f && r < INFINITY ? r : t;
}

// trace_dev.cu:200-232 (__raygen__view's walk) for one ray: its class and distance. Own-plane hits are stepped over
// (at most 3; the 4th ends the ray as an obstruction at its distance), panes labelled KGB_LABEL_PASS are passed (at most
// 16) and set the glazed bit; a downward ray ends 1 cm below the virtual ground, whose plane it reports on a miss. The
// distance of the hit that ends the walk is refine_t's.
void view_ray(const Engine& g, F3 o, F3 nn, F3 dir, bool none, bool cull, const kgb_view_in& v, uint8_t& cl, float& t) {
  const float inf = INFINITY;
  cl = 2;
  t = inf;
  if (none || (v.cull && dot(nn, dir) <= 0.f)) { cl = 254; return; }
  if (v.vground && dir.z < 0.f && !(o.z > v.groundZ)) { cl = 1; t = 0.1f; return; }
  const bool plane = v.vground && dir.z < 0.f;
  const float tg = plane ? (o.z - v.groundZ) / -dir.z : inf;
  const float tmax = plane ? (o.z - v.groundZ + 0.01f) / -dir.z : FLT_MAX;
  float tmin = 1e-5f;
  unsigned own = 0, panes = 0;
  const Ray ray = make_ray(o, dir);
  Hit hh;
  bool byHit = false;   // the walk ended on a hit (not past the last one)
  for (;;) {
    if (!closest(*g.sc, ray, tmin, tmax, cull, hh)) { cl = dir.z >= 0.f ? 0 : 1; t = tg; break; }
    t = hh.t;
    if (own_hit(*g.sc, hh, dir, nn)) { if (++own == 4) { byHit = true; break; } }
    else {
      const uint8_t lb = g.label.empty() ? 2 : g.label[hh.prim];
      if (lb != KGB_LABEL_PASS) { cl = lb; byHit = true; break; }
      if (++panes > KGB_MAX_PANES) { byHit = true; break; }
    }
    tmin = next_up(t);
  }
  if (byHit) t = refine_t(o, dir, g.sc->v[g.sc->tri[3 * hh.prim]], g.sc->v[g.sc->tri[3 * hh.prim + 1]], g.sc->v[g.sc->tri[3 * hh.prim + 2]], t);
  if (panes) cl |= KGB_VIEW_GLAZED;
}

// The frame of a sensor's view field (trace_dev.cu:186-197): world-fixed (360 mode, turned by north) or the normal's.
void view_frame(F3 nn, bool world, float cosN, float sinN, F3& f, F3& r, F3& u) {
  if (world) { f = f3(-sinN, cosN, 0.f); r = f3(cosN, sinN, 0.f); u = f3(0.f, 0.f, 1.f); return; }
  const float l = std::sqrt(nn.x * nn.x + nn.y * nn.y);
  f = nn;
  if (l > 1e-3f) r = f3(nn.y / l, -nn.x / l, 0.f);
  else {
    r = f3(cosN, sinN, 0.f);
    if (l > 0.f) { r = sub(r, mul(dot(r, nn), nn)); r = mul(1.f / std::sqrt(dot(r, r)), r); }
  }
  u = f3(r.y * f.z - r.z * f.y, r.z * f.x - r.x * f.z, r.x * f.y - r.y * f.x);
}

// params.h:77-89 (view_cell / view_local), sincospif as kgb_sincospi
F3 view_cell(unsigned d, unsigned col, float rsx, float rsy, float az0, float dAz, bool jitter, unsigned element, unsigned side) {
  float a = 0.5f, s = 0.5f * (rsx + rsy);
  if (jitter) { const U3 h = pcg3d(element, d, side); a = u01(h.x); s = rsx + u01(h.y) * (rsy - rsx); }
  float sa, ca;
  kgb_sincospi((az0 + (float(col) + a) * dAz) * (1.f / 180.f), &sa, &ca);
  const float c = std::sqrt(std::max(0.f, 1.f - s * s));
  return f3(c * sa, c * ca, s);
}

}  // namespace

// ============================================================================================================ C ABI
extern "C" {

KGB_API int32_t kgb_version(void) { return KGB_ABI_VERSION; }
KGB_API const char* kgb_last_error(void) { return g_err.c_str(); }

KGB_API kgb_engine* kgb_init(void) {
  Engine* g = new Engine;
  g->sc = new Scene;
  return reinterpret_cast<kgb_engine*>(g);
}
KGB_API void kgb_destroy(kgb_engine* e) {
  if (!e) return;
  Engine* g = reinterpret_cast<Engine*>(e);
  delete g->sc;
  delete g;
}

KGB_API uint64_t kgb_build_bytes(kgb_engine*, size_t nv, size_t nt, int slotted) {
  // the engine's formula (kit-sim_daylight_gb300/csrc/engine.cu: build_bytes): inputs + triangle records + nodes bound
  if (!nt) return 0;
  const uint64_t inputs = uint64_t(nv) * 12 + uint64_t(nt) * (12 + (slotted ? 4 : 0));
  const uint64_t out = uint64_t(nt) * 64 + (uint64_t(nt) / 2 + 2) * 80 + 4096;
  return inputs + 2 * out;
}

KGB_API int kgb_build(kgb_engine* e, const float* v, size_t nv, const uint32_t* tri, size_t nt, const uint32_t* slot,
                      const kgb_slot* slots, size_t nSlots, int perSlot) {
  Engine& g = *reinterpret_cast<Engine*>(e);
  delete g.sc; g.sc = new Scene;
  g.stats.gasBytes = 0;
  if (!nt) return 1;
  const auto t0 = Clk::now();
  // gpu.cu:386-392: slot checks
  if (slot) for (size_t k = 0; k < nt; ++k) if (slot[k] >= nSlots) return fail("gpu_build: a triangle's slot has no Slot");
  bool anyTau = false;
  for (size_t s = 0; s < nSlots; ++s) anyTau = anyTau || slots[s].tau > 0;
  const bool slotted = perSlot || anyTau;
  if (slotted && !slot) return fail("gpu_build: per-slot records need a slot per triangle");
  for (size_t k = 0; k < 3 * nt; ++k) if (tri[k] >= nv) return fail("gpu_build: a triangle's vertex index exceeds the vertices");
  Scene& s = *g.sc;
  s.v.resize(nv);
  for (size_t k = 0; k < nv; ++k) s.v[k] = f3(v[3 * k], v[3 * k + 1], v[3 * k + 2]);
  s.tri.assign(tri, tri + 3 * nt);
  s.slotted = slotted;
  s.slot.assign(nt, 0);
  s.translucent.assign(nt, 0);
  for (size_t k = 0; slotted && k < nt; ++k) { s.slot[k] = slot[k]; s.translucent[k] = slots[slot[k]].tau > 0; }
  build_bvh(s);
  s.bytes = uint64_t(nt) * 64 + uint64_t(s.nodes.size()) * 32;
  g.stats.gasBytes = s.bytes;
  g.stats.buildTempBytes = uint64_t(nt) * 36;
  g.stats.buildOutputBytes = s.bytes;
  g.stats.buildMs += ms_since(t0);
  return 1;
}

KGB_API void kgb_trim(kgb_engine* e, int sensors) {
  Engine& g = *reinterpret_cast<Engine*>(e);
  g.bits.clear(); g.bits.shrink_to_fit(); g.byt.clear(); g.byt.shrink_to_fit();
  g.dc.clear(); g.cls.clear(); g.dist.clear(); g.viewN = 0;
  if (sensors) { g.P.clear(); g.N.clear(); g.label.clear(); g.nSensors = 0; }
}

KGB_API int kgb_set_slots(kgb_engine* e, const kgb_slot* slots, size_t n) {
  Engine& g = *reinterpret_cast<Engine*>(e);
  g.slots.assign(slots, slots + n);
  if (g.slots.empty()) g.slots.push_back(kgb_slot{0.2f, 0.f, 0.f, 0u});
  return 1;
}

KGB_API kgb_scene kgb_detach(kgb_engine* e) {
  Engine& g = *reinterpret_cast<Engine*>(e);
  kgb_scene s{g.sc, g.sc->bytes};
  g.sc = new Scene;
  g.stats.gasBytes = 0;
  return s;
}
KGB_API void kgb_attach(kgb_engine* e, kgb_scene s) {
  Engine& g = *reinterpret_cast<Engine*>(e);
  delete g.sc;
  g.sc = s.handle ? static_cast<Scene*>(s.handle) : new Scene;
  g.stats.gasBytes = g.sc->bytes;
}
KGB_API void kgb_free_scene(kgb_scene* s) {
  if (!s) return;
  delete static_cast<Scene*>(s->handle);
  s->handle = nullptr; s->bytes = 0;
}
KGB_API uint64_t kgb_free_bytes(void) { return uint64_t(64) << 30; }

KGB_API int kgb_set_scene(kgb_engine* e, const float* P, const float* N, size_t nSensors, const float* D, size_t nDir) {
  Engine& g = *reinterpret_cast<Engine*>(e);
  g.nSensors = nSensors; g.nDir = nDir; g.nWords = (nDir + 31) / 32;
  g.P.resize(nSensors); g.N.resize(nSensors); g.D.resize(nDir);
  for (size_t k = 0; k < nSensors; ++k) { g.P[k] = f3(P[3 * k], P[3 * k + 1], P[3 * k + 2]); g.N[k] = f3(N[3 * k], N[3 * k + 1], N[3 * k + 2]); }
  for (size_t k = 0; k < nDir; ++k) g.D[k] = f3(D[3 * k], D[3 * k + 1], D[3 * k + 2]);
  return 1;
}

KGB_API int kgb_set_labels(kgb_engine* e, const uint8_t* label, size_t n) {
  Engine& g = *reinterpret_cast<Engine*>(e);
  g.label.assign(label, label + n);
  return 1;
}

KGB_API int kgb_trace(kgb_engine* e, size_t i0, size_t nc, uint32_t rayFlags) {
  Engine& g = *reinterpret_cast<Engine*>(e);
  if (i0 + nc > g.nSensors) return fail("gpu_trace: sensor range exceeds the scene");
  g.bytes = !(rayFlags & KGB_RAY_DISABLE_ANYHIT);
  g.i0 = i0;
  const bool cull = (rayFlags & KGB_RAY_CULL_BACK_FACING) != 0;
  if (g.bytes) g.byt.assign(g.nDir * nc, 0); else g.bits.assign(g.nWords * nc, 0u);
  if (nc == 0 || g.nWords == 0) return 1;
  sub_launches(g, nc, g.bytes, g.nWords, [&](size_t done, size_t n) {
    par_for(n, [&](size_t j) {
      const size_t i = done + j;
      const F3 n = g.N[i0 + i], o = offset_ray(g.P[i0 + i], n);
      if (g.bytes) {
        for (size_t d = 0; d < g.nDir; ++d) g.byt[d * nc + i] = visible_byte(g, o, n, g.D[d], cull);
      } else {
        for (size_t w = 0; w < g.nWords; ++w) {
          uint32_t word = 0;
          for (unsigned k = 0; k < 32 && w * 32 + k < g.nDir; ++k)
            if (visible_bit(g, o, n, g.D[w * 32 + k], cull)) word |= 1u << k;
          g.bits[w * nc + i] = word;
        }
      }
    });
  });
  return 1;
}

// gpu.cu:69-72 (dotf, rounded per operation) and 99-114 (k_reduce): FP32 products, FP64 sum in direction order.
static inline float dotf(F3 a, F3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }

KGB_API int kgb_reduce(kgb_engine* e, size_t nc, const float* W, int useCos, double* out) {
  Engine& g = *reinterpret_cast<Engine*>(e);
  if (nc == 0) return 1;
  const size_t have = g.bytes ? g.byt.size() : g.bits.size();
  if (have != (g.bytes ? g.nDir : g.nWords) * nc) return fail("gpu_reduce: no trace of this chunk");
  par_for(nc, [&](size_t i) {
    const F3 n = g.N[g.i0 + i];
    double acc = 0;
    for (size_t d = 0; d < g.nDir; ++d) {
      float at;
      if (g.bytes) { const uint8_t b = g.byt[d * nc + i]; if (!b) continue; at = float(b) / 255.f; }
      else { if (!((g.bits[(d >> 5) * nc + i] >> (d & 31)) & 1u)) continue; at = 1.f; }
      acc += (double)((useCos ? std::max(dotf(n, g.D[d]), 0.f) : 1.f) * at) * W[d];
    }
    out[i] = acc;
  });
  return 1;
}
// The restatement has no device memory to stage in: the no-allocation reduce is its reduce.
KGB_API int kgb_reduce_noalloc(kgb_engine* e, size_t nc, const float* W, int useCos, double* out) { return kgb_reduce(e, nc, W, useCos, out); }

// gpu.cu:116-169 (k_series, k_series_dc) as an FP64 contraction of the same FP32 per-direction weights: the reference
// the engine's FP32 and split-BF16 forms are measured against. E is float(the double sum).
KGB_API int kgb_series(kgb_engine* e, size_t nc, const kgb_series_in* in, float* E) {
  Engine& g = *reinterpret_cast<Engine*>(e);
  if (nc == 0 || in->T <= 0) return 1;
  if (in->Sdc && nc != g.dcN) return fail("gpu_series: no gpu_bounce rows for this chunk");
  const size_t T = size_t(in->T);
  par_for(nc, [&](size_t i) {
    const F3 n = g.N[g.i0 + i];
    std::vector<double> acc(T, 0.0);
    for (unsigned d = 0; d < in->nSky && d < g.nDir; ++d) {
      float at;
      if (g.bytes) { const uint8_t b = g.byt[size_t(d) * nc + i]; if (!b) continue; at = float(b) / 255.f; }
      else { if (!((g.bits[(d >> 5) * nc + i] >> (d & 31)) & 1u)) continue; at = 1.f; }
      const float c = std::max(dotf(n, g.D[d]), 0.f) * at * in->wsky[d];
      const float* s = in->S + size_t(in->row[d]) * T;
      for (size_t t = 0; t < T; ++t) acc[t] += double(c) * s[t];
    }
    for (size_t t = 0; t < T; ++t) acc[t] += double(in->G[i]) * in->g[t];
    for (unsigned j = 0; j < in->nSun; ++j) {
      const size_t d = in->sun0 + j;
      float at;
      if (g.bytes) { const uint8_t b = g.byt[d * nc + i]; if (!b) continue; at = float(b) / 255.f; }
      else { if (!((g.bits[(d >> 5) * nc + i] >> (d & 31)) & 1u)) continue; at = 1.f; }
      const F3 sv = f3(in->sunVec[3 * j], in->sunVec[3 * j + 1], in->sunVec[3 * j + 2]);
      acc[size_t(in->sunStep[j])] += double(std::max(dotf(n, sv), 0.f) * at * in->sunW[j]);
    }
    if (in->Sdc)
      for (size_t b = 0; b < g.nBins; ++b) {
        const float c = g.dc[b * nc + i];
        if (c == 0.f) continue;
        for (size_t t = 0; t < T; ++t) acc[t] += double(c) * in->Sdc[b * T + t];
      }
    for (size_t t = 0; t < T; ++t) E[i * T + t] = float(acc[t]);
  });
  return 1;
}

// gpu_series + the caller's fwrite of E (run.cpp:683-686): the same rows written to fd at offset
KGB_API int kgb_series_file(kgb_engine* e, size_t nc, const kgb_series_in* in, int fd, uint64_t offset) {
  if (fd < 0) return fail("gpu_series: no file");
  std::vector<float> E(nc * size_t(in->T > 0 ? in->T : 0));
  if (!kgb_series(e, nc, in, E.data())) return 0;
  const char* p = reinterpret_cast<const char*>(E.data());
  size_t left = E.size() * 4, at = 0;
  while (left) {
    const ssize_t n = pwrite(fd, p + at, left, off_t(offset + at));
    if (n < 0 && errno == EINTR) continue;
    if (n <= 0) return fail("gpu_series: writing the series file failed");
    at += size_t(n);
    left -= size_t(n);
  }
  return 1;
}

// trace_dev.cu:260-311 (__raygen__bounce) + gpu.cu:533-568. Closest hits by (t, primitive); the row sum in float,
// in sample order, each add rounded separately (the engine's kernel does the same, without contraction).
KGB_API int kgb_bounce(kgb_engine* e, size_t i0, size_t nc, uint32_t rayFlags, const kgb_bounce_in* b) {
  Engine& g = *reinterpret_cast<Engine*>(e);
  if (i0 + nc > g.nSensors) return fail("gpu_bounce: sensor range exceeds the scene");
  const unsigned mf = unsigned(b->mf);
  const double alphaD = (KGB_PI_D / 2.) / (7 * mf + .5);
  const float alpha = float(alphaD);
  g.nBins = size_t(144 * mf * mf + 1) + 1; g.dcN = nc; g.dcI0 = i0;
  g.dc.assign(g.nBins * nc, 0.f);
  if (nc == 0) return 1;
  const bool cull = (rayFlags & KGB_RAY_CULL_BACK_FACING) != 0;
  const double rad = b->north * KGB_PI_D / 180;
  const float cosN = float(std::cos(rad)), sinN = float(std::sin(rad));
  const unsigned M = b->M, NB = b->N, nBins = unsigned(g.nBins);
  for (size_t done = 0, n = std::clamp<size_t>((size_t(1) << 13) / nc, 1, 64); done < M;) {
    if (b->cancel && b->cancel(b->cancelCtx)) return fail("cancelled");
    n = std::min<size_t>(n, M - done);
    const unsigned s0 = unsigned(done), s1 = unsigned(done + n);
    const auto t0 = Clk::now();
    par_for(nc, [&](size_t i) {
      const unsigned gi = unsigned(i0 + i);
      const F3 nn = g.N[i0 + i], o0 = offset_ray(g.P[i0 + i], nn);
      const U3 rot = pcg3d(gi, ~0u, ~0u);
      const float r0 = u01(rot.x), r1 = u01(rot.y), weight = 3.14159265f / float(M);
      float* row = g.dc.data() + i;
      for (unsigned s = s0; s < s1; ++s) {
        const float u = float(s) / float(M) + r0, v = u01(brev(s)) + r1;
        F3 o = o0, d = cosine_dir(nn, u - std::floor(u), v - std::floor(v));
        float w = 1.f;
        unsigned diffuse = 0, k = 0;
        bool reflected = false;
        for (unsigned seg = 0; seg < NB + 16; ++seg) {
          Hit hh;
          if (!closest(*g.sc, make_ray(o, d), 1e-5f, FLT_MAX, cull, hh)) {
            if (reflected) { float& c = row[sky_bin(d, mf, nBins, alpha, cosN, sinN) * nc]; c = c + w * weight; }
            break;
          }
          const kgb_slot sl = record(g, hh.prim);
          TriHit h;
          if (!hit_triangle(*g.sc, hh, h)) break;
          if (seg == 0 && own_plane(h, hh.t, d, nn)) { o = through(h); continue; }
          if ((sl.flags & (KGB_SLOT_THIN | KGB_SLOT_TWIN)) == KGB_SLOT_THIN && h.front == ((sl.flags & KGB_SLOT_INWARD) != 0)) { o = through(h); continue; }
          const bool mirror = (sl.flags & KGB_SLOT_GLASS) != 0;
          float T = sl.tau, R = sl.rho;
          if (mirror) { glass_TR(std::fabs(dot(d, h.n)), sl.tn, T, R); if (!(sl.tau > 0.f)) T = 0.f; }
          else if (diffuse == NB) R = 0.f;
          if (!(T + R > 0.f)) break;
          const U3 r = pcg3d(gi, s, k++);
          w *= T + R;
          if (u01(r.x) * (T + R) < T) { o = through(h); continue; }
          reflected = true;
          if (mirror) d = sub(d, mul(2.f * dot(d, h.n), h.n));
          else {
            d = cosine_dir(h.n, u01(r.y), u01(r.z));
            if (++diffuse >= 2) {
              if (u01(pcg3d(gi, s, k++).x) >= w) break;
              w = 1.f;
            }
          }
          o = add(offset_ray(h.p, h.n), h.lift);
        }
      }
    });
    const double ms = ms_since(t0);
    g.stats.bounceMs += ms; g.stats.paths += n * nc; g.stats.bounceLaunches++;
    done += n;
    const double want = double(n) * 100 / std::max(ms, 1e-3);
    n = std::max<size_t>(1, std::min<size_t>(2 * n, want > 1e9 ? size_t(1e9) : size_t(want)));
  }
  return 1;
}

KGB_API int kgb_reduce_dc(kgb_engine* e, size_t nc, const float* W, double* out) {
  Engine& g = *reinterpret_cast<Engine*>(e);
  if (nc == 0) return 1;
  if (nc != g.dcN) return fail("gpu_reduce_dc: no gpu_bounce rows for this chunk");
  par_for(nc, [&](size_t i) {   // gpu.cu:93-114 (k_reduce<Dc>): every bin, no cosine
    double acc = 0;
    for (size_t b = 0; b < g.nBins; ++b) acc += (double)(1.f * g.dc[b * nc + i]) * W[b];
    out[i] = acc;
  });
  return 1;
}

KGB_API int kgb_download_dc(kgb_engine* e, size_t nc, float* out, size_t count) {
  Engine& g = *reinterpret_cast<Engine*>(e);
  if (nc != g.dcN) return fail("gpu_download_dc: no gpu_bounce rows for this chunk");
  if (count != g.nBins * nc) return fail("gpu_download_dc: wrong count");
  std::copy(g.dc.begin(), g.dc.end(), out);
  return 1;
}
KGB_API int kgb_download_bits(kgb_engine* e, size_t nc, uint32_t* out, size_t count) {
  Engine& g = *reinterpret_cast<Engine*>(e);
  if (g.bytes) return fail("gpu_download_bits: the last trace wrote bytes");
  if (count != g.nWords * nc || g.bits.size() != count) return fail("gpu_download_bits: wrong count");
  std::copy(g.bits.begin(), g.bits.end(), out);
  return 1;
}
KGB_API int kgb_download_bytes(kgb_engine* e, size_t nc, uint8_t* out, size_t count) {
  Engine& g = *reinterpret_cast<Engine*>(e);
  if (!g.bytes) return fail("gpu_download_bytes: the last trace wrote bits");
  if (count != g.nDir * nc || g.byt.size() != count) return fail("gpu_download_bytes: wrong count");
  std::copy(g.byt.begin(), g.byt.end(), out);
  return 1;
}
// run.cpp:659-671 (--dump-bits): the direction-major buffers as one row per sensor
KGB_API int kgb_download_bits_rows(kgb_engine* e, size_t nc, uint32_t* out, size_t count) {
  Engine& g = *reinterpret_cast<Engine*>(e);
  if (g.bytes) return fail("gpu_download_bits: the last trace wrote bytes");
  if (count != g.nWords * nc || g.bits.size() != count) return fail("gpu_download_bits: wrong count");
  for (size_t w = 0; w < g.nWords; ++w)
    for (size_t i = 0; i < nc; ++i) out[i * g.nWords + w] = g.bits[w * nc + i];
  return 1;
}
KGB_API int kgb_download_bytes_rows(kgb_engine* e, size_t nc, uint8_t* out, size_t count) {
  Engine& g = *reinterpret_cast<Engine*>(e);
  if (!g.bytes) return fail("gpu_download_bytes: the last trace wrote bits");
  if (count != g.nDir * nc || g.byt.size() != count) return fail("gpu_download_bytes: wrong count");
  for (size_t d = 0; d < g.nDir; ++d)
    for (size_t i = 0; i < nc; ++i) out[i * g.nDir + d] = g.byt[d * nc + i];
  return 1;
}

// trace_dev.cu:167-232 (__raygen__view) + gpu.cu:572-610. The closest-hit walk over the ray's hits ordered by
// (t, primitive): own planes (own_hit) pass, at most 3, the 4th ends the ray as an obstruction; a triangle labelled
// KGB_LABEL_PASS is passed (at most 16, the 17th ends it); the next hit starts past t (next float).
KGB_API int kgb_view(kgb_engine* e, size_t i0, size_t nc, uint32_t rayFlags, const kgb_view_in* v, size_t* launch) {
  Engine& g = *reinterpret_cast<Engine*>(e);
  if (i0 + nc > g.nSensors) return fail("gpu_view: sensor range exceeds the scene");
  const size_t K = size_t(v->nAz) * v->nEl, nWords = (K + 31) / 32;
  g.viewN = nc; g.viewK = K; g.viewI0 = i0; g.view = *v;
  g.rowSin.assign(v->rowSin, v->rowSin + 2 * size_t(v->nEl));
  g.view.rowSin = g.rowSin.data();
  g.cls.assign(K * nc, 0); g.dist.assign(K * nc, 0.f);
  if (nc == 0 || K == 0) return 1;
  const bool cull = (rayFlags & KGB_RAY_CULL_BACK_FACING) != 0;
  const double rad = v->north * KGB_PI_D / 180;
  const float cosN = float(std::cos(rad)), sinN = float(std::sin(rad));
  const size_t nMin = std::max<size_t>(1, (size_t(1) << 13) / nWords);
  size_t n = std::max(*launch, nMin);
  for (size_t done = 0; done < nc;) {
    if (v->cancel && v->cancel(v->cancelCtx)) return fail("cancelled");
    const size_t m = std::min(n, nc - done);
    const auto t0 = Clk::now();
    par_for(m, [&](size_t j) {
      const size_t i = done + j;
      const unsigned gi = unsigned(i0 + i), element = gi / v->nS, side = v->nS == 2 ? gi % 2 : unsigned(v->back != 0);
      const F3 nn = g.N[i0 + i], o = offset_ray(g.P[i0 + i], nn);
      const bool none = !(dot(nn, nn) > 0.f);
      F3 f, r, u;
      view_frame(nn, v->world != 0, cosN, sinN, f, r, u);
      for (size_t d = 0; d < K; ++d) {
        const unsigned col = unsigned(d % v->nAz), row = unsigned(d / v->nAz);
        const F3 l = view_cell(unsigned(d), col, g.rowSin[2 * row], g.rowSin[2 * row + 1], v->az0, v->dAz, v->jitter != 0, element, side);
        const F3 dir = add(add(mul(l.x, r), mul(l.y, f)), mul(l.z, u));
        uint8_t cl;
        float t;
        view_ray(g, o, nn, dir, none, cull, *v, cl, t);
        g.cls[d * nc + i] = cl;
        g.dist[d * nc + i] = t;
      }
    });
    const double ms = ms_since(t0);
    g.stats.traceMs += ms; g.stats.rays += m * K; g.stats.launches++;
    done += m;
    const double want = double(m) * 40 / std::max(ms, 1e-3);
    n = std::max(nMin, std::min(2 * n, want > 1e12 ? size_t(1) << 40 : size_t(want)));
  }
  *launch = n;
  return 1;
}

// gpu.cu:181-274 (warp_sum, iso_lane, k_iso, k_view): the lanes and the fixed shuffle tree restated exactly, so the
// doubles come out bit for bit as the engine's.
static double tree_sum(const double* lanes) {   // __shfl_down_sync tree, lane 0's result
  double v[32];
  std::copy(lanes, lanes + 32, v);
  for (unsigned s = 16; s; s >>= 1) {
    double nv[32];
    for (unsigned l = 0; l < 32; ++l) nv[l] = v[l] + (l + s < 32 ? v[l + s] : v[l]);
    std::copy(nv, nv + 32, v);
  }
  return v[0];
}

static float det3(F3 a, F3 b, F3 c) {
  const F3 u = sub(b, a), w = sub(c, a);
  return a.x * (u.y * w.z - u.z * w.y) + a.y * (u.z * w.x - u.x * w.z) + a.z * (u.x * w.y - u.y * w.x);
}

KGB_API int kgb_reduce_view(kgb_engine* e, size_t nc, const double* wRow, size_t nRow, uint32_t nClass, double farDist,
                            const float* reach, size_t nReach, int glazing, uint32_t isoDim, double* out) {
  Engine& g = *reinterpret_cast<Engine*>(e);
  if (nc == 0) return 1;
  if (nc != g.viewN) return fail("gpu_reduce_view: no gpu_view for this chunk");
  if (nClass > KGB_VIEW_CLASSES || nReach > 8) return fail("gpu_reduce_view: at most 16 groups and 8 reach distances");
  (void)nRow;
  const size_t NA = 3 * size_t(nClass) + 1 + nReach + (glazing ? 1 : 0) + (isoDim ? 1 : 0);
  const size_t K = g.viewK;
  const unsigned nAz = g.view.nAz, nEl = g.view.nEl;
  const float farF = float(farDist);
  const double lnFar = std::log(farDist);
  par_for(nc, [&](size_t i) {
    double w[32][KGB_VIEW_CLASSES] = {}, wl[32][KGB_VIEW_CLASSES] = {}, rc[32][8] = {}, own[32] = {}, gz[32] = {};
    float mn[KGB_VIEW_CLASSES];
    for (unsigned c = 0; c < KGB_VIEW_CLASSES; ++c) mn[c] = INFINITY;
    for (unsigned lane = 0; lane < 32; ++lane)
      for (size_t d = lane; d < K; d += 32) {
        unsigned c = g.cls[d * nc + i];
        const float t = g.dist[d * nc + i];
        const double wd = wRow[d / nAz];
        if (c == 254) { own[lane] += wd; continue; }
        if (c & KGB_VIEW_GLAZED) { gz[lane] += wd; c &= ~unsigned(KGB_VIEW_GLAZED); }
        const float dd = std::min(std::max(t, 0.1f), farF);
        w[lane][c] += wd;
        wl[lane][c] += wd * (dd == farF ? lnFar : dd == 0.1f ? -2.302585092994045684 : (double)kgb_logf(dd));
        mn[c] = std::min(mn[c], dd);
        for (size_t r = 0; r < nReach; ++r) if (t >= reach[r]) rc[lane][r] += wd;
      }
    double* o = out + i * NA;
    double lanes[32];
    for (unsigned c = 0; c < nClass; ++c) {
      for (unsigned l = 0; l < 32; ++l) lanes[l] = w[l][c];
      o[3 * c] = tree_sum(lanes);
      for (unsigned l = 0; l < 32; ++l) lanes[l] = wl[l][c];
      o[3 * c + 1] = tree_sum(lanes);
      o[3 * c + 2] = mn[c];
    }
    o[3 * nClass] = tree_sum(own);
    for (size_t r = 0; r < nReach; ++r) { for (unsigned l = 0; l < 32; ++l) lanes[l] = rc[l][r]; o[3 * nClass + 1 + r] = tree_sum(lanes); }
    if (glazing) o[3 * nClass + 1 + nReach] = tree_sum(gz);
    if (isoDim) {   // gpu.cu:204-236
      const kgb_view_in& v = g.view;
      const unsigned gi = unsigned(g.viewI0 + i), element = gi / v.nS, side = v.nS == 2 ? gi % 2 : unsigned(v.back != 0);
      const auto len = [&](unsigned k) { const size_t at = size_t(k) * nc + i; return g.cls[at] == 254 ? 0.f : std::min(g.dist[at], farF); };
      const auto dir = [&](unsigned d, unsigned col, unsigned row) {
        return view_cell(d, col, g.rowSin[2 * row], g.rowSin[2 * row + 1], v.az0, v.dAz, v.jitter != 0, element, side);
      };
      double lane_sum[32] = {};
      for (unsigned base = 0; base < nAz; base += 32) {
        // every lane's loads first (the shuffles read lane + 1's)
        for (unsigned lane = 0; lane < 32; ++lane) {
          const unsigned col = std::min(base + lane, nAz - 1), c1 = col + 1 == nAz ? 0 : col + 1;
          const bool on = base + lane < nAz && (v.world || col + 1 < nAz);
          const bool alone = lane == 31 || c1 == 0;
          const unsigned colN = std::min(base + lane + 1, nAz - 1);   // lane + 1's column (its l is what the shuffle gives)
          const auto pair = [&](unsigned row) {
            const float l = len(row * nAz + col);
            const float nb = lane == 31 ? l : len(row * nAz + colN);
            return std::make_pair(l, alone ? len(row * nAz + c1) : nb);
          };
          F3 a = dir(col, col, 0), b = dir(c1, c1, 0);
          auto l0 = pair(0);
          if (isoDim == 2) { if (on) lane_sum[lane] += double(0.5f * l0.first * l0.second * (a.y * b.x - a.x * b.y)); continue; }
          for (unsigned rr = 1; rr < nEl; ++rr) {
            const unsigned d = rr * nAz + col;
            const auto l1 = pair(rr);
            const F3 c = dir(d, col, rr), ee = dir(d - col + c1, c1, rr);
            if (on) lane_sum[lane] += double(l0.first * l0.second * l1.first * det3(a, b, c) + l0.second * l1.second * l1.first * det3(b, ee, c));
            a = c; b = ee; l0 = l1;
          }
        }
      }
      for (unsigned l = 0; l < 32; ++l) lanes[l] = isoDim == 2 ? lane_sum[l] : lane_sum[l] / 6;
      o[NA - 1] = tree_sum(lanes);
    }
  });
  return 1;
}

KGB_API int kgb_download_view(kgb_engine* e, size_t nc, uint8_t* cls, float* dist, size_t count) {
  Engine& g = *reinterpret_cast<Engine*>(e);
  if (nc != g.viewN) return fail("gpu_download_view: no gpu_view for this chunk");
  const size_t K = g.viewK;
  if (count != nc * K) return fail("gpu_download_view: wrong count");
  for (size_t d = 0; d < K; ++d)
    for (size_t i = 0; i < nc; ++i) { cls[i * K + d] = g.cls[d * nc + i]; dist[i * K + d] = g.dist[d * nc + i]; }
  return 1;
}

KGB_API kgb_stats kgb_get_stats(const kgb_engine* e) { return reinterpret_cast<const Engine*>(e)->stats; }
KGB_API int kgb_set_stream(kgb_engine*, void*) { return 1; }   // no device: nothing to select
// The sky side is not restated here: its checker is the reference's own sky.cpp / solar.cpp, whose outputs
// tests/golden/sky holds (oracle/ref_sky_golden.cpp).
// The server is the engine's batching of its own entry points; its checker is those entry points (alone vs in the mix).
KGB_API kgb_server* kgb_server_create(uint64_t) { fail("kgb_server_create: not restated (engine scheduling)"); return nullptr; }
KGB_API void kgb_server_destroy(kgb_server*) {}
KGB_API int kgb_server_add_scene(kgb_server*, const float*, size_t, const uint32_t*, size_t, int32_t*) { return fail("not restated"); }
KGB_API int kgb_server_autotune(kgb_server*) { return fail("not restated"); }
KGB_API int kgb_server_set_tuning(kgb_server*, uint32_t, uint64_t, uint64_t) { return fail("not restated"); }
KGB_API int kgb_server_set_priority(kgb_server*, double, double) { return fail("not restated"); }
KGB_API void kgb_server_tuning(kgb_server*, uint64_t* out) { out[0] = out[1] = out[2] = 0; }
KGB_API int kgb_server_submit(kgb_server*, const kgb_daylight_request*, uint64_t*) { return fail("not restated"); }
KGB_API int kgb_server_submit_views(kgb_server*, const kgb_views_request*, uint64_t*) { return fail("not restated"); }
KGB_API int kgb_server_submit_series(kgb_server*, const kgb_daylight_request*, const kgb_series_request*, uint64_t*) { return fail("not restated"); }
KGB_API int kgb_server_wait(kgb_server*, uint64_t, double) { return fail("not restated"); }
KGB_API void kgb_server_stats(kgb_server*, double* out) { for (int k = 0; k < 10; ++k) out[k] = 0; }
KGB_API void kgb_server_timing(kgb_server*, double* out) { for (int k = 0; k < 5; ++k) out[k] = 0; }
KGB_API int kgb_sky(kgb_engine*, int32_t, const kgb_sky_step*, size_t, double, int32_t, int32_t, int32_t, float*) {
  return fail("kgb_sky: the sky's checker is the reference's own code (tests/golden/sky)");
}
KGB_API int kgb_triangulate(kgb_engine*, const double*, size_t, const int32_t*, size_t, const int32_t*, const uint32_t*, const double*, uint32_t, uint32_t,
                            float*, uint32_t*, uint32_t*, size_t*, int32_t*) {
  return fail("kgb_triangulate: not restated here (the reference's own mesh code is the checker: tests/golden/mesh)");
}
KGB_API int kgb_thin_solids(kgb_engine*, const double*, size_t, const int32_t*, size_t, const int32_t*, const uint32_t*, uint32_t, const double*, uint32_t*) {
  return fail("kgb_thin_solids: not restated here (the reference's own mesh code is the checker: tests/golden/mesh)");
}
KGB_API int kgb_mesh_read(kgb_engine* e, const void* data, size_t size, const char* name, kgb_mesh_info* info) {
  if (!info) return fail("kgb_mesh_read: no info to write");
  if (size && !data) return fail("kgb_mesh_read: no image");
  return dmesh_parse(*reinterpret_cast<Engine*>(e), static_cast<const char*>(data), size, name ? name : "", info);
}
KGB_API int kgb_mesh_file(kgb_engine* e, const char* path, kgb_mesh_info* info) {   // read_dmesh(path): the whole file, then the image's parse
  const std::string p = path ? path : "";
  if (!info) return fail("kgb_mesh_file: no info to write");
  std::FILE* f = std::fopen(p.c_str(), "rb");
  if (!f) return fail("cannot open " + p);
  std::fseek(f, 0, SEEK_END);
  const long n = std::ftell(f);
  std::vector<char> buf(n > 0 ? size_t(n) : 0);
  std::rewind(f);
  const bool ok = n >= 0 && std::fread(buf.data(), 1, buf.size(), f) == buf.size();
  std::fclose(f);
  if (!ok) return fail(p + ": truncated");
  return dmesh_parse(*reinterpret_cast<Engine*>(e), buf.data(), buf.size(), p, info);
}
KGB_API int kgb_mesh_download(kgb_engine* e, uint32_t id, double* points, int32_t* counts, int32_t* indices, uint16_t* slot) {
  const HostMesh* m = host_mesh(*reinterpret_cast<Engine*>(e), id);
  if (!m) return fail("kgb_mesh_download: no mesh " + std::to_string(id));
  if (points) std::copy(m->points.begin(), m->points.end(), points);
  if (counts) std::copy(m->counts.begin(), m->counts.end(), counts);
  if (indices) std::copy(m->indices.begin(), m->indices.end(), indices);
  if (slot) std::copy(m->slot.begin(), m->slot.end(), slot);
  return 1;
}
KGB_API int kgb_mesh_free(kgb_engine* e, uint32_t id) {
  Engine& g = *reinterpret_cast<Engine*>(e);
  if (!host_mesh(g, id)) return fail("kgb_mesh_free: no mesh " + std::to_string(id));
  g.meshes[id].reset();
  return 1;
}
KGB_API int kgb_mesh_thin_solids(kgb_engine*, uint32_t, const double*, uint32_t*) {
  return fail("kgb_mesh_thin_solids: not restated here (the reference's own mesh code is the checker: tests/golden/mesh)");
}
KGB_API int kgb_build_meshes(kgb_engine*, const uint32_t*, size_t, const uint8_t*, const double*, const kgb_slot*, size_t, int, uint64_t*, int32_t*) {
  return fail("kgb_build_meshes: not restated here (the scene's checker is kgb_build on the triangulated arrays)");
}
KGB_API int kgb_sky_ladybug(kgb_engine*, int32_t, const double*, size_t, double, double, double, double, double, double*, float*, float*, float*) {
  return fail("kgb_sky_ladybug: the sky is not restated here (the reference's own sky code is the checker: tests/golden/ladybug)");
}
KGB_API int kgb_sun_noaa(kgb_engine*, const double*, size_t, double*) {
  return fail("kgb_sun_noaa: the sun's checker is the reference's own code (tests/golden/sky)");
}
// The restatement has one builder (its binary SAH tree): every builder choice gives the same results.
KGB_API int kgb_set_builder(kgb_engine*, int which) { return which == 0 || which == 1 ? 1 : fail("kgb_set_builder: 0 or 1"); }
// The engine's bounded-execution limits guard its device walks; the oracle's host recursion needs none, so there is
// nothing to lower here.
KGB_API int kgb_set_limits(kgb_engine*, uint32_t, uint64_t, uint64_t, uint32_t) { return 1; }
KGB_API int kgb_set_series_form(kgb_engine*, int form) { return form == 0 || form == 1 ? 1 : fail("kgb_set_series_form: 0 or 1"); }
KGB_API int kgb_trace_counters(kgb_engine*, size_t, size_t, uint32_t, uint64_t out[4]) {
  out[0] = out[1] = out[2] = out[3] = 0;
  return fail("kgb_trace_counters: the oracle has no device traversal to count");
}
KGB_API uint32_t kgb_ray_flags(int cullBackfaces, int translucent) {
  return KGB_RAY_TERMINATE_ON_FIRST_HIT | (translucent ? 0u : KGB_RAY_DISABLE_ANYHIT) | (cullBackfaces ? KGB_RAY_CULL_BACK_FACING : 0u);
}
KGB_API uint32_t kgb_bounce_flags(int cullBackfaces) { return KGB_RAY_DISABLE_ANYHIT | (cullBackfaces ? KGB_RAY_CULL_BACK_FACING : 0u); }
KGB_API void kgb_dims(const kgb_engine* e, uint64_t out[6]) {
  const Engine& g = *reinterpret_cast<const Engine*>(e);
  out[0] = g.nSensors; out[1] = g.nDir; out[2] = g.nWords; out[3] = g.nBins; out[4] = g.viewK; out[5] = g.bytes ? 1 : 0;
}

}  // extern "C"

// ============================================================================================ FP64 re-decision
// TEST INFRASTRUCTURE ONLY, like the rest of this file. The engine and this oracle decide every hit with one watertight
// float test (hit_tri), so they agree bit for bit; the functions below measure how far that shared decision lies from
// exact geometry. Each ray of a sample is decided twice: by the float code above (the engine's decision), and with every
// ray/triangle test and every per-hit rule (hemisphere cull, own plane, the 1/32 m and tmin bounds, the virtual ground's
// ray end) evaluated in double from the same float inputs (vertices, origin after offset_ray, direction, normal). Double
// rounding is 2^-29 of float's, so where the two differ the float decision is the one off exact geometry. A ray whose
// decisions differ is attributed to
//   edge       a triangle that the two tests hit differently, where the ray passes within edgeRel x (|o|max + t) of the
//              triangle's nearest edge (the ray's point on the triangle's plane, to the nearest point of its boundary);
//              the float test's rounding scales with the coordinates relative to the origin;
//   grazing    such a triangle met at |cos| < 0.05 (the reference's exclusion of grazing hits, validate/README.md:189);
//   threshold  no triangle hit differently, but a sign or threshold test of the rules decided differently (the reference
//              excludes rays within 1e-6 of a sign test and hits within 1 mm of the downward ray's end);
//   tie        (views) the same triangles hit in both, but the two nearest lie within 1e-5 of each other's distance, so
//              their order differs;
//   rounding   (views) the same triangle decides in both with the same class, but the float distance differs from the
//              double one by more than the reference's distance check (1e-5 t + 1e-4 m);
//   other      none of these (the tests require none).
namespace {

struct D3 { double x, y, z; };
inline D3 d3(F3 a) { return D3{a.x, a.y, a.z}; }
inline D3 dsub(D3 a, D3 b) { return D3{a.x - b.x, a.y - b.y, a.z - b.z}; }
inline D3 dadd(D3 a, D3 b) { return D3{a.x + b.x, a.y + b.y, a.z + b.z}; }
inline D3 dmul(double s, D3 a) { return D3{s * a.x, s * a.y, s * a.z}; }
inline double ddot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline D3 dcross(D3 a, D3 b) { return D3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline double dcomp(D3 a, int k) { return k == 0 ? a.x : k == 1 ? a.y : a.z; }
inline double dlen(D3 a) { return std::sqrt(ddot(a, a)); }

struct HitD { double t = 0, u = 0, v = 0; uint32_t prim = 0; bool front = false; };
// hit_tri's test in double: the same dominant axis and shear, edge functions, tie rule on exact zeros and t range
bool hit_tri_d(const Ray& rf, D3 o, D3 d, D3 v0, D3 v1, D3 v2, double tmin, double tmax, bool cullBack, HitD& h) {
  const int kx = rf.kx, ky = rf.ky, kz = rf.kz;
  const double dz = dcomp(d, kz), Sx = dcomp(d, kx) / dz, Sy = dcomp(d, ky) / dz, Sz = 1.0 / dz;
  const D3 A = dsub(v0, o), B = dsub(v1, o), C = dsub(v2, o);
  const double Ax = dcomp(A, kx) - Sx * dcomp(A, kz), Ay = dcomp(A, ky) - Sy * dcomp(A, kz);
  const double Bx = dcomp(B, kx) - Sx * dcomp(B, kz), By = dcomp(B, ky) - Sy * dcomp(B, kz);
  const double Cx = dcomp(C, kx) - Sx * dcomp(C, kz), Cy = dcomp(C, ky) - Sy * dcomp(C, kz);
  const double U = Cx * By - Cy * Bx, V = Ax * Cy - Ay * Cx, W = Bx * Ay - By * Ax;
  if ((U < 0 || V < 0 || W < 0) && (U > 0 || V > 0 || W > 0)) return false;
  const double det = U + V + W;
  if (det == 0) return false;
  if (cullBack && det < 0) return false;
  if (U == 0 || V == 0 || W == 0) {
    const double s = det > 0 ? 1 : -1;
    const auto owns = [](double ex, double ey) { return ey > 0 || (ey == 0 && ex > 0); };
    if (U == 0 && !owns(s * (Cx - Bx), s * (Cy - By))) return false;
    if (V == 0 && !owns(s * (Ax - Cx), s * (Ay - Cy))) return false;
    if (W == 0 && !owns(s * (Bx - Ax), s * (By - Ay))) return false;
  }
  const double t = (U * (Sz * dcomp(A, kz)) + V * (Sz * dcomp(B, kz)) + W * (Sz * dcomp(C, kz))) / det;
  if (!(t >= tmin && t <= tmax)) return false;
  h.t = t; h.u = V / det; h.v = W / det; h.front = det > 0;
  return true;
}
// own_hit's rules in double (trace_dev.cu:60-72): t (n.d) under 1/32 m, the hit within ext 2^-22 of the sensor's plane
// along the ray and the triangle's normal on the ray's side facing away from the sensor's
bool own_hit_d(D3 v0, D3 v1, D3 v2, const HitD& h, D3 d, D3 n, double* margin) {
  const D3 e1 = dsub(v1, v0), e2 = dsub(v2, v0), ng = dcross(e1, e2);
  const double l2 = ddot(ng, ng);
  const double a = h.t * ddot(n, d), lim1 = 1.0 / 32;
  double m = std::fabs(a - lim1) / lim1;
  bool ok = a < lim1 && l2 > 0;
  if (l2 > 0) {
    const D3 hn = dmul((h.front ? 1 : -1) / std::sqrt(l2), ng);
    const double ext = std::max({std::fabs(e1.x), std::fabs(e1.y), std::fabs(e1.z), std::fabs(e2.x), std::fabs(e2.y), std::fabs(e2.z)});
    const double lhs = h.t * std::fabs(ddot(d, hn)), rhs = ext * double(2.3841858e-7f), nh = ddot(n, hn);
    ok = ok && lhs < rhs && nh <= 0;
    m = std::min({m, std::fabs(lhs - rhs) / std::max(rhs, 1e-300), std::fabs(nh)});
  }
  if (margin) *margin = m;
  return ok;
}
// The ray's point on the triangle's plane, its distance to the triangle's boundary, and |cos| with the plane's normal.
void edge_metrics(D3 o, D3 d, D3 v0, D3 v1, D3 v2, double& dist, double& cosA, double& tPlane) {
  const D3 ng = dcross(dsub(v1, v0), dsub(v2, v0));
  const double ln = dlen(ng), dn = ddot(d, ng);
  cosA = ln > 0 ? std::fabs(dn) / (ln * dlen(d)) : 0;
  dist = 0; tPlane = 0;
  if (!(ln > 0) || dn == 0) return;
  tPlane = ddot(dsub(v0, o), ng) / dn;
  const D3 X = dadd(o, dmul(tPlane, d));
  const auto seg = [&](D3 a, D3 b) {
    const D3 ab = dsub(b, a);
    const double L = ddot(ab, ab), s = L > 0 ? std::clamp(ddot(dsub(X, a), ab) / L, 0.0, 1.0) : 0.0;
    return dlen(dsub(X, dadd(a, dmul(s, ab))));
  };
  dist = std::min({seg(v0, v1), seg(v1, v2), seg(v2, v0)});
}
// The triangles whose boxes the ray passes (every triangle the ray meets at t >= 0 is among them: the boxes are
// conservative, expanded by 2^-16 of the scene's largest coordinate).
template <class Fn>
void for_candidates(const Scene& s, const Ray& r, Fn&& f) {
  if (s.nodes.empty()) return;
  uint32_t stack[128];
  int sp = 0;
  stack[sp++] = 0;
  while (sp) {
    const Node& nd = s.nodes[stack[--sp]];
    if (!box_hit(nd, r, 0.f, INFINITY)) continue;
    if (nd.count) for (uint32_t j = nd.first; j < nd.first + nd.count; ++j) f(s.order[j]);
    else { stack[sp++] = nd.left; stack[sp++] = nd.right; }
  }
}

enum { kAgree = 0, kEdge = 1, kGrazing = 2, kThreshold = 3, kTie = 4, kRounding = 5, kOther = 6 };
struct Tally {   // what one sensor's rays add to the report (kgbo_recheck_*'s out[])
  double v[24] = {};
  void flip_metrics(double dist, double rel, double cosA) {
    const double edges[5] = {1e-7, 1e-6, 1e-5, 1e-4, 1e-3};
    int b = 0;
    while (b < 5 && dist >= edges[b]) ++b;
    v[8 + b] += 1;
    v[14 + (cosA < 0.05 ? 0 : cosA < 0.2 ? 1 : 2)] += 1;
    v[17] = std::max(v[17], dist);
    v[18] = std::max(v[18], rel);
  }
};
struct Tri3 { D3 a, b, c; };
Tri3 tri_d(const Scene& s, uint32_t k) { return Tri3{d3(s.v[s.tri[3 * k]]), d3(s.v[s.tri[3 * k + 1]]), d3(s.v[s.tri[3 * k + 2]])}; }
double omax(F3 o) { return std::max({std::fabs(o.x), std::fabs(o.y), std::fabs(o.z)}); }

// One visibility bit decided in float (visible_bit) and in double; the category of a difference.
int recheck_bit(const Engine& g, F3 o, F3 n, F3 dir, bool cull, double edgeRel, Tally& T) {
  const bool f = visible_bit(g, o, n, dir, cull);
  const D3 od = d3(o), dd = d3(dir), nd = d3(n);
  const double cd = ddot(nd, dd);
  const bool cullF = n.x * dir.x + n.y * dir.y + n.z * dir.z > 0.f;
  const Ray r = make_ray(o, dir);
  const double tmin = double(1e-5f);
  bool dvis = cd > 0;
  std::vector<uint32_t> cand;
  if (cullF || dvis) for_candidates(*g.sc, r, [&](uint32_t k) { cand.push_back(k); });
  if (dvis) {
    int own = 0;
    for (uint32_t k : cand) {
      const Tri3 t = tri_d(*g.sc, k);
      HitD h;
      if (!hit_tri_d(r, od, dd, t.a, t.b, t.c, tmin, INFINITY, cull, h)) continue;
      if (own_hit_d(t.a, t.b, t.c, h, dd, nd, nullptr) && ++own <= 3) continue;
      dvis = false;
      break;
    }
  }
  if (cullF) T.v[0] += 1;
  if (f == dvis) return kAgree;
  T.v[1] += 1;
  if ((cd > 0) != cullF) return kThreshold;   // the hemisphere's sign test
  // the triangles the two tests hit differently, and hits whose own-plane status differs
  double best = INFINITY, bestRel = INFINITY, bestCos = 1;
  bool member = false, thresh = false;
  for (uint32_t k : cand) {
    const Tri3 t = tri_d(*g.sc, k);
    const F3 a = g.sc->v[g.sc->tri[3 * k]], b = g.sc->v[g.sc->tri[3 * k + 1]], c = g.sc->v[g.sc->tri[3 * k + 2]];
    Hit hf;
    HitD hd;
    const bool fh = hit_tri(r, a, b, c, 1e-5f, INFINITY, cull, hf), dh = hit_tri_d(r, od, dd, t.a, t.b, t.c, tmin, INFINITY, cull, hd);
    if (fh != dh) {
      Hit x;
      HitD y;
      const bool fe = hit_tri(r, a, b, c, -INFINITY, INFINITY, cull, x), de = hit_tri_d(r, od, dd, t.a, t.b, t.c, -INFINITY, INFINITY, cull, y);
      if (fe == de) { thresh = true; continue; }   // the same edge decision: the t range's bound decided
      double dist, cosA, tp;
      edge_metrics(od, dd, t.a, t.b, t.c, dist, cosA, tp);
      const double rel = dist / (omax(o) + std::fabs(tp) + 1e-30);
      if (!member || rel < bestRel) { best = dist; bestRel = rel; bestCos = cosA; }
      member = true;
    } else if (fh) {
      hf.prim = k;
      const bool of = own_hit(*g.sc, hf, dir, n), od2 = own_hit_d(t.a, t.b, t.c, hd, dd, nd, nullptr);
      if (of != od2) thresh = true;
    }
  }
  if (member) {
    T.flip_metrics(best, bestRel, bestCos);
    if (bestCos < 0.05) return kGrazing;
    return bestRel <= edgeRel ? kEdge : kOther;
  }
  return thresh ? kThreshold : kOther;
}

// One view ray decided in float (view_ray) and in double: classes and distances; the category of a difference.
// out flags: bit 0 class differs, bit 1 distance differs (beyond 1e-5 t + 1e-4 m, the reference's distance check).
int recheck_view(const Engine& g, F3 o, F3 nn, F3 dir, bool none, bool cull, const kgb_view_in& v, double edgeRel, Tally& T) {
  uint8_t clF;
  float tF;
  view_ray(g, o, nn, dir, none, cull, v, clF, tF);
  if (clF == 254 || none) { T.v[0] += 1; return kAgree; }
  const D3 od = d3(o), dd = d3(dir), nd = d3(nn);
  T.v[0] += 1;
  if (v.cull && ((ddot(nd, dd) <= 0) != (dot(nn, dir) <= 0.f))) { T.v[1] += 1; T.v[19] += 1; return kThreshold; }
  if (v.vground && dir.z < 0.f && !(o.z > v.groundZ)) return kAgree;   // exact comparisons: the same in double
  const bool plane = v.vground && dir.z < 0.f;
  const double gz = v.groundZ;
  const double tg = plane ? (od.z - gz) / -dd.z : INFINITY;
  const double tmax = plane ? (od.z - gz + double(0.01f)) / -dd.z : double(FLT_MAX);
  const double tmin = double(1e-5f);
  const Ray r = make_ray(o, dir);
  std::vector<HitD> hits;
  std::vector<uint32_t> cand;
  for_candidates(*g.sc, r, [&](uint32_t k) { cand.push_back(k); });
  for (uint32_t k : cand) {
    const Tri3 t = tri_d(*g.sc, k);
    HitD h;
    if (hit_tri_d(r, od, dd, t.a, t.b, t.c, tmin, tmax, cull, h)) { h.prim = k; hits.push_back(h); }
  }
  std::sort(hits.begin(), hits.end(), [](const HitD& a, const HitD& b) { return a.t < b.t || (a.t == b.t && a.prim < b.prim); });
  uint8_t clD = 2;
  double tD = INFINITY;
  unsigned own = 0, panes = 0;
  double last = -INFINITY;
  uint32_t decider = ~0u;
  bool ended = false;
  for (const HitD& h : hits) {
    if (!(h.t > last)) continue;   // the float walk resumes past the hit's distance
    const Tri3 t = tri_d(*g.sc, h.prim);
    tD = h.t;
    last = h.t;
    decider = h.prim;
    if (own_hit_d(t.a, t.b, t.c, h, dd, nd, nullptr)) { if (++own == 4) { ended = true; break; } continue; }
    const uint8_t lb = g.label.empty() ? 2 : g.label[h.prim];
    if (lb != KGB_LABEL_PASS) { clD = lb; ended = true; break; }
    if (++panes > KGB_MAX_PANES) { ended = true; break; }
  }
  if (!ended) { clD = dir.z >= 0.f ? 0 : 1; tD = tg; decider = ~0u; }
  if (panes) clD |= KGB_VIEW_GLAZED;
  const bool clsDiff = clD != clF;
  if (!clsDiff && ended && tD > 0) T.v[21] = std::max(T.v[21], std::fabs(double(tF) - tD) / tD);
  const bool distDiff = !clsDiff && std::isfinite(tD) && std::fabs(double(tF) - tD) > 1e-5 * tD + 1e-4;
  if (!clsDiff && !distDiff) return kAgree;
  T.v[1] += 1;
  T.v[clsDiff ? 19 : 20] += 1;
  // the float walk's deciding hit
  uint32_t fDecider = ~0u;
  double tFd = 0;
  {
    float tmn = 1e-5f;
    unsigned ow = 0, pn = 0;
    const float tmaxF = plane ? (o.z - v.groundZ + 0.01f) / -dir.z : FLT_MAX;
    for (;;) {
      Hit hh;
      if (!closest(*g.sc, r, tmn, tmaxF, cull, hh)) break;
      fDecider = hh.prim; tFd = hh.t;
      if (own_hit(*g.sc, hh, dir, nn)) { if (++ow == 4) break; }
      else {
        const uint8_t lb = g.label.empty() ? 2 : g.label[hh.prim];
        if (lb != KGB_LABEL_PASS) break;
        if (++pn > KGB_MAX_PANES) break;
      }
      tmn = next_up(hh.t);
      fDecider = ~0u;
    }
  }
  // a deciding hit at the downward ray's end (1 cm below the ground plane): the reference's 1 mm exclusion
  const double tEnd = tmax;
  if (plane && ((decider != ~0u && std::fabs(tD - tEnd) * -dd.z < 1e-3) || (fDecider != ~0u && std::fabs(tFd - tEnd) * -dd.z < 1e-3)))
    return kThreshold;
  // the triangles that decided: did the two tests hit them differently?
  double best = INFINITY, bestRel = INFINITY, bestCos = 1;
  bool member = false;
  for (uint32_t k : {decider, fDecider}) {
    if (k == ~0u) continue;
    const Tri3 t = tri_d(*g.sc, k);
    const F3 a = g.sc->v[g.sc->tri[3 * k]], b = g.sc->v[g.sc->tri[3 * k + 1]], c = g.sc->v[g.sc->tri[3 * k + 2]];
    Hit hf;
    HitD hd;
    const bool fh = hit_tri(r, a, b, c, 1e-5f, plane ? (o.z - v.groundZ + 0.01f) / -dir.z : FLT_MAX, cull, hf);
    const bool dh = hit_tri_d(r, od, dd, t.a, t.b, t.c, tmin, tmax, cull, hd);
    if (fh == dh) continue;
    double dist, cosA, tp;
    edge_metrics(od, dd, t.a, t.b, t.c, dist, cosA, tp);
    const double rel = dist / (omax(o) + std::fabs(tp) + 1e-30);
    if (!member || rel < bestRel) { best = dist; bestRel = rel; bestCos = cosA; }
    member = true;
  }
  if (member) {
    T.flip_metrics(best, bestRel, bestCos);
    if (bestCos < 0.05) return kGrazing;
    return bestRel <= edgeRel ? kEdge : kOther;
  }
  // both deciding triangles hit in both precisions: the same triangle (the float distance's rounding), the order of
  // two close hits, or an own-plane rule decided differently
  if (decider == fDecider && !clsDiff) return decider != ~0u ? kRounding : kOther;
  if (decider != ~0u && fDecider != ~0u && decider != fDecider && std::fabs(tD - tFd) <= 1e-5 * std::max(tD, tFd)) return kTie;
  for (uint32_t k : {decider, fDecider}) {   // a deciding hit whose own-plane status differs
    if (k == ~0u) continue;
    const Tri3 t = tri_d(*g.sc, k);
    const F3 a = g.sc->v[g.sc->tri[3 * k]], b = g.sc->v[g.sc->tri[3 * k + 1]], c = g.sc->v[g.sc->tri[3 * k + 2]];
    Hit hf;
    HitD hd;
    if (hit_tri(r, a, b, c, 1e-5f, INFINITY, cull, hf) && hit_tri_d(r, od, dd, t.a, t.b, t.c, tmin, INFINITY, cull, hd)) {
      hf.prim = k;
      if (own_hit(*g.sc, hf, dir, nn) != own_hit_d(t.a, t.b, t.c, hd, dd, nd, nullptr)) return kThreshold;
    }
  }
  return kOther;
}

void tally_out(const std::vector<Tally>& per, const std::vector<int64_t>& firstOther, size_t i0, double* out) {
  for (int k = 0; k < 24; ++k) out[k] = 0;
  out[22] = out[23] = -1;
  for (size_t i = 0; i < per.size(); ++i) {
    for (int k = 0; k < 22; ++k) out[k] = (k == 17 || k == 18 || k == 21) ? std::max(out[k], per[i].v[k]) : out[k] + per[i].v[k];
    if (firstOther[i] >= 0 && out[22] < 0) { out[22] = double(i0 + i); out[23] = double(firstOther[i]); }
  }
}
}  // namespace

extern "C" {
// out[24] (doubles, summed over the chunk's rays): [0] rays traced (bits: past the hemisphere cull), [1] rays decided
// differently in double, of which [2] edge, [3] grazing, [4] threshold, [5] tie, [6] rounding, [7] other; [8..13] the
// nearest-edge distance of the differences with a triangle hit differently, bins < 1e-7, 1e-6, 1e-5, 1e-4, 1e-3,
// >= 1e-3 m; [14..16] their |cos|: < 0.05, < 0.2, >= 0.2; [17] the largest such distance (m), [18] the largest relative
// to |o|max + t; [19] class differences, [20] distance-only differences (views); [21] the largest relative difference
// between the float and the double distance over the rays whose class agrees and that end on a hit (views); [22], [23]
// sensor and direction of the first ray of category other (-1: none).
// Test-only: 0 switches refine_t off (the float walk's own distances), 1 back on; a test plants that error and checks
// that the FP64 re-decision catches it.
KGB_API void kgbo_set_refine(int on) { g_refine = on != 0; }

KGB_API int kgbo_recheck_bits(kgb_engine* e, size_t i0, size_t nc, uint32_t rayFlags, double edgeRel, double* out) {
  Engine& g = *reinterpret_cast<Engine*>(e);
  if (i0 + nc > g.nSensors) return fail("kgbo_recheck_bits: sensor range exceeds the scene");
  const bool cull = (rayFlags & KGB_RAY_CULL_BACK_FACING) != 0;
  std::vector<Tally> per(nc);
  std::vector<int64_t> firstOther(nc, -1);
  par_for(nc, [&](size_t i) {
    const F3 n = g.N[i0 + i], o = offset_ray(g.P[i0 + i], n);
    for (size_t d = 0; d < g.nDir; ++d) {
      const int c = recheck_bit(g, o, n, g.D[d], cull, edgeRel, per[i]);
      if (c) per[i].v[1 + c] += 1;
      if (c == kOther && firstOther[i] < 0) firstOther[i] = int64_t(d);
    }
  });
  tally_out(per, firstOther, i0, out);
  return 1;
}

KGB_API int kgbo_recheck_view(kgb_engine* e, size_t i0, size_t nc, uint32_t rayFlags, const kgb_view_in* v, double edgeRel, double* out) {
  Engine& g = *reinterpret_cast<Engine*>(e);
  if (i0 + nc > g.nSensors) return fail("kgbo_recheck_view: sensor range exceeds the scene");
  const size_t K = size_t(v->nAz) * v->nEl;
  const bool cull = (rayFlags & KGB_RAY_CULL_BACK_FACING) != 0;
  const double rad = v->north * KGB_PI_D / 180;
  const float cosN = float(std::cos(rad)), sinN = float(std::sin(rad));
  std::vector<float> rs(v->rowSin, v->rowSin + 2 * size_t(v->nEl));
  std::vector<Tally> per(nc);
  std::vector<int64_t> firstOther(nc, -1);
  par_for(nc, [&](size_t i) {
    const unsigned gi = unsigned(i0 + i), element = gi / v->nS, side = v->nS == 2 ? gi % 2 : unsigned(v->back != 0);
    const F3 nn = g.N[i0 + i], o = offset_ray(g.P[i0 + i], nn);
    const bool none = !(dot(nn, nn) > 0.f);
    F3 f, r, u;
    view_frame(nn, v->world != 0, cosN, sinN, f, r, u);
    for (size_t d = 0; d < K; ++d) {
      const unsigned col = unsigned(d % v->nAz), row = unsigned(d / v->nAz);
      const F3 l = view_cell(unsigned(d), col, rs[2 * row], rs[2 * row + 1], v->az0, v->dAz, v->jitter != 0, element, side);
      const F3 dir = add(add(mul(l.x, r), mul(l.y, f)), mul(l.z, u));
      const int c = recheck_view(g, o, nn, dir, none, cull, *v, edgeRel, per[i]);
      if (c) per[i].v[1 + c] += 1;
      if (c == kOther && firstOther[i] < 0) firstOther[i] = int64_t(d);
    }
  });
  tally_out(per, firstOther, i0, out);
  return 1;
}
}  // extern "C"
