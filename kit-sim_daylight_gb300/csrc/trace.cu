// Ray-casting kernels of the engine (compiled with -fmad=false: see rt.cuh):
//  k_bits   visibility bits, any-hit (replaces the reference's __raygen__bits, trace_dev.cu:91-108)
//  k_bytes  transmittance bytes (replaces __raygen__bytes + __anyhit__tr, trace_dev.cu:115-165)
//  k_view   class + distance of the closest hit per view cell (replaces __raygen__view, trace_dev.cu:177-232)
//  k_bounce_paths, k_bounce_step, k_bounce_accum
//           reflected-light paths binned by sky patch (replaces __raygen__bounce, trace_dev.cu:260-311), as a wavefront
//           of segments: first segments, then steps over a compacted queue of the paths that go on
// The visibility kernels are persistent: each warp takes tasks of 32 consecutive sensors x one 32-direction word
// from a global counter, so a warp traces one direction for 32 neighbouring sensors at a time (coherent rays). k_bits
// and k_bytes take a call's sensors in the engine's tracing order (grouped by the orientation of their normals:
// TraceArgs::order), so that a warp's sensors face the same way more often; each result goes to its sensor's column.
#include "engine.h"
#include "rt.cuh"

namespace kgb {

// The sensor (scene index) at lane position i of a launch and its output column (see TraceArgs::order).
__device__ __forceinline__ void task_sensor(const TraceArgs& a, uint32_t i, uint32_t& gi, uint32_t& col) {
  if (!a.order) { gi = a.first + i; col = a.out0 + i; return; }
  const uint32_t p = a.p0 + i;
  uint32_t g = a.pieceG[0];   // the runs' ends do not decrease: the last one passed names the run
  if (p >= a.pieceEnd[0]) g = a.pieceG[1];
  if (p >= a.pieceEnd[1]) g = a.pieceG[2];
  if (p >= a.pieceEnd[2]) g = a.pieceG[3];
  if (p >= a.pieceEnd[3]) g = a.pieceG[4];
  if (p >= a.pieceEnd[4]) g = a.pieceG[5];
  gi = a.order[g + p];
  col = gi - a.callI0;
}

__device__ __forceinline__ uint32_t next_task(uint32_t* counter) {
  uint32_t t = 0;
  if ((threadIdx.x & 31) == 0) t = atomicAdd(counter, 1u);
  return __shfl_sync(~0u, t, 0);
}

// ---------------------------------------------------------------------------------------------------- bits
// Direction d of a sensor is visible when n.d > 0 and every hit from tmin 1e-5 on is an own-plane hit, at most 3.
// COUNT: the instrumented variant (same results) that adds up nodes visited, triangles tested and rays traced.
template <bool COUNT>
__global__ void __launch_bounds__(256) k_bits(TraceArgs a) {
  const Scene s{a.nodes, a.tris, a.nNodes};
  const bool cull = (a.rayFlags & KGB_RAY_CULL_BACK_FACING) != 0;
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t blocks = (a.n + 31) / 32, nTasks = blocks * a.nWords;
  uint32_t overflow = 0;
  Count ctr;
  uint32_t rays = 0;
  for (uint32_t task = next_task(a.counter); task < nTasks; task = next_task(a.counter)) {
    const uint32_t b = task / a.nWords, w = task % a.nWords, i = b * 32 + lane;
    if (i >= a.n) continue;
    uint32_t gi, col;
    task_sensor(a, i, gi, col);
    const F3 n = ld3(a.N + 3 * gi), o = offset_ray(ld3(a.P + 3 * gi), n);
    const uint32_t word = trace_word<COUNT>(s, n, o, a.D, a.rayTab, a.nDir, w, cull, overflow, ctr, rays);
    a.bits[size_t(w) * a.stride + col] = word;
  }
  if (overflow) atomicOr(a.status, (overflow & 1u ? kStatusStackOverflow : 0u) | (overflow & 2u ? kStatusVisitLimit : 0u));
  if (COUNT) {
    unsigned long long* c = reinterpret_cast<unsigned long long*>(a.status + 1);   // ctl words 2..7: three u64 counters
    atomicAdd(c, (unsigned long long)ctr.nodes);
    atomicAdd(c + 1, (unsigned long long)ctr.tris);
    atomicAdd(c + 2, (unsigned long long)rays);
  }
}

// ---------------------------------------------------------------------------------------------------- bytes
// A translucent slot's crossing: tau, 1 on a thin solid's exit face, Radiance glass T(cos) (trace_dev.cu:147-165).
__device__ __forceinline__ float crossing(const kgb_slot* slots, const float2* slotLog, uint32_t nSlots, uint32_t slot, bool front, F3 v0, F3 v1,
                                         F3 v2, F3 d) {
  const kgb_slot sl = slot < nSlots ? slots[slot] : kgb_slot{0.2f, 0.f, 0.f, 0u};
  float T = sl.tau;
  if ((sl.flags & KGB_SLOT_THIN) && front == ((sl.flags & KGB_SLOT_INWARD) != 0)) T = 1.f;
  else if (sl.flags & KGB_SLOT_GLASS) {
    const float ax = v1.x - v0.x, ay = v1.y - v0.y, az = v1.z - v0.z;
    const float bx = v2.x - v0.x, by = v2.y - v0.y, bz = v2.z - v0.z;
    const float nx = ay * bz - az * by, ny = az * bx - ax * bz, nz = ax * by - ay * bx;
    float R;
    glass_TR(fabsf(nx * d.x + ny * d.y + nz * d.z) * (1.f / sqrtf(nx * nx + ny * ny + nz * nz)), sl.tn, slotLog[slot], T, R);
  }
  return T;
}

constexpr int kMaxCross = 16;   // translucent crossings a ray keeps in registers before it walks them in order instead

// Own-plane hits pass (at most 3), an opaque hit blocks, translucent crossings multiply in (t, primitive) order.
// d: the direction's index, whose precomputed ray part (a.rayTab, when set) gives the ray make_ray would.
__device__ uint8_t trace_byte(const Scene& s, const TraceArgs& a, F3 o, F3 n, uint32_t d, F3 dir, bool cull, uint32_t& overflow) {
  if (!(n.x * dir.x + n.y * dir.y + n.z * dir.z > 0.f)) return 0;
  const Ray r = a.rayTab ? ray_from(a.rayTab, d, o) : make_ray(o, dir);
  bool blocked = false, spill = false;
  int own = 0, nx = 0;
  float ct[kMaxCross], cf[kMaxCross];
  uint32_t cp[kMaxCross];
  for_hits<false, true>(s, r, 1e-5f, INFINITY, cull, [&](const Hit& h, F3 v0, F3 v1, F3 v2, uint32_t flags, uint32_t slot) {
    if (own_hit(v0, v1, v2, h, dir, n)) { if (++own <= 3) return false; blocked = true; return true; }
    if (!(flags & kTriTranslucent)) { blocked = true; return true; }
    if (nx < kMaxCross) { ct[nx] = h.t; cp[nx] = h.prim; cf[nx] = crossing(a.slots, a.slotLog, a.nSlots, slot, h.front, v0, v1, v2, dir); ++nx; }
    else spill = true;
    return false;
  }, overflow);
  if (blocked) return 0;
  float T = 1.f;
  if (!spill) {
    for (int x = 1; x < nx; ++x) {   // insertion sort by (t, primitive)
      const float tx = ct[x], fx = cf[x];
      const uint32_t px = cp[x];
      int y = x - 1;
      while (y >= 0 && (ct[y] > tx || (ct[y] == tx && cp[y] > px))) { ct[y + 1] = ct[y]; cp[y + 1] = cp[y]; cf[y + 1] = cf[y]; --y; }
      ct[y + 1] = tx; cp[y + 1] = px; cf[y + 1] = fx;
    }
    for (int x = 0; x < nx; ++x) {
      T *= cf[x];
      if (!(T >= 1.f / 510.f)) return 0;
    }
    return (uint8_t)__float2uint_rn(T * 255.f);
  }
  // more than kMaxCross crossings: walk them one at a time in (t, primitive) order
  float lastT = -INFINITY;
  uint32_t lastP = 0;
  for (;;) {
    bool found = false;
    float bt = 0.f, bf = 0.f;
    uint32_t bp = 0;
    for_hits<false, true>(s, r, 1e-5f, INFINITY, cull, [&](const Hit& h, F3 v0, F3 v1, F3 v2, uint32_t flags, uint32_t slot) {
      if (!(flags & kTriTranslucent) || own_hit(v0, v1, v2, h, dir, n)) return false;
      if (h.t < lastT || (h.t == lastT && h.prim <= lastP)) return false;
      if (!found || h.t < bt || (h.t == bt && h.prim < bp)) {
        found = true; bt = h.t; bp = h.prim;
        bf = crossing(a.slots, a.slotLog, a.nSlots, slot, h.front, v0, v1, v2, dir);
      }
      return false;
    }, overflow);
    if (!found) break;
    T *= bf;
    if (!(T >= 1.f / 510.f)) return 0;
    lastT = bt; lastP = bp;
  }
  return (uint8_t)__float2uint_rn(T * 255.f);
}

__global__ void __launch_bounds__(256, 3) k_bytes(TraceArgs a) {   // 3 blocks an SM: 21.3 ms for a precision chunk, 24.6 at 2 (no spills)
  const Scene s{a.nodes, a.tris, a.nNodes};
  const bool cull = (a.rayFlags & KGB_RAY_CULL_BACK_FACING) != 0;
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t blocks = (a.n + 31) / 32, nTasks = blocks * a.nWords;
  uint32_t overflow = 0;
  for (uint32_t task = next_task(a.counter); task < nTasks; task = next_task(a.counter)) {
    const uint32_t b = task / a.nWords, w = task % a.nWords, i = b * 32 + lane;
    if (i >= a.n) continue;
    uint32_t gi, col;
    task_sensor(a, i, gi, col);
    const F3 n = ld3(a.N + 3 * gi), o = offset_ray(ld3(a.P + 3 * gi), n);
    for (uint32_t k = 0; k < 32; ++k) {
      const uint32_t d = w * 32 + k;
      if (d >= a.nDir) break;
      a.bytes[size_t(d) * a.stride + col] = trace_byte(s, a, o, n, d, ld3(a.D + 3 * d), cull, overflow);
    }
  }
  if (overflow) atomicOr(a.status, (overflow & 1u ? kStatusStackOverflow : 0u) | (overflow & 2u ? kStatusVisitLimit : 0u));
}

// ---------------------------------------------------------------------------------------------------- views
// params.h:77-89 (view_cell), sincospif as kgb_sincospi
__device__ __forceinline__ F3 view_cell(uint32_t d, uint32_t col, float rsx, float rsy, float az0, float dAz, bool jitter, uint32_t element, uint32_t side) {
  float a = 0.5f, s = 0.5f * (rsx + rsy);
  if (jitter) { const U3 h = pcg3d(element, d, side); a = u01(h.x); s = rsx + u01(h.y) * (rsy - rsx); }
  float sa, ca;
  kgb_sincospi((az0 + (float(col) + a) * dAz) * (1.f / 180.f), &sa, &ca);
  const float c = sqrtf(fmaxf(0.f, 1.f - s * s));
  return f3(c * sa, c * ca, s);
}

// The reported distance of the hit that ended a view ray. The watertight test's t = T / det rounds with the vertices'
// coordinates relative to the origin, so a triangle whose vertices lie far beyond the hit (a kilometre-long ground quad
// seen from 100 m) gives t off by up to 1e-3 relative. Where a vertex lies more than 4 t from the origin along an axis
// (in float), t is recomputed from the triangle's plane in double, float(dot(v0 - o, ng)) / float(dot(d, ng)) with
// ng = (v1 - v0) x (v2 - v0): the differences and products of float coordinates are exact or within 2^-52 in double,
// so the result lies within 2 ulps of the exact distance. About 9 % of the views city's hits take this path, and every
// distance then lies within 3.2e-6 of a double-precision walk's. The walk (which hits, their order, the own-plane
// rules) keeps the float t; the oracle's view_ray applies the same rule with the same operations.
__device__ __noinline__ float refine_t(F3 o, F3 d, F3 v0, F3 v1, F3 v2, float t) {
  const float reach = fmaxf(fmaxf(fmaxf(fabsf(v0.x - o.x), fabsf(v0.y - o.y)), fmaxf(fabsf(v0.z - o.z), fabsf(v1.x - o.x))),
                            fmaxf(fmaxf(fmaxf(fabsf(v1.y - o.y), fabsf(v1.z - o.z)), fmaxf(fabsf(v2.x - o.x), fabsf(v2.y - o.y))), fabsf(v2.z - o.z)));
  if (!(reach > 4.f * t)) return t;
  const double ex = double(v1.x) - double(v0.x), ey = double(v1.y) - double(v0.y), ez = double(v1.z) - double(v0.z);
  const double fx = double(v2.x) - double(v0.x), fy = double(v2.y) - double(v0.y), fz = double(v2.z) - double(v0.z);
  const double nx = ey * fz - ez * fy, ny = ez * fx - ex * fz, nz = ex * fy - ey * fx;
  const double num = ((double(v0.x) - double(o.x)) * nx + (double(v0.y) - double(o.y)) * ny) + (double(v0.z) - double(o.z)) * nz;
  const double den = (double(d.x) * nx + double(d.y) * ny) + double(d.z) * nz;
  const float r = __fdiv_rn(__double2float_rn(num), __double2float_rn(den));
  return r > 0.f && r < __int_as_float(0x7f800000) ? r : t;
}

__global__ void __launch_bounds__(256, 3) k_view(ViewArgs a) {   // 3 blocks an SM: more warps to hide latency beat the few spills
  const Scene s{a.nodes, a.tris, a.nNodes};
  const bool cull = (a.rayFlags & KGB_RAY_CULL_BACK_FACING) != 0;
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t blocks = (a.n + 31) / 32, nTasks = blocks * a.nWords;
  const float inf = __int_as_float(0x7f800000);
  uint32_t overflow = 0;
  for (uint32_t task = next_task(a.counter); task < nTasks; task = next_task(a.counter)) {
    const uint32_t b = task / a.nWords, w = task % a.nWords, i = b * 32 + lane;
    if (i >= a.n) continue;
    const uint32_t gl = a.first + i;           // sensor within the engine's arrays
    const uint32_t gi = a.i0 + a.out0 + i;     // global sensor index (seeds)
    const uint32_t element = gi / a.nS, side = a.nS == 2 ? gi % 2 : a.back;
    const F3 n = ld3(a.N + 3 * gl), o = offset_ray(ld3(a.P + 3 * gl), n);
    const bool none = !(dot(n, n) > 0.f);
    F3 f, r, u;
    if (a.world) { f = f3(-a.sinN, a.cosN, 0.f); r = f3(a.cosN, a.sinN, 0.f); u = f3(0.f, 0.f, 1.f); }
    else {
      const float l = sqrtf(n.x * n.x + n.y * n.y);
      f = n;
      if (l > 1e-3f) r = f3(n.y / l, -n.x / l, 0.f);
      else {
        r = f3(a.cosN, a.sinN, 0.f);
        if (l > 0.f) { r = sub(r, mul(dot(r, n), n)); r = mul(1.f / sqrtf(dot(r, r)), r); }
      }
      u = f3(r.y * f.z - r.z * f.y, r.z * f.x - r.x * f.z, r.x * f.y - r.y * f.x);
    }
    for (uint32_t k = 0; k < 32; ++k) {
      const uint32_t d = w * 32 + k;
      if (d >= a.K) break;
      const uint32_t col = d % a.nAz, row = d / a.nAz;
      const F3 l = view_cell(d, col, a.rowSin[2 * row], a.rowSin[2 * row + 1], a.az0, a.dAz, a.jitter != 0, element, side);
      const F3 dir = add(add(mul(l.x, r), mul(l.y, f)), mul(l.z, u));
      uint32_t cl = 2;
      float t = inf;
      if (none || (a.cull && dot(n, dir) <= 0.f)) cl = 254;
      else if (a.vground && dir.z < 0.f && !(o.z > a.groundZ)) { cl = 1; t = 0.1f; }
      else {
        const bool plane = a.vground && dir.z < 0.f;
        const float tg = plane ? (o.z - a.groundZ) / -dir.z : inf;
        const float tmax = plane ? (o.z - a.groundZ + 0.01f) / -dir.z : FLT_MAX;
        float tmin = 1e-5f;
        uint32_t own = 0, panes = 0;
        const Ray ray = make_ray(o, dir);
        ClosestOut c;
        bool byHit = false;   // the walk ended on a hit (not past the last one)
        for (;;) {
          if (!closest(s, ray, tmin, tmax, cull, c, overflow)) { cl = dir.z >= 0.f ? 0 : 1; t = tg; break; }
          t = c.h.t;
          if (own_hit(c.v0, c.v1, c.v2, c.h, dir, n)) { if (++own == 4) { byHit = true; break; } }
          else {
            const uint32_t lb = a.label ? a.label[c.h.prim] : 2u;
            if (lb != KGB_LABEL_PASS) { cl = lb; byHit = true; break; }
            if (++panes > KGB_MAX_PANES) { byHit = true; break; }
          }
          tmin = next_up(t);
        }
        if (byHit) t = refine_t(o, dir, c.v0, c.v1, c.v2, t);
        if (panes) cl |= KGB_VIEW_GLAZED;
      }
      const size_t at = size_t(d) * a.stride + a.out0 + i;
      a.cls[at] = uint8_t(cl);
      a.dist[at] = t;
    }
  }
  if (overflow) atomicOr(a.status, (overflow & 1u ? kStatusStackOverflow : 0u) | (overflow & 2u ? kStatusVisitLimit : 0u));
}

// ---------------------------------------------------------------------------------------------------- bounce
__device__ __forceinline__ F3 cosine_dir(F3 n, float u, float v) {   // trace_dev.cu:235-242 (Duff et al. 2017 basis)
  const float sg = copysignf(1.f, n.z), a = -1.f / (sg + n.z), b = n.x * n.y * a;
  const F3 t = f3(1.f + sg * n.x * n.x * a, sg * b, -sg * n.x), w = f3(b, sg + n.y * n.y * a, -n.y);
  float s, c;
  kgb_sincospi(2.f * v, &s, &c);
  const float r = sqrtf(u);
  return add(add(mul(r * c, t), mul(r * s, w)), mul(sqrtf(fmaxf(0.f, 1.f - u)), n));
}
__constant__ uint32_t kTnaz[7] = {30, 30, 24, 24, 18, 12, 6};
__device__ __forceinline__ uint32_t sky_bin(F3 d, uint32_t mf, uint32_t nBins, float alpha, float cosN, float sinN) {   // trace_dev.cu:248-258
  if (!(d.z >= 0.f)) return 0;
  const uint32_t r = min(uint32_t(kgb_asin(fminf(d.z, 1.f)) / alpha), 7 * mf);
  if (r == 7 * mf) return nBins - 1;
  const uint32_t n = kTnaz[r / mf] * mf;
  uint32_t b = 1 + (r % mf) * n;
  for (uint32_t q = 0; q < r / mf; ++q) b += kTnaz[q] * mf * mf;
  float az = kgb_atan2(d.x * cosN + d.y * sinN, d.y * cosN - d.x * sinN);
  if (az < 0.f) az += 6.28318531f;
  return b + uint32_t(az * (float(n) / 6.28318531f) + .5f) % n;
}

constexpr uint32_t kNoBin = 0xffffffffu;

// A path between segments (48 bytes): where it is, where it goes, its weight and counters.
struct __align__(16) PathState {
  float ox, oy, oz;
  uint32_t gi;       // global sensor index
  float dx, dy, dz;
  uint32_t smp;      // sample
  float w;
  uint32_t k;        // random-number counter
  uint32_t bits;     // diffuse reflections (bits 0-7), reflected (bit 8), segments done (bits 16-31)
  uint32_t at;       // its result's index: contrib[(sample - s0) n + i]
};

// One segment of a path: the body of the reference's per-sample loop (trace_dev.cu:260-311). Returns true when the path
// goes on (o, d, w, k, diffuse, reflected updated), false when it has ended (bin and gain set if it escaped after a
// reflection). nn: the sensor's normal, read on the first segment only.
__device__ __forceinline__ bool bounce_segment(const BounceArgs& a, const Scene& s, bool cull, uint32_t seg, F3 nn, uint32_t gi, uint32_t smp, F3& o,
                                               F3& d, float& w, uint32_t& k, uint32_t& diffuse, bool& reflected, uint32_t& bin, float& gain,
                                               uint32_t& overflow) {
  ClosestOut c;
  const bool found = closest<true>(s, make_ray(o, d), 1e-5f, FLT_MAX, cull, c, overflow);
  if (overflow & 2u) {   // the walk gave up: the first such path leaves its ray for the error message
    uint32_t* diag = a.status + 15;   // ctl words 16..
    if (atomicCAS(diag, 0u, 1u) == 0u) {
      diag[1] = gi; diag[2] = smp; diag[3] = seg;
      diag[4] = __float_as_uint(o.x); diag[5] = __float_as_uint(o.y); diag[6] = __float_as_uint(o.z);
      diag[7] = __float_as_uint(d.x); diag[8] = __float_as_uint(d.y); diag[9] = __float_as_uint(d.z);
    }
    return false;
  }
  if (!found) {
    if (reflected) { bin = sky_bin(d, a.mf, a.nBins, a.alpha, a.cosN, a.sinN); gain = w * (3.14159265f / float(a.M)); }
    return false;
  }
  const kgb_slot sl = c.slot < a.nSlots ? a.slots[c.slot] : kgb_slot{0.2f, 0.f, 0.f, 0u};
  TriHit h;
  if (!tri_geom(c.v0, c.v1, c.v2, c.h, h)) return false;
  if (seg == 0 && own_plane(h, c.h.t, d, nn)) { o = through(h); return true; }
  if ((sl.flags & (KGB_SLOT_THIN | KGB_SLOT_TWIN)) == KGB_SLOT_THIN && h.front == ((sl.flags & KGB_SLOT_INWARD) != 0)) { o = through(h); return true; }
  const bool mirror = (sl.flags & KGB_SLOT_GLASS) != 0;
  float T = sl.tau, R = sl.rho;
  if (mirror) { glass_TR(fabsf(dot(d, h.n)), sl.tn, a.slotLog[c.slot], T, R); if (!(sl.tau > 0.f)) T = 0.f; }
  else if (diffuse == a.nBounce) R = 0.f;
  if (!(T + R > 0.f)) return false;
  const U3 rr = pcg3d(gi, smp, k++);
  w *= T + R;
  if (u01(rr.x) * (T + R) < T) { o = through(h); return true; }
  reflected = true;
  if (mirror) d = sub(d, mul(2.f * dot(d, h.n), h.n));
  else {
    d = cosine_dir(h.n, u01(rr.y), u01(rr.z));
    if (++diffuse >= 2) {
      if (u01(pcg3d(gi, smp, k++).x) >= w) return false;
      w = 1.f;
    }
  }
  o = add(offset_ray(h.p, h.n), h.lift);
  return true;
}

// The warp's paths that go on, appended to the queue in lane order with one atomic per warp.
__device__ __forceinline__ void enqueue(bool go, const PathState& st, PathState* q, uint32_t* count) {
  const uint32_t lane = threadIdx.x & 31, act = __activemask(), m = __ballot_sync(act, go);
  if (!m) return;
  const uint32_t leader = __ffs(act) - 1;
  uint32_t base = 0;
  if (lane == leader) base = atomicAdd(count, __popc(m));
  base = __shfl_sync(act, base, leader);
  if (go) q[base + __popc(m & ((1u << lane) - 1u))] = st;
}

// One mask for the sum and its leader: two reads of __activemask() may see different sets of converged lanes.
__device__ __forceinline__ void add_segments(const BounceArgs& a, uint32_t segments) {
  const uint32_t m = __activemask();
  const uint32_t sum = __reduce_add_sync(m, segments);
  if ((threadIdx.x & 31) == __ffs(m) - 1) atomicAdd(reinterpret_cast<unsigned long long*>(a.status + 1), (unsigned long long)sum);
}

// Paths as a wavefront: k_bounce_paths traces every path's first segment, one thread a path; with a.order, sensor
// i = t / S and sample a.order[t % S] (S = s1 - s0): a warp's 32 paths start at one sensor and the order (the host sorts
// the launch's samples by their first direction before the per-sensor rotation) keeps their first directions in a
// narrow cone, so their walks share nodes; without it sensor i = t % n, sample s0 + t / n. The paths that go on are
// compacted into a queue, and k_bounce_step runs one more segment of each queued path, at most nBounce + 15 times, so
// a warp's lanes stay busy whatever the lengths of its paths. A path's segments are the reference's loop body in order
// with its own counters, so where and when it runs changes no result. A path that ends leaves its sky bin (where it
// escaped after a reflection, or none) and contribution (w x pi / M) in contrib[(sample - s0) n + i]; k_bounce_accum
// adds them to each sensor's rows in sample order, as the reference's per-sensor loop over samples does.
__global__ void __launch_bounds__(128) k_bounce_paths(BounceArgs a) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t S = a.s1 - a.s0;
  if (t >= a.n * S) return;
  const uint32_t i = a.order ? t / S : t % a.n, smp = a.order ? a.order[t % S] : a.s0 + t / a.n;
  const Scene s{a.nodes, a.tris, a.nNodes};
  const bool cull = (a.rayFlags & KGB_RAY_CULL_BACK_FACING) != 0;
  const uint32_t gi = a.i0 + i;
  const F3 nn = ld3(a.N + 3 * gi);
  F3 o = offset_ray(ld3(a.P + 3 * gi), nn);
  const U3 rot = pcg3d(gi, ~0u, ~0u);
  const float r0 = u01(rot.x), r1 = u01(rot.y);
  const float u = float(smp) / float(a.M) + r0, v = u01(__brev(smp)) + r1;
  F3 d = cosine_dir(nn, u - floorf(u), v - floorf(v));
  float w = 1.f, gain = 0.f;
  uint32_t k = 0, diffuse = 0, bin = kNoBin, overflow = 0;
  bool reflected = false;
  const uint32_t at = (smp - a.s0) * a.n + i;
  const bool go = bounce_segment(a, s, cull, 0, nn, gi, smp, o, d, w, k, diffuse, reflected, bin, gain, overflow) && a.nBounce + 16 > 1;
  PathState st;
  if (go) {
    st.ox = o.x; st.oy = o.y; st.oz = o.z; st.gi = gi; st.dx = d.x; st.dy = d.y; st.dz = d.z; st.smp = smp;
    st.w = w; st.k = k; st.bits = diffuse | (reflected ? 0x100u : 0u) | (1u << 16); st.at = at;
  } else {
    a.contrib[at] = make_uint2(bin, __float_as_uint(gain));
  }
  enqueue(go, st, a.qOut, a.qOutCount);
  add_segments(a, 1u);
  if (overflow) atomicOr(a.status, (overflow & 1u ? kStatusStackOverflow : 0u) | (overflow & 2u ? kStatusVisitLimit : 0u));
}

// One more segment of each path in the queue (grid-stride); the ones that go on into the next queue.
__global__ void __launch_bounds__(128) k_bounce_step(BounceArgs a) {
  const Scene s{a.nodes, a.tris, a.nNodes};
  const bool cull = (a.rayFlags & KGB_RAY_CULL_BACK_FACING) != 0;
  const uint32_t count = *a.qInCount, stride = gridDim.x * blockDim.x;
  uint32_t overflow = 0, segments = 0;
  const uint64_t start = clock_ns();
  bool late = false;
  for (uint32_t q0 = blockIdx.x * blockDim.x; q0 < count; q0 += stride) {   // whole warps in step: enqueue is warp-wide
    const uint32_t qi = q0 + threadIdx.x;
    const bool mine = qi < count;
    PathState st{};
    bool go = false;
    if (mine && !late && clock_ns() - start >= a.limitNs) late = true;
    if (mine && late) {   // past the limit: the path ends with no contribution, and the call fails
      a.contrib[a.qIn[qi].at] = make_uint2(kNoBin, 0u);
    } else if (mine) {
      st = a.qIn[qi];
      F3 o = f3(st.ox, st.oy, st.oz), d = f3(st.dx, st.dy, st.dz);
      float w = st.w, gain = 0.f;
      uint32_t k = st.k, diffuse = st.bits & 0xffu, bin = kNoBin;
      bool reflected = (st.bits & 0x100u) != 0;
      const uint32_t seg = st.bits >> 16;
      go = bounce_segment(a, s, cull, seg, f3(0.f, 0.f, 0.f), st.gi, st.smp, o, d, w, k, diffuse, reflected, bin, gain, overflow) &&
           seg + 1 < a.nBounce + 16;
      ++segments;
      if (go) {
        st.ox = o.x; st.oy = o.y; st.oz = o.z; st.dx = d.x; st.dy = d.y; st.dz = d.z; st.w = w; st.k = k;
        st.bits = diffuse | (reflected ? 0x100u : 0u) | ((seg + 1) << 16);
      } else {
        a.contrib[st.at] = make_uint2(bin, __float_as_uint(gain));
      }
    }
    enqueue(go, st, a.qOut, a.qOutCount);
  }
  add_segments(a, segments);
  if (overflow || late)
    atomicOr(a.status, (overflow & 1u ? kStatusStackOverflow : 0u) | (overflow & 2u ? kStatusVisitLimit : 0u) | (late ? kStatusTimeout : 0u));
}

// Per sensor, the launch's samples in order: row[bin] = row[bin] + contribution (the reference's float additions).
__global__ void __launch_bounds__(256) k_bounce_accum(BounceArgs a) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  float* row = a.dc + i;
  for (uint32_t q = 0; q < a.s1 - a.s0; ++q) {
    const uint2 c = a.contrib[size_t(q) * a.n + i];
    if (c.x != kNoBin) { float* p = row + size_t(c.x) * a.nc; *p = *p + __uint_as_float(c.y); }
  }
}

// ---------------------------------------------------------------------------------------------------- launches
__global__ void __launch_bounds__(256) k_ray_table(const float* D, uint32_t nDir, RayDir* tab) {
  const uint32_t d = blockIdx.x * blockDim.x + threadIdx.x;
  if (d < nDir) tab[d] = ray_dir_of(ld3(D + 3 * d));
}
// A sensor's orientation class: twice the dominant axis of its normal (x 0, y 1, z 2), plus one when that component is
// positive.
__global__ void k_sensor_classes(const float* N, uint32_t n, uint8_t* cls, uint32_t* flags) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t c = 6;   // no sensor
  if (i < n) {
    const float x = N[3 * i], y = N[3 * i + 1], z = N[3 * i + 2];
    const float ax = fabsf(x), ay = fabsf(y), az = fabsf(z);
    const uint32_t k = (ax >= ay && ax >= az) ? 0u : (ay >= az ? 1u : 2u);
    c = 2u * k + ((k == 0 ? x : k == 1 ? y : z) > 0.f ? 1u : 0u);
    if (cls[i] != c) { cls[i] = uint8_t(c); atomicOr(flags, 1u); }
  }
  for (uint32_t k = 0; k < 6; ++k) {   // counts, one atomic per warp and class
    const uint32_t m = __ballot_sync(~0u, c == k);
    if ((threadIdx.x & 31) == 0 && m) atomicAdd(flags + 1 + k, uint32_t(__popc(m)));
  }
}
void launch_sensor_classes(const float* N, uint32_t n, uint8_t* cls, uint32_t* flags, cudaStream_t st) {
  if (n) k_sensor_classes<<<(n + 255) / 256, 256, 0, st>>>(N, n, cls, flags);
}

void launch_ray_table(const float* D, uint32_t nDir, void* tab, cudaStream_t st) {
  if (nDir) k_ray_table<<<(nDir + 255) / 256, 256, 0, st>>>(D, nDir, static_cast<RayDir*>(tab));
}
int bytes_blocks_per_sm() {   // resident blocks of k_bytes per SM
  int b = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_bytes, 256, 0) != cudaSuccess || b < 1) b = 1;
  return b;
}
int view_blocks_per_sm() {   // resident blocks of k_view per SM
  int b = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_view, 256, 0) != cudaSuccess || b < 1) b = 1;
  return b;
}
int bits_blocks_per_sm() {   // resident blocks of k_bits per SM (its persistent grid fills the GPU once)
  int b = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_bits<false>, 256, 0) != cudaSuccess || b < 1) b = 1;
  return b;
}
void launch_bits(const TraceArgs& a, int grid, cudaStream_t st, bool count) {
  if (count) k_bits<true><<<grid, 256, 0, st>>>(a);
  else k_bits<false><<<grid, 256, 0, st>>>(a);
}
void launch_bytes(const TraceArgs& a, int grid, cudaStream_t st) { k_bytes<<<grid, 256, 0, st>>>(a); }
void launch_view(const ViewArgs& a, int grid, cudaStream_t st) { k_view<<<grid, 256, 0, st>>>(a); }
// ln tn of each slot as a float pair (glass_TR's logarithm, once per slot; kgb_ln_pair, as kgb_powf takes it)
__global__ void k_slot_logs(const kgb_slot* slots, uint32_t n, float2* out) {
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  float h = 0.f, l = 0.f;
  if (slots[s].tn > 0.f) kgb_ln_pair(slots[s].tn, &h, &l);
  out[s] = make_float2(h, l);
}
void launch_slot_logs(const kgb_slot* slots, uint32_t n, float2* out, cudaStream_t st) {
  if (n) k_slot_logs<<<(n + 127) / 128, 128, 0, st>>>(slots, n, out);
}

// The first segments, then up to nBounce + 15 steps over the queue of paths that go on (two queues in turn; a step
// over an empty queue does nothing), then the accumulation. qCount: two counters; queues: two of n (s1 - s0) paths.
void launch_bounce(const BounceArgs& args, PathState* queues, uint32_t* qCount, int stepGrid, cudaStream_t st) {
  BounceArgs a = args;
  const size_t paths = size_t(a.n) * (a.s1 - a.s0);
  a.qOut = queues; a.qOutCount = qCount;
  cudaMemsetAsync(qCount, 0, 8, st);
  k_bounce_paths<<<unsigned((paths + 127) / 128), 128, 0, st>>>(a);
  for (uint32_t step = 1; step < a.nBounce + 16; ++step) {
    const int in = int((step + 1) & 1);   // the queue the previous launch filled
    a.qIn = queues + size_t(in) * paths; a.qInCount = qCount + in;
    a.qOut = queues + size_t(in ^ 1) * paths; a.qOutCount = qCount + (in ^ 1);
    cudaMemsetAsync(a.qOutCount, 0, 4, st);
    k_bounce_step<<<stepGrid, 128, 0, st>>>(a);
  }
  k_bounce_accum<<<(a.n + 255) / 256, 256, 0, st>>>(a);
}
size_t bounce_state_bytes() { return sizeof(PathState); }
int bounce_step_blocks_per_sm() {   // resident blocks of k_bounce_step per SM (its grid-stride grid fills the GPU once)
  int b = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_bounce_step, 128, 0) != cudaSuccess || b < 1) b = 1;
  return b;
}

}  // namespace kgb
