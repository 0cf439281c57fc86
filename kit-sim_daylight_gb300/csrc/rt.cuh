// Device-side ray casting of the engine: the watertight ray/triangle test, the 8-wide BVH traversal
// (any-hit and closest-hit), and the reference's per-hit rules (own planes, glass, offsets, hashes).
//
// Numerics contract: the code deciding a result (hit or miss, t, own plane, transmittance byte, direction cell, sky
// bin) is a fixed sequence of IEEE-754 float operations: this header is compiled with -fmad=false and divisions /
// square roots are the correctly rounded ones, so the results equal a host restatement compiled without contraction
// bit for bit. Box tests only filter: they are conservative (boxes expanded at build, see bvh_build.cpp) and may use
// fused operations.
#pragma once
#include <cfloat>
#include <cstdint>
#include "kgb_detmath.h"
#include "kitsim_gb300.h"
#include "engine.h"

namespace kgb {

// ------------------------------------------------------------------------------------------------ data layout (HBM)
// BVH8 node, 208 bytes = 13 x 16 B:
//   n0: childBase | imask << 24 (childBase: index of the node's first inner child, below 2^24; its inner children are
//       consecutive in slot order; imask bit k: child k is an inner node), triBase (index of the node's first
//       triangle record), meta[8] (leaf child k: count << 5 | offset of its triangles from triBase, below 128; 0: empty
//       slot); bit 7 of meta[0], meta[1], meta[2] holds bit 0, 1, 2 of slots - 1 (slots: 1 + the last slot in use, so
//       these bits fall on slots in use only)
//   n1 n2: lo.x of children 0..3, 4..7 (float)   n3 n4: hi.x
//   n5 n6: lo.y                                  n7 n8: hi.y
//   n9 n10: lo.z                                 n11 n12: hi.z
//   (an empty slot holds lo = +inf, hi = -inf, which no ray enters)
// The child boxes are plain floats: the box test reads a ray's near and far planes straight from the two vectors its
// octant picks (Ray::nearX..: n1 or n3 for x; the far one is the index ^ 2), with no decoding. (The 80-byte form
// with 8-bit child boxes of Ylitie, Karras and Laine 2017 spent most of the box test's instructions decoding bytes:
// the test is 87 % of the any-hit walk's instructions.)
// Triangle record, 48 bytes = 3 x 16 B: v0.xyz + primitive index | v1.xyz + flags | v2.xyz + slot.
struct __align__(16) Node8 { uint4 n[kNodeWords / 4]; };
static_assert(sizeof(Node8) == 4 * kNodeWords, "node record size");
struct __align__(16) TriRec { float4 a, b, c; };
enum : uint32_t { kTriTranslucent = 1u };   // TriRec.b.w flag bits: the slot transmitted at build (any-hit)

struct F3 { float x, y, z; };
__device__ __forceinline__ F3 f3(float x, float y, float z) { return F3{x, y, z}; }
__device__ __forceinline__ F3 add(F3 a, F3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ F3 sub(F3 a, F3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ F3 mul(float s, F3 a) { return f3(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ float dot(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float comp(F3 a, int k) { return k == 0 ? a.x : k == 1 ? a.y : a.z; }
__device__ __forceinline__ F3 ld3(const float* p) { return f3(p[0], p[1], p[2]); }
__device__ __forceinline__ float next_up(float t) { return __uint_as_float(__float_as_uint(t) + 1u); }

// Waechter & Binder 2019 (Ray Tracing Gems, ch. 6), as the reference's offset_ray (trace_dev.cu:16-25).
__device__ __forceinline__ F3 offset_ray(F3 p, F3 n) {
  const float origin = 1.f / 32.f, floatScale = 1.f / 65536.f, intScale = 256.f;
  const int ox = int(intScale * n.x), oy = int(intScale * n.y), oz = int(intScale * n.z);
  const float px = __int_as_float(__float_as_int(p.x) + (p.x < 0.f ? -ox : ox));
  const float py = __int_as_float(__float_as_int(p.y) + (p.y < 0.f ? -oy : oy));
  const float pz = __int_as_float(__float_as_int(p.z) + (p.z < 0.f ? -oz : oz));
  return f3(fabsf(p.x) < origin ? p.x + floatScale * n.x : px, fabsf(p.y) < origin ? p.y + floatScale * n.y : py,
            fabsf(p.z) < origin ? p.z + floatScale * n.z : pz);
}

// Jarzynski & Olano 2020 (JCGT 9(3)): the reference's pcg3d / u01 (params.h:64-71).
struct U3 { uint32_t x, y, z; };
__device__ __forceinline__ U3 pcg3d(uint32_t x, uint32_t y, uint32_t z) {
  x = x * 1664525u + 1013904223u; y = y * 1664525u + 1013904223u; z = z * 1664525u + 1013904223u;
  x += y * z; y += z * x; z += x * y;
  x ^= x >> 16; y ^= y >> 16; z ^= z >> 16;
  x += y * z; y += z * x; z += x * y;
  return U3{x, y, z};
}
__device__ __forceinline__ float u01(uint32_t v) { return float(v >> 8) * (1.f / 16777216.f); }

// Radiance glass (the reference's glass_TR, glass.h:17-25; rad5R4 m_glass.c), powf as kgb_powf. lnTn: the slot's ln tn
// as a float pair (kgb_ln_pair, computed once per slot by k_slot_logs), so tn^(1 / c2) = kgb_pow_ln(lnTn, 1 / c2) is
// kgb_powf's value bit for bit, in float arithmetic only.
__device__ __forceinline__ void glass_TR(float c, float tn, float2 lnTn, float& T, float& R) {
  const float n = 1.52f;
  const float c2 = sqrtf((1.f - 1.f / (n * n)) + c * c / (n * n));
  const float d = tn > 0.f ? kgb_pow_ln(lnTn.x, lnTn.y, 1.f / c2) : 0.f, d2 = d * d;
  float rs = (c - n * c2) / (c + n * c2), rp = (c2 - n * c) / (c2 + n * c);
  rs *= rs; rp *= rp;
  T = .5f * (1.f - rs) * (1.f - rs) * d / (1.f - rs * rs * d2) + .5f * (1.f - rp) * (1.f - rp) * d / (1.f - rp * rp * d2);
  R = .5f * rs * (1.f + (1.f - 2.f * rs) * d2) / (1.f - rs * rs * d2) + .5f * rp * (1.f + (1.f - 2.f * rp) * d2) / (1.f - rp * rp * d2);
}

// x >= 0 as a double, exactly, without the FP64 pipe for a normal float: the exponent rebiased (+896) and the
// mantissa moved up 29 bits by integer operations (zero and subnormals take the conversion instruction).
__device__ __forceinline__ double widen(float x) {
  const uint32_t b = __float_as_uint(x);
  return x >= 1.17549435e-38f ? __hiloint2double(int((b >> 3) + (896u << 20)), int(b << 29)) : (double)x;
}

// ------------------------------------------------------------------------------------------------ the ray
struct Ray {
  F3 o, d;
  int kx, ky, kz;
  float Sx, Sy, Sz;
  F3 inv;     // box test: 1 / d with zero components replaced by +-2^-80
  F3 oinv;    // o * inv
  uint32_t oct;   // sign bits of d (closest-hit child order)
  uint32_t nearX, nearY, nearZ;   // node vectors of the near planes per axis (lo if inv >= 0, else hi); far: ^ 2
};
__device__ __forceinline__ void near_planes(Ray& r) {
  r.nearX = r.inv.x < 0.f ? 3u : 1u;
  r.nearY = r.inv.y < 0.f ? 7u : 5u;
  r.nearZ = r.inv.z < 0.f ? 11u : 9u;
}
__device__ __forceinline__ Ray make_ray(F3 o, F3 d) {
  Ray r;
  r.o = o; r.d = d;
  const float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
  r.kz = ax >= ay ? (ax >= az ? 0 : 2) : (ay >= az ? 1 : 2);
  r.kx = r.kz == 2 ? 0 : r.kz + 1;
  r.ky = r.kx == 2 ? 0 : r.kx + 1;
  if (comp(d, r.kz) < 0.f) { const int t = r.kx; r.kx = r.ky; r.ky = t; }
  const float dz = comp(d, r.kz);
  r.Sx = comp(d, r.kx) / dz;
  r.Sy = comp(d, r.ky) / dz;
  r.Sz = 1.f / dz;
  const float tiny = 8.27180613e-25f;   // 2^-80
  const float dx = ax > tiny ? d.x : copysignf(tiny, d.x), dy = ay > tiny ? d.y : copysignf(tiny, d.y), dzz = az > tiny ? d.z : copysignf(tiny, d.z);
  r.inv = f3(1.f / dx, 1.f / dy, 1.f / dzz);
  r.oinv = f3(o.x * r.inv.x, o.y * r.inv.y, o.z * r.inv.z);
  r.oct = (d.x < 0.f ? 1u : 0u) | (d.y < 0.f ? 2u : 0u) | (d.z < 0.f ? 4u : 0u);
  near_planes(r);
  return r;
}

// The direction-only part of a ray (everything but the origin), 48 bytes, computed once per direction table by
// make_ray itself: a = d.xyz, Sx | b = inv.xyz, Sy | c = Sz, kx | ky << 8 | kz << 16 | oct << 24, 0, 0.
struct __align__(16) RayDir { float4 a, b, c; };
__device__ __forceinline__ RayDir ray_dir_of(F3 d) {
  const Ray r = make_ray(f3(0.f, 0.f, 0.f), d);
  RayDir t;
  t.a = make_float4(r.d.x, r.d.y, r.d.z, r.Sx);
  t.b = make_float4(r.inv.x, r.inv.y, r.inv.z, r.Sy);
  t.c = make_float4(r.Sz, __uint_as_float(uint32_t(r.kx) | uint32_t(r.ky) << 8 | uint32_t(r.kz) << 16 | r.oct << 24), 0.f, 0.f);
  return t;
}
// make_ray(o, d) from direction d's precomputed part: the same values, with o * inv the only arithmetic.
__device__ __forceinline__ Ray ray_from(const RayDir* tab, uint32_t d, F3 o) {
  const float4 a = __ldg(&tab[d].a), b = __ldg(&tab[d].b), c = __ldg(&tab[d].c);
  Ray r;
  r.o = o; r.d = f3(a.x, a.y, a.z);
  const uint32_t k = __float_as_uint(c.y);
  r.kx = int(k & 0xffu); r.ky = int((k >> 8) & 0xffu); r.kz = int((k >> 16) & 0xffu); r.oct = k >> 24;
  r.Sx = a.w; r.Sy = b.w; r.Sz = c.x;
  r.inv = f3(b.x, b.y, b.z);
  r.oinv = f3(o.x * r.inv.x, o.y * r.inv.y, o.z * r.inv.z);
  near_planes(r);
  return r;
}

struct Hit { float t, u, v; uint32_t prim; bool front; };

// Woop, Benthin, Wald 2013 (JCGT 2(1)) with a tie rule on edges: the same operation sequence as the oracle's hit_tri.
__device__ __forceinline__ bool hit_tri(const Ray& r, F3 v0, F3 v1, F3 v2, float tmin, float tmax, bool cullBack, Hit& h) {
  const F3 A = sub(v0, r.o), B = sub(v1, r.o), C = sub(v2, r.o);
  const float Akz = comp(A, r.kz), Bkz = comp(B, r.kz), Ckz = comp(C, r.kz);
  const float Ax = comp(A, r.kx) - r.Sx * Akz, Ay = comp(A, r.ky) - r.Sy * Akz;
  const float Bx = comp(B, r.kx) - r.Sx * Bkz, By = comp(B, r.ky) - r.Sy * Bkz;
  const float Cx = comp(C, r.kx) - r.Sx * Ckz, Cy = comp(C, r.ky) - r.Sy * Ckz;
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
    if (U == 0.f) { const float ex = s * (Cx - Bx), ey = s * (Cy - By); if (!(ey > 0.f || (ey == 0.f && ex > 0.f))) return false; }
    if (V == 0.f) { const float ex = s * (Ax - Cx), ey = s * (Ay - Cy); if (!(ey > 0.f || (ey == 0.f && ex > 0.f))) return false; }
    if (W == 0.f) { const float ex = s * (Bx - Ax), ey = s * (By - Ay); if (!(ey > 0.f || (ey == 0.f && ex > 0.f))) return false; }
  }
  const float Az = r.Sz * Akz, Bz = r.Sz * Bkz, Cz = r.Sz * Ckz;
  const float T = U * Az + V * Bz + W * Cz;
  const float t = T / det;
  if (!(t >= tmin && t <= tmax)) return false;
  h.t = t; h.u = V / det; h.v = W / det; h.front = det > 0.f;
  return true;
}

// The reference's hit_triangle (trace_dev.cu:37-52): point, unit normal on the ray's side (1/sqrt), ext, lift.
struct TriHit { F3 p, n, lift; float ext; bool front; };
__device__ __forceinline__ bool tri_geom(F3 v0, F3 v1, F3 v2, const Hit& hh, TriHit& h) {
  const F3 e1 = sub(v1, v0), e2 = sub(v2, v0);
  const F3 ng = f3(e1.y * e2.z - e1.z * e2.y, e1.z * e2.x - e1.x * e2.z, e1.x * e2.y - e1.y * e2.x);
  const float l2 = dot(ng, ng);
  if (!(l2 > 0.f)) return false;
  const float inv = 1.f / sqrtf(l2);
  h.front = hh.front;
  h.n = mul(h.front ? inv : -inv, ng);
  h.p = add(add(v0, mul(hh.u, e1)), mul(hh.v, e2));
  h.ext = fmaxf(fmaxf(fmaxf(fabsf(e1.x), fabsf(e1.y)), fmaxf(fabsf(e1.z), fabsf(e2.x))), fmaxf(fabsf(e2.y), fabsf(e2.z)));
  h.lift = mul(h.ext * 9.5367432e-7f, h.n);
  return true;
}
// own_plane / own_hit / through (trace_dev.cu:60-72, 63)
__device__ __forceinline__ bool own_plane(const TriHit& h, float t, F3 d, F3 n) {
  return t * fabsf(dot(d, h.n)) < h.ext * 2.3841858e-7f && dot(n, h.n) <= 0.f;
}
__device__ __forceinline__ bool own_hit(F3 v0, F3 v1, F3 v2, const Hit& hh, F3 d, F3 n) {
  if (!(hh.t * dot(n, d) < 1.f / 32.f)) return false;
  TriHit h;
  return tri_geom(v0, v1, v2, hh, h) && own_plane(h, hh.t, d, n);
}
__device__ __forceinline__ F3 through(const TriHit& h) { return sub(offset_ray(h.p, mul(-1.f, h.n)), h.lift); }

// ------------------------------------------------------------------------------------------------ BVH8 traversal
__device__ __forceinline__ uint32_t byte_of(uint32_t w, int k) { return (w >> (8 * k)) & 0xffu; }

// The helpers below hold inline PTX; their host branches (plain C++, the same values) let tests and tools compile
// this header for the CPU.
__device__ __forceinline__ float max3f(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
  float r;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
#else
  return fmaxf(fmaxf(a, b), c);
#endif
}
__device__ __forceinline__ float min3f(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
  float r;
  asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
#else
  return fminf(fminf(a, b), c);
#endif
}

// Two floats in one 64-bit register pair, for the packed FP32 instructions (add / mul / fma .f32x2, sm_100 and
// later): each half is rounded exactly as the scalar instruction rounds it.
__device__ __forceinline__ unsigned long long pk2(float a, float b) {
#if defined(__CUDA_ARCH__)
  unsigned long long r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
  return r;
#else
  return (unsigned long long)__float_as_uint(a) | ((unsigned long long)__float_as_uint(b) << 32);
#endif
}
__device__ __forceinline__ void up2(unsigned long long r, float& a, float& b) {
#if defined(__CUDA_ARCH__)
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(r));
#else
  a = __uint_as_float(uint32_t(r)); b = __uint_as_float(uint32_t(r >> 32));
#endif
}
__device__ __forceinline__ unsigned long long fma2(unsigned long long a, unsigned long long b, unsigned long long c) {
#if defined(__CUDA_ARCH__)
  unsigned long long r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
  return r;
#else
  float a0, a1, b0, b1, c0, c1;
  up2(a, a0, a1); up2(b, b0, b1); up2(c, c0, c1);
  return pk2(fmaf(a0, b0, c0), fmaf(a1, b1, c1));
#endif
}
__device__ __forceinline__ unsigned long long mul2(unsigned long long a, unsigned long long b) {
#if defined(__CUDA_ARCH__)
  unsigned long long r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
#else
  float a0, a1, b0, b1;
  up2(a, a0, a1); up2(b, b0, b1);
  return pk2(a0 * b0, a1 * b1);
#endif
}
// Two words as one packed pair (the low word first).
__device__ __forceinline__ unsigned long long pku(uint32_t a, uint32_t b) {
#if defined(__CUDA_ARCH__)
  unsigned long long r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "r"(a), "r"(b));
  return r;
#else
  return (unsigned long long)a | ((unsigned long long)b << 32);
#endif
}

// Child boxes of the node at p against the ray in [tmin, tmax] (tmin >= 0): returns the mask of hit children (bit k),
// their entry distances in tn[8]. Per axis the slab distance of a plane is fma(plane, inv, -o inv); the near planes
// are the low ones when inv >= 0, else the high ones, and the ray's nearX.. index picks their vector (the far one is
// the other). Children go in pairs through the packed fma: per pair one fma.f32x2 per plane, per child one 3-input max
// and one 3-input min. Conservative: the triangle boxes were expanded at build by 2^-16 of the scene's largest
// coordinate, far beyond the rounding of these distances, and the exit distance is widened by 2^-20 besides. Empty
// child slots (lo +inf, hi -inf) fail the test; a leaf slot without triangles that passes tests nothing.
// CLIP: the exit is also clipped at tmax (closest hit, where tmax shrinks to the best hit). Without it boxes beyond
// tmax pass as well, which is conservative: the triangle test applies tmax (the any-hit walks run to infinity).
// 1 + the node's last slot in use, from bit 7 of its first three meta bytes (the word of meta[0..3]).
__device__ __forceinline__ uint32_t node_slots(uint32_t meta03) {
  return 1u + (((meta03 >> 7) & 1u) | ((meta03 >> 14) & 2u) | ((meta03 >> 21) & 4u));
}

// SKIP: slots past the node's last child (empty boxes, which fail the test anyway) are neither read nor tested. The
// byte-mode trace and the bounce's walks run faster with it (10.5 against 9.8 G rays/s, 1283 against 1200 M paths/s);
// the visibility bits' walk and the views' closest hits run slower (the extra branches cost more than the tests they
// save: 64.9 against 61.0 ms for the urban trace), so those test every slot.
template <bool CLIP = true, bool SKIP = false>
__device__ __forceinline__ uint32_t node_hits(const uint4* p, const Ray& r, float tmin, float tmax, uint32_t slots, float* tn) {
  const unsigned long long IX = pk2(r.inv.x, r.inv.x), IY = pk2(r.inv.y, r.inv.y), IZ = pk2(r.inv.z, r.inv.z);
  const unsigned long long OX = pk2(-r.oinv.x, -r.oinv.x), OY = pk2(-r.oinv.y, -r.oinv.y), OZ = pk2(-r.oinv.z, -r.oinv.z);
  const unsigned long long WIDEN = pk2(1.00000095367431640625f, 1.00000095367431640625f);
  const uint32_t fX = r.nearX ^ 2u, fY = r.nearY ^ 2u, fZ = r.nearZ ^ 2u;
  uint32_t mask = 0;
#pragma unroll
  for (int h = 0; h < 2; ++h) {   // children 4h .. 4h + 3: the second vector of each plane set
    if (SKIP && 4 * h >= int(slots)) break;
    const uint4 nx = __ldg(p + r.nearX + h), fx = __ldg(p + fX + h);
    const uint4 ny = __ldg(p + r.nearY + h), fy = __ldg(p + fY + h);
    const uint4 nz = __ldg(p + r.nearZ + h), fz = __ldg(p + fZ + h);
#pragma unroll
    for (int j = 0; j < 2; ++j) {   // the pair 4h + 2j, 4h + 2j + 1
      const int k = 4 * h + 2 * j;
      if (SKIP && k >= int(slots)) break;
      float tnx[2], tny[2], tnz[2], tfx[2], tfy[2], tfz[2];
      up2(fma2(j ? pku(nx.z, nx.w) : pku(nx.x, nx.y), IX, OX), tnx[0], tnx[1]);
      up2(fma2(j ? pku(fx.z, fx.w) : pku(fx.x, fx.y), IX, OX), tfx[0], tfx[1]);
      up2(fma2(j ? pku(ny.z, ny.w) : pku(ny.x, ny.y), IY, OY), tny[0], tny[1]);
      up2(fma2(j ? pku(fy.z, fy.w) : pku(fy.x, fy.y), IY, OY), tfy[0], tfy[1]);
      up2(fma2(j ? pku(nz.z, nz.w) : pku(nz.x, nz.y), IZ, OZ), tnz[0], tnz[1]);
      up2(fma2(j ? pku(fz.z, fz.w) : pku(fz.x, fz.y), IZ, OZ), tfz[0], tfz[1]);
      // exit widened to tfar (1 + 2^-20): for tfar >= 0 the value fma(|tfar|, 2^-20, tfar), and a negative tfar fails
      // against tnear >= tmin >= 0 either way
      float tf[2];
      up2(mul2(pk2(min3f(tfx[0], tfy[0], tfz[0]), min3f(tfx[1], tfy[1], tfz[1])), WIDEN), tf[0], tf[1]);
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        const float tnear = max3f(tnx[e], tny[e], fmaxf(tnz[e], tmin));
        const float tfar = CLIP ? fminf(tf[e], tmax) : tf[e];
        if (tnear <= tfar) { mask |= 1u << (k + e); tn[k + e] = tnear; }
      }
    }
  }
  return mask;
}

__device__ __forceinline__ void load_tri(const TriRec* tris, uint32_t j, F3& v0, F3& v1, F3& v2, uint32_t& prim, uint32_t& flags, uint32_t& slot) {
  const float4* p = reinterpret_cast<const float4*>(tris + j);
  const float4 a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2);
  v0 = f3(a.x, a.y, a.z); v1 = f3(b.x, b.y, b.z); v2 = f3(c.x, c.y, c.z);
  prim = __float_as_uint(a.w); flags = __float_as_uint(b.w); slot = __float_as_uint(c.w);
}

struct Scene {
  const Node8* nodes;
  const TriRec* tris;
  uint32_t nNodes;    // 0: empty scene, every ray misses
};

// the GPU's nanosecond clock (kernels with a wall-time limit read it)
__device__ __forceinline__ uint64_t clock_ns() {
#if defined(__CUDA_ARCH__)
  uint64_t t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
#else
  return 0;
#endif
}

constexpr int kStack = 48;   // node-group stack entries (one per level at most)
// Node visits of one query past which the traversal gives up (overflow bit 2): a query visits a node of a tree at
// most once, so more than the node count (or 2^20) means a damaged walk; it ends at once instead of running on.
constexpr uint32_t kMaxVisits = 1u << 20;
__device__ __forceinline__ uint32_t visit_cap(const Scene& s) { return min(kMaxVisits, s.nNodes + 8u); }

// Traversal counters of the instrumented kernels (nodes visited, triangles tested); compiled out otherwise.
struct Count {
  uint32_t nodes = 0, tris = 0;
};

// Visit every triangle hit in [tmin, tmax] (any order); f(hit, v0, v1, v2, flags, slot) returns true to stop.
template <bool COUNT = false, bool SKIP = false, class Fn>
__device__ __forceinline__ void for_hits(const Scene& s, const Ray& r, float tmin, float tmax, bool cull, Fn&& f, uint32_t& overflow,
                                         Count* ctr = nullptr) {
  if (!s.nNodes) return;
  uint2 stack[kStack];   // node group: x = childBase, y = imask << 8 | remaining inner children
  int sp = 0;
  uint32_t cur = 0;      // node to visit
  const uint32_t cap = visit_cap(s);
  for (uint32_t visits = 0;; ++visits) {
    if (visits >= cap || cur >= s.nNodes) { overflow |= 2u; return; }
    const uint4* np = reinterpret_cast<const uint4*>(s.nodes + cur);
    const uint4 hd = __ldg(np);
    if (COUNT) ctr->nodes++;
    float tn[8];
    const uint32_t hit = node_hits<false, SKIP>(np, r, tmin, tmax, SKIP ? node_slots(hd.z) : 8u, tn);
    const uint32_t imask = hd.x >> 24, childBase = hd.x & 0xffffffu;
    uint32_t leaves = hit & ~imask;
    while (leaves) {
      const int k = __ffs(leaves) - 1;
      leaves &= leaves - 1;
      const uint32_t meta = byte_of(k < 4 ? hd.z : hd.w, k & 3);
      const uint32_t first = hd.y + (meta & 31u), cnt = (meta >> 5) & 3u;
      for (uint32_t j = first; j < first + cnt; ++j) {
        F3 v0, v1, v2;
        uint32_t prim, flags, slot;
        load_tri(s.tris, j, v0, v1, v2, prim, flags, slot);
        if (COUNT) ctr->tris++;
        Hit h;
        if (hit_tri(r, v0, v1, v2, tmin, tmax, cull, h)) {
          h.prim = prim;
          if (f(h, v0, v1, v2, flags, slot)) return;
        }
      }
    }
    const uint32_t inner = hit & imask;
    if (inner) {
      const int k = __ffs(inner) - 1;
      const uint32_t rest = inner & (inner - 1);
      if (rest) {
        if (sp < kStack) stack[sp++] = make_uint2(childBase, (imask << 8) | rest);
        else overflow = 1;
      }
      cur = childBase + __popc(imask & ((1u << k) - 1u));
      continue;
    }
    if (!sp) return;
    uint2& g = stack[sp - 1];
    const uint32_t rem = g.y & 0xffu, im = g.y >> 8;
    const int k = __ffs(rem) - 1;
    cur = g.x + __popc(im & ((1u << k) - 1u));
    const uint32_t left = rem & (rem - 1);
    if (left) g.y = (im << 8) | left; else --sp;
  }
}

// The closest hit in [tmin, tmax], ties broken by the smaller primitive index. Children are visited near to far: the
// nearest inner child next, the others pushed far to near; a node whose entry lies beyond the best hit so far is
// skipped. The visiting order changes nothing but the work: the result is the closest hit of the whole hit set.
struct ClosestOut { Hit h; F3 v0, v1, v2; uint32_t flags, slot; };
template <bool SKIP = false>
__device__ __forceinline__ bool closest(const Scene& s, const Ray& r, float tmin, float tmax, bool cull, ClosestOut& out, uint32_t& overflow) {
  if (!s.nNodes) return false;
  struct Entry { uint32_t node; float t; };
  Entry stack[kStack * 4];
  int sp = 0;
  bool any = false;
  float best = tmax;
  uint32_t cur = 0, visits = 0;
  const uint32_t cap = visit_cap(s);
  for (;;) {
    if (++visits > cap || cur >= s.nNodes) { overflow |= 2u; return any; }
    const uint4* np = reinterpret_cast<const uint4*>(s.nodes + cur);
    const uint4 hd = __ldg(np);
    float tn[8];
    const uint32_t hit = node_hits<true, SKIP>(np, r, tmin, best, SKIP ? node_slots(hd.z) : 8u, tn);
    const uint32_t imask = hd.x >> 24, childBase = hd.x & 0xffffffu;
    uint32_t leaves = hit & ~imask;
    while (leaves) {
      const int k = __ffs(leaves) - 1;
      leaves &= leaves - 1;
      const uint32_t meta = byte_of(k < 4 ? hd.z : hd.w, k & 3);
      const uint32_t first = hd.y + (meta & 31u), cnt = (meta >> 5) & 3u;
      for (uint32_t j = first; j < first + cnt; ++j) {
        F3 v0, v1, v2;
        uint32_t prim, flags, slot;
        load_tri(s.tris, j, v0, v1, v2, prim, flags, slot);
        Hit h;
        if (hit_tri(r, v0, v1, v2, tmin, best, cull, h)) {
          h.prim = prim;
          if (!any || h.t < out.h.t || (h.t == out.h.t && prim < out.h.prim)) {
            out.h = h; out.v0 = v0; out.v1 = v1; out.v2 = v2; out.flags = flags; out.slot = slot;
            any = true;
            best = h.t;
          }
        }
      }
    }
    // inner children still in front of the best hit, sorted far to near: the nearest is visited next
    uint32_t inner = hit & imask;
    Entry ch[8];
    int m = 0;
    while (inner) {
      const int k = __ffs(inner) - 1;
      inner &= inner - 1;
      if (tn[k] > best) continue;
      const Entry x{childBase + __popc(imask & ((1u << k) - 1u)), tn[k]};
      int b = m - 1;
      while (b >= 0 && ch[b].t < x.t) { ch[b + 1] = ch[b]; --b; }
      ch[b + 1] = x;
      ++m;
    }
    if (m) {
      if (sp + m - 1 > kStack * 4) { overflow |= 1u; m = 1; }
      for (int a = 0; a < m - 1; ++a) stack[sp++] = ch[a];
      cur = ch[m - 1].node;
      continue;
    }
    for (;;) {   // the next pushed node still in front of the best hit
      if (!sp) return any;
      const Entry e = stack[--sp];
      if (e.t <= best) { cur = e.node; break; }
    }
  }
}

// One visibility word: bit k = direction w*32+k of a sensor (normal n, ray origin o) passes the hemisphere cull and every
// hit from tmin 1e-5 on is an own-plane hit, at most 3 (the reference's __raygen__bits, trace_dev.cu:91-108, restated
// over the ray's hit set). COUNT adds traversal counters and rays traced.
// tab: the directions' precomputed RayDir entries, or null (the rays are made from D).
template <bool COUNT>
__device__ __forceinline__ uint32_t trace_word(const Scene& s, F3 n, F3 o, const float* D, const RayDir* tab, uint32_t nDir, uint32_t w, bool cull,
                                               uint32_t& overflow, Count& ctr, uint32_t& rays) {
  uint32_t word = 0;
  for (uint32_t k = 0; k < 32; ++k) {
    const uint32_t d = w * 32 + k;
    if (d >= nDir) break;
    const F3 dir = ld3(D + 3 * d);
    if (!(n.x * dir.x + n.y * dir.y + n.z * dir.z > 0.f)) continue;
    const Ray r = tab ? ray_from(tab, d, o) : make_ray(o, dir);
    bool blocked = false;
    int own = 0;
    if (COUNT) ++rays;
    for_hits<COUNT>(s, r, 1e-5f, INFINITY, cull, [&](const Hit& h, F3 v0, F3 v1, F3 v2, uint32_t, uint32_t) {
      if (own_hit(v0, v1, v2, h, dir, n) && ++own <= 3) return false;
      blocked = true;
      return true;
    }, overflow, &ctr);
    if (!blocked) word |= 1u << k;
  }
  return word;
}

}  // namespace kgb
