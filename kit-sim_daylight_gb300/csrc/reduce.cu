// Accumulation kernels over the visibility the ray-casting kernels leave on the device (compiled with -fmad=false):
//  k_reduce_bits / k_reduce_bytes / k_reduce_dc  out[i] = sum over d (or bins) in order of
//      double(float(max(0, N_i . D_d) x T) ) x W[d]   (replaces the reference's k_reduce, gpu.cu:99-114)
//  k_view_reduce  per sensor and class: weight, weight x ln d, min d; own weight; reach; glazing (replaces k_view,
//      gpu.cu:238-274), one warp per sensor, lane l summing d = l, l + 32, ..., then a fixed shuffle tree
//  k_iso          the isovist area / volume through the rays' end points (replaces k_iso + iso_lane, gpu.cu:187-236)
// The summation orders are fixed (direction order per thread; lane order + shuffle tree per warp), so a sensor's
// doubles do not depend on the chunk it is in, and equal the oracle's restatement bit for bit.
#include "engine.h"
#include "rt.cuh"

namespace kgb {

__device__ __forceinline__ float dotf(F3 a, F3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }   // per-op rounding (gpu.cu:69-72)

// GB300's FP64 pipe is narrow (a few lanes per clock per SM), so each term of a sum costs one FP64 instruction:
//  - the float factor x > 0 becomes a double exactly by integer operations (widen, rt.cuh);
//  - the weights are read as doubles: converted once per call into a device array (or, where the caller has no room
//    for one, once per block into shared memory);
//  - the product of two floats is exact in double, so fma(x, w, acc) equals acc + x * w rounded once, as the
//    reference's separate multiply and add;
//  - a zero factor adds +0, which leaves the sum as it is: it is skipped.

constexpr uint32_t kReduceSmemDirs = 24576;   // weights held as doubles in shared memory (192 KB) up to this many

template <bool SMEM>
__device__ __forceinline__ const double* weights_to_smem(const float* W, uint32_t n, double* sW) {
  if constexpr (SMEM) {
    for (uint32_t d = threadIdx.x; d < n; d += blockDim.x) sW[d] = (double)__ldg(W + d);
    __syncthreads();
    return sW;
  } else {
    return nullptr;
  }
}
template <bool SMEM>
__device__ __forceinline__ double weight(const double* sW, const float* W, uint32_t d) { return SMEM ? sW[d] : (double)__ldg(W + d); }

template <bool SMEM>
__global__ void __launch_bounds__(256) k_reduce_bits(const uint32_t* __restrict__ bits, uint32_t nc, uint32_t nWords, uint32_t nDir,
                                                     const float* __restrict__ N, const float* __restrict__ D, const float* __restrict__ W,
                                                     int useCos, double* __restrict__ out) {
  extern __shared__ double sW[];
  const double* w64 = weights_to_smem<SMEM>(W, nDir, sW);
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nc) return;
  const F3 n = ld3(N + 3 * size_t(i));
  double acc = 0;
  for (uint32_t w = 0; w < nWords; ++w) {
    uint32_t m = bits[size_t(w) * nc + i];
    while (m) {
      const uint32_t d = w * 32 + (__ffs(m) - 1);
      m &= m - 1;
      const float c = useCos ? fmaxf(dotf(n, ld3(D + 3 * d)), 0.f) : 1.f;
      if (c != 0.f) acc = __fma_rn(widen(c), weight<SMEM>(w64, W, d), acc);
    }
  }
  out[i] = acc;
}

template <bool SMEM>
__global__ void __launch_bounds__(256) k_reduce_bytes(const uint8_t* __restrict__ bytes, uint32_t nc, uint32_t nDir, const float* __restrict__ N,
                                                      const float* __restrict__ D, const float* __restrict__ W, int useCos, double* __restrict__ out) {
  extern __shared__ double sW[];
  const double* w64 = weights_to_smem<SMEM>(W, nDir, sW);
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nc) return;
  const F3 n = ld3(N + 3 * size_t(i));
  double acc = 0;
  // 16 directions' bytes are loaded before any is used (16 loads in flight per thread: a chunk of the reference's
  // size leaves few threads per SM), then added in direction order
  constexpr uint32_t G = 16;
  for (uint32_t d0 = 0; d0 < nDir; d0 += G) {
    uint32_t bb[G];
#pragma unroll
    for (uint32_t k = 0; k < G; ++k) bb[k] = d0 + k < nDir ? uint32_t(__ldg(bytes + size_t(d0 + k) * nc + i)) : 0u;
#pragma unroll
    for (uint32_t k = 0; k < G; ++k) {
      if (!bb[k]) continue;
      const uint32_t d = d0 + k;
      const float at = float(bb[k]) / 255.f;
      const float c = useCos ? fmaxf(dotf(n, ld3(D + 3 * d)), 0.f) : 1.f;
      const float x = c * at;
      if (x != 0.f) acc = __fma_rn(widen(x), weight<SMEM>(w64, W, d), acc);
    }
  }
  out[i] = acc;
}

__global__ void __launch_bounds__(256) k_reduce_dc(const float* __restrict__ dc, uint32_t nc, uint32_t nBins, const float* __restrict__ W, double* __restrict__ out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nc) return;
  double acc = 0;
  for (uint32_t b = 0; b < nBins; ++b) acc += (double)(1.f * dc[size_t(b) * nc + i]) * (double)__ldg(W + b);
  out[i] = acc;
}

__device__ __forceinline__ double warp_sum(double v) {
  for (uint32_t s = 16; s; s >>= 1) v += __shfl_down_sync(~0u, v, s);
  return v;
}

// One warp per sensor. A lane's per-class sums sit in shared memory as [class][lane] (a warp's lanes touch 32
// different banks whatever their classes), so a ray costs its own class's three updates, not a select over every
// class: GB300's FP64 pipe is narrow, and predicated double operations still take its slots. Classes at or past nClass
// are never reported and are not kept; the reach sums likewise hold nReach slots.
constexpr uint32_t kViewWarps = 8;   // warps (sensors) per block
__global__ void __launch_bounds__(256) k_view_reduce(ViewReduceArgs a) {
  extern __shared__ double vsm[];
  const uint32_t warp = threadIdx.x / 32, lane = threadIdx.x & 31, i = blockIdx.x * kViewWarps + warp;
  const uint32_t C = a.nClass, R = a.nReach;
  double* sw = vsm + size_t(warp) * (2 * C + R) * 32;   // w [C][32], wl [C][32], reach [R][32]
  double* swl = sw + C * 32;
  double* src = swl + C * 32;
  float* smn = reinterpret_cast<float*>(vsm + size_t(kViewWarps) * (2 * C + R) * 32) + size_t(warp) * C * 32;   // mn [C][32]
  for (uint32_t c = 0; c < C; ++c) { sw[c * 32 + lane] = 0; swl[c * 32 + lane] = 0; smn[c * 32 + lane] = __int_as_float(0x7f800000); }
  for (uint32_t r = 0; r < R; ++r) src[r * 32 + lane] = 0;
  if (i >= a.nc) return;   // whole warps
  double own = 0, gz = 0;
  for (uint32_t d = lane; d < a.K; d += 32) {
    uint32_t c = a.cls[size_t(d) * a.nc + i];
    const float t = a.dist[size_t(d) * a.nc + i];
    const double wd = a.wRow[d / a.nAz];
    if (c == 254) { own += wd; continue; }
    if (c & KGB_VIEW_GLAZED) { gz += wd; c &= ~uint32_t(KGB_VIEW_GLAZED); }
    const float dd = fminf(fmaxf(t, 0.1f), a.farDist);
    const double ln = dd == a.farDist ? a.lnFar : dd == 0.1f ? -2.302585092994045684 : (double)kgb_logf(dd);
    if (c < C) {
      const uint32_t at = c * 32 + lane;
      sw[at] += wd;
      swl[at] += wd * ln;
      smn[at] = fminf(smn[at], dd);
    }
    for (uint32_t r = 0; r < R; ++r) if (t >= a.reach[r]) src[r * 32 + lane] += wd;
  }
  double* o = a.out + size_t(i) * a.NA;
  for (uint32_t c = 0; c < C; ++c) {
    float m = smn[c * 32 + lane];
    for (uint32_t s = 16; s; s >>= 1) m = fminf(m, __shfl_down_sync(~0u, m, s));
    const double x = warp_sum(sw[c * 32 + lane]), y = warp_sum(swl[c * 32 + lane]);
    if (!lane) { o[3 * c] = x; o[3 * c + 1] = y; o[3 * c + 2] = m; }
  }
  const double ow = warp_sum(own);
  if (!lane) o[3 * C] = ow;
  for (uint32_t r = 0; r < R; ++r) {
    const double x = warp_sum(src[r * 32 + lane]);
    if (!lane) o[3 * C + 1 + r] = x;
  }
  if (a.glazing) {
    const double x = warp_sum(gz);
    if (!lane) o[3 * C + 1 + R] = x;
  }
}

// view cell of direction d (the reference's view_cell, params.h:77-89), sincospif as kgb_sincospi
__device__ __forceinline__ F3 iso_cell(uint32_t d, uint32_t col, float rsx, float rsy, float az0, float dAz, bool jitter, uint32_t element, uint32_t side) {
  float a = 0.5f, s = 0.5f * (rsx + rsy);
  if (jitter) { const U3 h = pcg3d(element, d, side); a = u01(h.x); s = rsx + u01(h.y) * (rsy - rsx); }
  float sa, ca;
  kgb_sincospi((az0 + (float(col) + a) * dAz) * (1.f / 180.f), &sa, &ca);
  const float c = sqrtf(fmaxf(0.f, 1.f - s * s));
  return f3(c * sa, c * ca, s);
}
__device__ __forceinline__ float det3(F3 a, F3 b, F3 c) {
  const F3 u = sub(b, a), w = sub(c, a);
  return a.x * (u.y * w.z - u.z * w.y) + a.y * (u.z * w.x - u.x * w.z) + a.z * (u.x * w.y - u.y * w.x);
}

// Isovist of a sensor, one warp per sensor. A ray's end point is its clipped length (0 on the sensor's own surface, at
// most farDist) along its cell's direction in the field's own frame. isoDim 2: the area of the polygon through row 0's
// end points, one triangle (eye, column c, column c + 1) per column. isoDim 3: the volume enclosed by the end points,
// as the signed volumes of two tetrahedra with the eye per cell quad between rows r - 1 and r and columns c and c + 1.
// Column c + 1 of the last column is column 0 for a full circle; a narrower fan has no piece after its last column.
// Lane l owns the columns l, l + 32, ... Each piece is evaluated in float and added to the lane's double sum in row
// order; the lanes' sums are then combined by warp_sum's fixed tree. Those two orders and the float expressions of the
// pieces decide the resulting double, so they are kept equal to the reference's k_iso (gpu.cu:197-236).
struct IsoEnds { float here, next; };   // end lengths of a lane's column and of the column after it, in one row

__device__ __forceinline__ float iso_len(const ViewReduceArgs& a, uint32_t i, uint32_t k) {
  const size_t at = size_t(k) * a.nc + i;
  return a.cls[at] == 254 ? 0.f : fminf(a.dist[at], a.farDist);
}
// The next column's length comes from lane + 1 by shuffle, except where lane + 1 does not hold it (lane 31, or the wrap
// to column 0), which reads it itself. Every lane calls this in every group of columns, so the shuffle has the whole warp.
__device__ __forceinline__ IsoEnds iso_ends(const ViewReduceArgs& a, uint32_t i, uint32_t row, uint32_t col, uint32_t nxt, bool readsNext) {
  IsoEnds e;
  e.here = iso_len(a, i, row * a.nAz + col);
  const float fromNeighbour = __shfl_down_sync(~0u, e.here, 1);
  e.next = readsNext ? iso_len(a, i, row * a.nAz + nxt) : fromNeighbour;
  return e;
}

__global__ void __launch_bounds__(256) k_iso(ViewReduceArgs a) {
  const uint32_t i = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32, lane = threadIdx.x & 31;
  if (i >= a.nc) return;   // the whole warp leaves together
  const uint32_t gi = a.i0 + i, element = gi / a.nS, side = a.nS == 2 ? gi % 2 : a.back;
  const bool jit = a.jitter != 0;
  double sum = 0;
  for (uint32_t base = 0; base < a.nAz; base += 32) {
    // lanes past the last column repeat it and add nothing, but still take part in the shuffles
    const uint32_t col = min(base + lane, a.nAz - 1);
    const uint32_t nxt = col + 1 == a.nAz ? 0 : col + 1;
    const bool adds = base + lane < a.nAz && (a.world || col + 1 < a.nAz);
    const bool readsNext = lane == 31 || nxt == 0;
    F3 up0 = iso_cell(col, col, a.rowSin[0], a.rowSin[1], a.az0, a.dAz, jit, element, side);   // row 0, columns col, nxt
    F3 up1 = iso_cell(nxt, nxt, a.rowSin[0], a.rowSin[1], a.az0, a.dAz, jit, element, side);
    IsoEnds top = iso_ends(a, i, 0, col, nxt, readsNext);
    if (a.isoDim == 2) {   // the triangle's area: half the two lengths times the sine of the clockwise turn
      if (adds) sum += double(0.5f * top.here * top.next * (up0.y * up1.x - up0.x * up1.y));
      continue;
    }
    for (uint32_t r = 1; r < a.nEl; ++r) {
      const uint32_t d = r * a.nAz + col;
      const IsoEnds low = iso_ends(a, i, r, col, nxt, readsNext);
      const F3 lo0 = iso_cell(d, col, a.rowSin[2 * r], a.rowSin[2 * r + 1], a.az0, a.dAz, jit, element, side);
      const F3 lo1 = iso_cell(d - col + nxt, nxt, a.rowSin[2 * r], a.rowSin[2 * r + 1], a.az0, a.dAz, jit, element, side);
      // six times the volumes of (eye, up0, up1, lo0) and (eye, up1, lo1, lo0), each determinant scaled by its lengths
      if (adds) sum += double(top.here * top.next * low.here * det3(up0, up1, lo0) + top.next * low.next * low.here * det3(up1, lo1, lo0));
      up0 = lo0; up1 = lo1; top = low;
    }
  }
  const double v = warp_sum(a.isoDim == 2 ? sum : sum / 6);
  if (!lane) a.out[size_t(i) * a.NA + a.NA - 1] = v;
}

// The weights go to shared memory as doubles when they fit (kReduceSmemDirs); the kernels' sums are the same either way.
static bool reduce_smem_ready() {
  static bool ok = [] {
    const int bytes = int(kReduceSmemDirs * sizeof(double));
    return cudaFuncSetAttribute(k_reduce_bits<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) == cudaSuccess &&
           cudaFuncSetAttribute(k_reduce_bytes<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) == cudaSuccess;
  }();
  return ok;
}
// The weights as doubles in global memory (read through L1), one thread per sensor in blocks of 128: no shared memory
// per block, so the SMs hold as many blocks as their registers allow and take new ones as blocks end. The shared-memory
// form below (a block's copy of every weight, 45 KB at 5610 directions) kept four or five 256-thread blocks an SM, about
// one wave for the urban block, and the blocks of heavy sensors (roofs see most directions) held their SMs while the
// others idled: the urban step's four reduces took 8.85 ms that way, 4.93 ms this way (sums bit-identical; blocks of
// 64 and 256 threads: 5.23 and 5.76 ms). Widening the float weights in the kernel instead of converting them once
// took 9.95 ms.
constexpr uint32_t kReduceBlock = 128;
__global__ void k_weights64(const float* __restrict__ W, uint32_t n, double* __restrict__ W64) {
  const uint32_t d = blockIdx.x * blockDim.x + threadIdx.x;
  if (d < n) W64[d] = (double)W[d];
}
__global__ void __launch_bounds__(kReduceBlock) k_reduce_bits_w64(const uint32_t* __restrict__ bits, uint32_t nc, uint32_t nWords,
                                                                  const float* __restrict__ N, const float* __restrict__ D,
                                                                  const double* __restrict__ W64, int useCos, double* __restrict__ out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nc) return;
  const F3 n = ld3(N + 3 * size_t(i));
  double acc = 0;
  for (uint32_t w = 0; w < nWords; ++w) {
    uint32_t m = bits[size_t(w) * nc + i];
    while (m) {
      const uint32_t d = w * 32 + (__ffs(m) - 1);
      m &= m - 1;
      const float c = useCos ? fmaxf(dotf(n, ld3(D + 3 * d)), 0.f) : 1.f;
      if (c != 0.f) acc = __fma_rn(widen(c), __ldg(W64 + d), acc);
    }
  }
  out[i] = acc;
}
__global__ void __launch_bounds__(kReduceBlock) k_reduce_bytes_w64(const uint8_t* __restrict__ bytes, uint32_t nc, uint32_t nDir,
                                                                   const float* __restrict__ N, const float* __restrict__ D,
                                                                   const double* __restrict__ W64, int useCos, double* __restrict__ out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nc) return;
  const F3 n = ld3(N + 3 * size_t(i));
  double acc = 0;
  constexpr uint32_t G = 16;   // 16 directions' bytes in flight before any is used, then added in direction order
  for (uint32_t d0 = 0; d0 < nDir; d0 += G) {
    uint32_t bb[G];
#pragma unroll
    for (uint32_t k = 0; k < G; ++k) bb[k] = d0 + k < nDir ? uint32_t(__ldg(bytes + size_t(d0 + k) * nc + i)) : 0u;
#pragma unroll
    for (uint32_t k = 0; k < G; ++k) {
      if (!bb[k]) continue;
      const uint32_t d = d0 + k;
      const float at = float(bb[k]) / 255.f;
      const float c = useCos ? fmaxf(dotf(n, ld3(D + 3 * d)), 0.f) : 1.f;
      const float x = c * at;
      if (x != 0.f) acc = __fma_rn(widen(x), __ldg(W64 + d), acc);
    }
  }
  out[i] = acc;
}

void launch_reduce_bits(const uint32_t* bits, uint32_t nc, uint32_t nWords, uint32_t nDir, const float* N, const float* D, const float* W,
                        int useCos, double* out, cudaStream_t st, double* w64) {
  if (w64) {
    k_weights64<<<(nDir + 255) / 256, 256, 0, st>>>(W, nDir, w64);
    k_reduce_bits_w64<<<(nc + kReduceBlock - 1) / kReduceBlock, kReduceBlock, 0, st>>>(bits, nc, nWords, N, D, w64, useCos, out);
  } else if (nDir <= kReduceSmemDirs && reduce_smem_ready())
    k_reduce_bits<true><<<(nc + 255) / 256, 256, nDir * sizeof(double), st>>>(bits, nc, nWords, nDir, N, D, W, useCos, out);
  else k_reduce_bits<false><<<(nc + 255) / 256, 256, 0, st>>>(bits, nc, nWords, nDir, N, D, W, useCos, out);
}
void launch_reduce_bytes(const uint8_t* bytes, uint32_t nc, uint32_t nDir, const float* N, const float* D, const float* W, int useCos,
                         double* out, cudaStream_t st, double* w64) {
  if (w64) {
    k_weights64<<<(nDir + 255) / 256, 256, 0, st>>>(W, nDir, w64);
    k_reduce_bytes_w64<<<(nc + kReduceBlock - 1) / kReduceBlock, kReduceBlock, 0, st>>>(bytes, nc, nDir, N, D, w64, useCos, out);
  } else if (nDir <= kReduceSmemDirs && reduce_smem_ready())
    k_reduce_bytes<true><<<(nc + 255) / 256, 256, nDir * sizeof(double), st>>>(bytes, nc, nDir, N, D, W, useCos, out);
  else k_reduce_bytes<false><<<(nc + 255) / 256, 256, 0, st>>>(bytes, nc, nDir, N, D, W, useCos, out);
}
void launch_reduce_dc(const float* dc, uint32_t nc, uint32_t nBins, const float* W, double* out, cudaStream_t st) {
  k_reduce_dc<<<(nc + 255) / 256, 256, 0, st>>>(dc, nc, nBins, W, out);
}
void launch_reduce_view(const ViewReduceArgs& a, cudaStream_t st) {
  // shared memory: per warp 2 C + R doubles and C floats per lane (at most 19 classes and 8 reach distances: 111 KB)
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_view_reduce, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         int(kViewWarps * 32 * ((2 * KGB_VIEW_CLASSES + 8) * 8 + KGB_VIEW_CLASSES * 4)));
    attr = true;
  }
  const size_t smem = size_t(kViewWarps) * 32 * ((2 * a.nClass + a.nReach) * 8 + a.nClass * 4);
  k_view_reduce<<<(a.nc + kViewWarps - 1) / kViewWarps, kViewWarps * 32, smem, st>>>(a);
  if (a.isoDim) k_iso<<<(a.nc + 7) / 8, 256, 0, st>>>(a);
}

}  // namespace kgb
