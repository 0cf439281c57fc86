// The hourly time series of a chunk, plain FP32 form: one thread per sensor, t in tiles of 32 held in registers, the
// sky directions' visibility walked per tile (restates the reference's k_series / k_series_dc, gpu.cu:116-169, as the
// required one-request-per-launch baseline). E[i*T + t] = sum_{sky d visible} max(0, N.D_d) T_d wsky_d S[row_d, t]
// + G_i g_t + sun term at its step [+ sum_b dc(b, i) Sdc[b, t]].
#include "engine.h"

namespace kgb {

__device__ __forceinline__ float vis_at(const SeriesArgs& a, uint32_t d, uint32_t i) {
  if (a.bytes) { const uint32_t b = a.bytes[size_t(d) * a.nc + i]; return b ? float(b) / 255.f : 0.f; }
  return float((a.bits[size_t(d >> 5) * a.nc + i] >> (d & 31)) & 1u);
}
__device__ __forceinline__ uint32_t vis_mask(const SeriesArgs& a, uint32_t w, uint32_t i) {
  if (!a.bytes) return a.bits[size_t(w) * a.nc + i];
  uint32_t m = 0;
  for (uint32_t k = 0; k < 32 && w * 32 + k < a.nDir; ++k) m |= uint32_t(a.bytes[size_t(w * 32 + k) * a.nc + i] != 0) << k;
  return m;
}
__device__ __forceinline__ float dotf(const float* n, const float* d) { return __fadd_rn(__fadd_rn(__fmul_rn(n[0], d[0]), __fmul_rn(n[1], d[1])), __fmul_rn(n[2], d[2])); }

__global__ void __launch_bounds__(128) k_series_fp32(SeriesArgs a) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.nc) return;
  const float* n = a.N + 3 * size_t(i);
  float* Ei = a.E + size_t(i) * a.T;
  for (uint32_t t0 = 0; t0 < a.T; t0 += 32) {
    float e[32];
#pragma unroll
    for (int tt = 0; tt < 32; ++tt) e[tt] = 0.f;
    for (uint32_t w = 0; w * 32 < a.nSky; ++w) {
      uint32_t m = vis_mask(a, w, i);
      while (m) {
        const uint32_t d = w * 32 + (__ffs(m) - 1);
        m &= m - 1;
        if (d >= a.nSky) break;
        const float c = fmaxf(dotf(n, a.D + 3 * d), 0.f) * vis_at(a, d, i) * a.wsky[d];
        const float* s = a.S + size_t(a.row[d]) * a.T + t0;
#pragma unroll
        for (int tt = 0; tt < 32; ++tt) if (t0 + tt < a.T) e[tt] += c * __ldg(s + tt);
      }
    }
    if (a.dc) {
      for (uint32_t b = 0; b < a.nBins; ++b) {
        const float c = a.dc[size_t(b) * a.nc + i];
        if (c == 0.f) continue;
        const float* s = a.Sdc + size_t(b) * a.T + t0;
#pragma unroll
        for (int tt = 0; tt < 32; ++tt) if (t0 + tt < a.T) e[tt] += c * __ldg(s + tt);
      }
    }
    for (uint32_t tt = 0; tt < 32 && t0 + tt < a.T; ++tt) Ei[t0 + tt] = e[tt] + a.G[i] * a.g[t0 + tt];
  }
  for (uint32_t j = 0; j < a.nSun; ++j) {
    const uint32_t d = a.sun0 + j;
    const float at = vis_at(a, d, i);
    if (at != 0.f) Ei[a.sunStep[j]] += fmaxf(dotf(n, a.sunVec + 3 * j), 0.f) * at * a.sunW[j];
  }
}

void launch_series_fp32(const SeriesArgs& a, cudaStream_t st) { k_series_fp32<<<(a.nc + 127) / 128, 128, 0, st>>>(a); }

}  // namespace kgb
