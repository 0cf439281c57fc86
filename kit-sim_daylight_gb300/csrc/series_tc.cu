// The hourly time series of a chunk on the 5th-generation tensor cores (sm_103a tcgen05 + TMA), split-BF16:
//
//   E[i, t] = sum_k V[i, k] S[k, t]  +  sun term of column t (FP32, epilogue)
//
// with k over the sky patches (V = the cos- and transmission-weighted visibility per patch, S = the patch radiance per
// step), then the ground (V = G, S = g) and the reflected-light bins (V = dc, S = Sdc): the reference's k_series +
// k_series_dc (gpu.cu:116-169) as one dense contraction. Each operand is split x = hi + lo in bf16 (16 significant
// bits) and three products run per K block (hi.hi + hi.lo + lo.hi, fp32 accumulation in tensor memory); the sun term
// (one direction per step, exact in the reference's float arithmetic) is added in the epilogue, where each output is
// finished in registers and streamed to HBM with 128-byte row stores.
//
// Kernel k_series_tc, one CTA per SM, persistent over 128 x 128 output tiles (sensors x steps, steps fastest so that
// the CTAs running at once share a few V panels and all of S in L2):
//   warp 0      TMA producer: per 64-wide K block, V_hi, V_lo (128 x 64) and S_hi, S_lo (128 x 64) bf16 tiles,
//               128-byte swizzled, into a 3-stage shared-memory ring (64 KB a stage)
//   warp 1      MMA issuer (one thread): 12 tcgen05.mma (M 128, N 128, K 16) per stage into one of two TMEM
//               accumulators (128 columns each), tcgen05.commit to free the stage / to hand the tile to the epilogue
//   warps 2-5   epilogue: tcgen05.ld 32 columns at a time (warp w reads TMEM lanes 32 (w % 4) ..), the sun term,
//               a per-warp shared-memory transpose, coalesced stores of E rows
// Every wait on an mbarrier is bounded: past the limit the kernel records kStatusTimeout and leaves its loops (the
// TMEM it holds is released on the way out).
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include "engine.h"

#include <algorithm>

namespace kgb {

constexpr int BM = 128, BN = 128, BK = 64, STAGES = 3;
constexpr int TILE_BYTES = BM * BK * 2;              // 16 KB: one bf16 operand tile (rows x 128 B)
constexpr int STAGE_BYTES = 4 * TILE_BYTES;          // V_hi, V_lo, S_hi, S_lo
constexpr int EPI_WARPS = 4;
constexpr int THREADS = 32 * (2 + EPI_WARPS);
constexpr int STAGE_PAD = 33;                        // floats per row of the per-warp transpose buffer
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + EPI_WARPS * 32 * STAGE_PAD * 4 + 1024 /* align */ + 256 /* barriers */;
constexpr uint32_t TMEM_COLS = 2 * BN;               // two accumulators
constexpr uint64_t kWaitLimitNs = 4000000000ull;   // 4 s: no wait of a healthy run comes near it

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ uint64_t globaltimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}
// Bounded wait for the phase of the given parity; false (and the status bit) once kWaitLimitNs have passed.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t* status) {
  uint64_t t0 = 0;
  for (uint32_t k = 0;; ++k) {
    uint32_t ok;
    asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
                 : "=r"(ok) : "r"(smem_u32(bar)), "r"(parity) : "memory");
    if (ok) return true;
    if ((k & 255) == 0) {
      const uint64_t t = globaltimer();
      if (!t0) t0 = t;
      else if (t - t0 > kWaitLimitNs) { atomicOr(status, kStatusTimeout); return false; }
    }
  }
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
  asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
               ::"r"(smem_u32(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar)) : "memory");
}

// K-major operand tile, 128-byte swizzle: rows of 64 bf16 (128 B), 8-row atoms 1024 B apart (SBO), version 1.
__device__ __forceinline__ uint64_t smem_desc(const void* tile) {
  const uint64_t a = smem_u32(tile);
  return ((a >> 4) & 0x3FFFull) | (uint64_t(1024 >> 4) << 32) | (uint64_t(1) << 46) | (uint64_t(2) << 61);
}
// kind::f16 instruction descriptor: D f32, A and B bf16, both K-major, N = BN, M = BM.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(BN >> 3) << 17) | (uint32_t(BM >> 4) << 24);

__device__ __forceinline__ void mma_bf16(uint32_t dTmem, uint64_t aDesc, uint64_t bDesc, uint32_t accumulate) {
  asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
               ::"r"(dTmem), "l"(aDesc), "l"(bDesc), "r"(kIdesc), "r"(accumulate));
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,"
      "%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]),
        "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]),
        "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
        "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int k = 0; k < 32; ++k) v[k] = __uint_as_float(r[k]);
}

struct SeriesTcArgs {
  uint32_t nc, T, Kp, mTiles, nTiles;
  // sun term of the epilogue (the reference's k_series tail, gpu.cu:145-148): column t's sun direction, if any
  const int32_t* sunOfCol;   // [T] -> j or -1
  const float* sunVec;       // [nSun x 3]
  const float* sunW;         // [nSun]
  uint32_t sun0;
  const uint32_t* bits;      // visibility (bits, or bytes when non-null)
  const uint8_t* bytes;
  const float* N;            // chunk normals
  float* E;                  // [nc x T]
  uint32_t* status;
};

__device__ __forceinline__ float dotf_rn(const float* n, const float* d) {
  return __fadd_rn(__fadd_rn(__fmul_rn(n[0], d[0]), __fmul_rn(n[1], d[1])), __fmul_rn(n[2], d[2]));
}

__global__ void __launch_bounds__(THREADS, 1) k_series_tc(const __grid_constant__ CUtensorMap mapVhi, const __grid_constant__ CUtensorMap mapVlo,
                                                          const __grid_constant__ CUtensorMap mapShi, const __grid_constant__ CUtensorMap mapSlo,
                                                          SeriesTcArgs a) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  float* stageBuf = reinterpret_cast<float*>(smem + STAGES * STAGE_BYTES);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + STAGES * STAGE_BYTES + EPI_WARPS * 32 * STAGE_PAD * 4);
  uint64_t* full = bars;               // [STAGES] TMA -> MMA
  uint64_t* empty = bars + STAGES;     // [STAGES] MMA -> TMA
  uint64_t* accFull = bars + 2 * STAGES;       // [2] MMA -> epilogue
  uint64_t* accEmpty = bars + 2 * STAGES + 2;  // [2] epilogue -> MMA
  uint32_t* tmemSlot = reinterpret_cast<uint32_t*>(bars + 2 * STAGES + 4);
  __shared__ volatile uint32_t abortFlag;

  const uint32_t warp = threadIdx.x / 32, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) { mbar_init(&full[s], 1); mbar_init(&empty[s], 1); }
    for (int b = 0; b < 2; ++b) { mbar_init(&accFull[b], 1); mbar_init(&accEmpty[b], EPI_WARPS * 32); }
    abortFlag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {   // TMEM: two accumulators of BN fp32 columns x 128 lanes
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmemSlot)), "r"(TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmemBase = *tmemSlot;
  const uint32_t kBlocks = a.Kp / BK;
  const uint32_t nTilesAll = a.mTiles * a.nTiles;

  if (warp == 0) {
    if (lane == 0) {   // ---------------- TMA producer
      uint32_t stage = 0, phase = 0;
      for (uint32_t tile = blockIdx.x; tile < nTilesAll && !abortFlag; tile += gridDim.x) {
        const int m0 = int(tile / a.nTiles) * BM, n0 = int(tile % a.nTiles) * BN;
        for (uint32_t kb = 0; kb < kBlocks; ++kb) {
          if (!mbar_wait(&empty[stage], phase ^ 1, a.status)) { abortFlag = 1; break; }
          uint8_t* s = smem + stage * STAGE_BYTES;
          mbar_expect_tx(&full[stage], STAGE_BYTES);
          const int k0 = int(kb) * BK;
          tma_load_2d(s, &mapVhi, k0, m0, &full[stage]);
          tma_load_2d(s + TILE_BYTES, &mapVlo, k0, m0, &full[stage]);
          tma_load_2d(s + 2 * TILE_BYTES, &mapShi, k0, n0, &full[stage]);
          tma_load_2d(s + 3 * TILE_BYTES, &mapSlo, k0, n0, &full[stage]);
          if (++stage == STAGES) { stage = 0; phase ^= 1; }
        }
      }
    }
    __syncwarp();
  } else if (warp == 1) {
    if (lane == 0) {   // ---------------- MMA issuer
      uint32_t stage = 0, phase = 0, local = 0;
      for (uint32_t tile = blockIdx.x; tile < nTilesAll && !abortFlag; tile += gridDim.x, ++local) {
        const uint32_t buf = local & 1, use = local >> 1;
        if (!mbar_wait(&accEmpty[buf], (use & 1) ^ 1, a.status)) { abortFlag = 1; break; }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t dTmem = tmemBase + buf * BN;
        for (uint32_t kb = 0; kb < kBlocks; ++kb) {
          if (!mbar_wait(&full[stage], phase, a.status)) { abortFlag = 1; break; }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint8_t* s = smem + stage * STAGE_BYTES;
          const uint64_t dVhi = smem_desc(s), dVlo = smem_desc(s + TILE_BYTES), dShi = smem_desc(s + 2 * TILE_BYTES),
                         dSlo = smem_desc(s + 3 * TILE_BYTES);
#pragma unroll
          for (int k = 0; k < BK / 16; ++k) {   // 16 bf16 = 32 bytes along K: +2 in the descriptor's address field
            const uint64_t off = uint64_t(2 * k);
            mma_bf16(dTmem, dVhi + off, dShi + off, (kb | k) != 0);
            mma_bf16(dTmem, dVhi + off, dSlo + off, 1);
            mma_bf16(dTmem, dVlo + off, dShi + off, 1);
          }
          mma_commit(&empty[stage]);   // the stage is free once these MMAs have read it
          if (++stage == STAGES) { stage = 0; phase ^= 1; }
        }
        mma_commit(&accFull[buf]);     // the tile's accumulator is complete
      }
    }
    __syncwarp();
  } else {   // ---------------- epilogue: warps 2..5
    const uint32_t q = warp & 3;                       // TMEM lane quarter this warp may read
    float* tb = stageBuf + (warp - 2) * 32 * STAGE_PAD;
    uint32_t local = 0;
    for (uint32_t tile = blockIdx.x; tile < nTilesAll; tile += gridDim.x, ++local) {
      const uint32_t buf = local & 1, use = local >> 1;
      bool ok = mbar_wait(&accFull[buf], use & 1, a.status);
      ok = __all_sync(~0u, ok);
      if (!ok || abortFlag) { abortFlag = 1; break; }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t m0 = (tile / a.nTiles) * BM, n0 = (tile % a.nTiles) * BN;
      const uint32_t row = m0 + q * 32 + lane;         // this thread's sensor
      float nrm[3] = {0.f, 0.f, 0.f};
      if (row < a.nc) { nrm[0] = a.N[3 * row]; nrm[1] = a.N[3 * row + 1]; nrm[2] = a.N[3 * row + 2]; }
      for (uint32_t c0 = 0; c0 < BN; c0 += 32) {
        float v[32];
        tmem_ld32(tmemBase + ((q * 32u) << 16) + buf * BN + c0, v);
#pragma unroll 4
        for (int c = 0; c < 32; ++c) {
          const uint32_t t = n0 + c0 + c;
          if (t < a.T && row < a.nc) {
            const int j = __ldg(a.sunOfCol + t);
            if (j >= 0) {
              const uint32_t d = a.sun0 + uint32_t(j);
              float at;
              if (a.bytes) { const uint32_t b = a.bytes[size_t(d) * a.nc + row]; at = b ? float(b) / 255.f : 0.f; }
              else at = float((a.bits[size_t(d >> 5) * a.nc + row] >> (d & 31)) & 1u);
              if (at != 0.f) v[c] = __fadd_rn(v[c], __fmul_rn(__fmul_rn(fmaxf(dotf_rn(nrm, a.sunVec + 3 * j), 0.f), at), a.sunW[j]));
            }
          }
          tb[lane * STAGE_PAD + c] = v[c];
        }
        __syncwarp();
        // the warp's 32 rows x 32 columns: one 128-byte row segment per store instruction
        const uint32_t t = n0 + c0 + lane;
        for (int r = 0; r < 32; ++r) {
          const uint32_t rr = m0 + q * 32 + r;
          if (rr < a.nc && t < a.T) a.E[size_t(rr) * a.T + t] = tb[r * STAGE_PAD + lane];
        }
        __syncwarp();
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      mbar_arrive(&accEmpty[buf]);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmemBase), "r"(TMEM_COLS));
  }
}

// ------------------------------------------------------------------------------------------------ operand builds
// V per chunk: V[i, k] = sum over the sky directions d of patch k (in d order) of max(0, N_i . D_d) T_d wsky_d (float),
// then G_i (k = P), then dc(b, i) (k = P + 1 + b); split into bf16 hi + lo, rows of Kp (zero padded). A block computes 32
// sensors x 64 columns: lanes = sensors (coalesced visibility reads), then the rows leave through shared memory.
struct VBuildArgs {
  const uint32_t* bits;
  const uint8_t* bytes;
  uint32_t nc, P, nBins, Kp, nDirTotal;
  const float* N;
  const float* D;
  const int32_t* patchFirst;   // [P + 1] CSR of the sky directions per patch
  const int32_t* patchDirs;
  const float* wsky;
  const float* G;
  const float* dc;             // [nBins x nc] or null
  __nv_bfloat16* vhi;
  __nv_bfloat16* vlo;
};

__global__ void __launch_bounds__(256) k_build_v(VBuildArgs a) {
  __shared__ float tile[64][33];
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t i0 = blockIdx.x * 32, k0 = blockIdx.y * 64;
  const uint32_t i = i0 + lane;
  float n[3] = {0.f, 0.f, 0.f};
  if (i < a.nc) { n[0] = a.N[3 * i]; n[1] = a.N[3 * i + 1]; n[2] = a.N[3 * i + 2]; }
  for (uint32_t kk = warp; kk < 64; kk += 8) {
    const uint32_t k = k0 + kk;
    float v = 0.f;
    if (i < a.nc) {
      if (k < a.P) {
        for (int32_t q = a.patchFirst[k]; q < a.patchFirst[k + 1]; ++q) {
          const uint32_t d = uint32_t(a.patchDirs[q]);
          float at;
          if (a.bytes) { const uint32_t b = a.bytes[size_t(d) * a.nc + i]; at = b ? float(b) / 255.f : 0.f; }
          else at = float((a.bits[size_t(d >> 5) * a.nc + i] >> (d & 31)) & 1u);
          if (at != 0.f) v = __fadd_rn(v, __fmul_rn(__fmul_rn(fmaxf(dotf_rn(n, a.D + 3 * d), 0.f), at), a.wsky[d]));
        }
      } else if (k == a.P) v = a.G[i];
      else if (a.dc && k < a.P + 1 + a.nBins) v = a.dc[size_t(k - a.P - 1) * a.nc + i];
    }
    tile[kk][lane] = v;
  }
  __syncthreads();
  // write rows: each warp writes 4 sensors' 64 columns (2 values per lane)
  for (uint32_t r = warp; r < 32; r += 8) {
    const uint32_t ii = i0 + r;
    if (ii >= a.nc) continue;
    for (uint32_t h = 0; h < 2; ++h) {
      const uint32_t kk = h * 32 + lane;
      const float x = tile[kk][r];
      const __nv_bfloat16 hi = __float2bfloat16_rn(x);
      const __nv_bfloat16 lo = __float2bfloat16_rn(x - __bfloat162float(hi));
      a.vhi[size_t(ii) * a.Kp + k0 + kk] = hi;
      a.vlo[size_t(ii) * a.Kp + k0 + kk] = lo;
    }
  }
}

// S^T per chunk (K-major rows of the steps): St[t, k] = S[k, t] (k < P), g[t] (k = P), Sdc[k - P - 1, t]; hi + lo.
__global__ void __launch_bounds__(256) k_build_st(const float* S, const float* g, const float* Sdc, uint32_t P, uint32_t nBins, uint32_t T,
                                                  uint32_t Kp, __nv_bfloat16* shi, __nv_bfloat16* slo) {
  __shared__ float tile[32][33];
  const uint32_t t0 = blockIdx.x * 32, k0 = blockIdx.y * 32;
  const uint32_t tx = threadIdx.x & 31, ty = threadIdx.x >> 5;   // 8 rows of 32
  for (uint32_t r = ty; r < 32; r += 8) {
    const uint32_t k = k0 + r, t = t0 + tx;
    float v = 0.f;
    if (t < T) {
      if (k < P) v = S[size_t(k) * T + t];
      else if (k == P) v = g[t];
      else if (Sdc && k < P + 1 + nBins) v = Sdc[size_t(k - P - 1) * T + t];
    }
    tile[r][tx] = v;
  }
  __syncthreads();
  for (uint32_t r = ty; r < 32; r += 8) {
    const uint32_t t = t0 + r, k = k0 + tx;
    if (t >= T) continue;
    const float x = tile[tx][r];
    const __nv_bfloat16 hi = __float2bfloat16_rn(x);
    shi[size_t(t) * Kp + k] = hi;
    slo[size_t(t) * Kp + k] = __float2bfloat16_rn(x - __bfloat162float(hi));
  }
}

// ------------------------------------------------------------------------------------------------ host
static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    cudaDriverEntryPointQueryResult q;
    void* p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

// A [rows x Kp] bf16, K contiguous: boxes of 64 (128 B) x 128 rows, 128-byte swizzle, zero fill past the rows.
static bool make_map(CUtensorMap* m, const void* base, uint64_t rows, uint64_t Kp) {
  auto fn = encode_fn();
  if (!fn) return false;
  const cuuint64_t dims[2] = {Kp, rows};
  const cuuint64_t strides[1] = {Kp * 2};
  const cuuint32_t box[2] = {BK, BM};
  const cuuint32_t estr[2] = {1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

const char* series_tc(const SeriesTcPlan& p, cudaStream_t st) {
  if (p.nc == 0 || p.T == 0) return nullptr;
  if (p.Kp % BK) return "series_tc: K not padded to 64";
  CUtensorMap mVhi, mVlo, mShi, mSlo;
  if (!make_map(&mVhi, p.vhi, p.nc, p.Kp) || !make_map(&mVlo, p.vlo, p.nc, p.Kp) || !make_map(&mShi, p.shi, p.T, p.Kp) ||
      !make_map(&mSlo, p.slo, p.T, p.Kp))
    return "series_tc: cuTensorMapEncodeTiled failed";
  static bool attr = false;
  if (!attr) {
    if (cudaFuncSetAttribute(k_series_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES) != cudaSuccess)
      return "series_tc: cannot reserve shared memory";
    attr = true;
  }
  SeriesTcArgs a{};
  a.nc = p.nc; a.T = p.T; a.Kp = p.Kp;
  a.mTiles = (p.nc + BM - 1) / BM; a.nTiles = (p.T + BN - 1) / BN;
  a.sunOfCol = p.sunOfCol; a.sunVec = p.sunVec; a.sunW = p.sunW; a.sun0 = p.sun0;
  a.bits = p.bits; a.bytes = p.bytes; a.N = p.N; a.E = p.E; a.status = p.status;
  const int grid = int(std::min<uint32_t>(uint32_t(p.numSMs), a.mTiles * a.nTiles));
  k_series_tc<<<grid, THREADS, SMEM_BYTES, st>>>(mVhi, mVlo, mShi, mSlo, a);
  return nullptr;
}

void build_series_operands(const SeriesTcPlan& p, const SeriesOperands& o, cudaStream_t st) {
  VBuildArgs v{};
  v.bits = p.bits; v.bytes = p.bytes; v.nc = p.nc; v.P = o.P; v.nBins = o.nBins; v.Kp = p.Kp; v.N = p.N; v.D = o.D;
  v.patchFirst = o.patchFirst; v.patchDirs = o.patchDirs; v.wsky = o.wsky; v.G = o.G; v.dc = o.dc;
  v.vhi = static_cast<__nv_bfloat16*>(p.vhi); v.vlo = static_cast<__nv_bfloat16*>(p.vlo);
  k_build_v<<<dim3((p.nc + 31) / 32, p.Kp / 64), 256, 0, st>>>(v);
  if (o.rebuildS)
    k_build_st<<<dim3((p.T + 31) / 32, p.Kp / 32), 256, 0, st>>>(o.S, o.g, o.Sdc, o.P, o.nBins, p.T, p.Kp, static_cast<__nv_bfloat16*>(p.shi),
                                                                 static_cast<__nv_bfloat16*>(p.slo));
}

}  // namespace kgb
