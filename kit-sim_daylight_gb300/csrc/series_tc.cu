// The hourly time series of a chunk on the 5th-generation tensor cores (sm_103a tcgen05 + TMA), split-BF16:
//
//   E[i, t] = sum_k V[i, k] S[k, t]  +  sun term of column t (FP32, epilogue)
//
// with k over the sky patches (V = the cos- and transmission-weighted visibility per patch, S = the patch radiance per
// step), then the ground (V = G, S = g) and the reflected-light bins (V = dc, S = Sdc): the reference's k_series +
// k_series_dc (gpu.cu:116-169) as one dense contraction.
//
// Precision (within 1e-6 of an FP64 contraction per output column):
//  - each FP32 operand is split x = hi + mid + lo exactly into three bf16 pieces (24 significant bits), and six
//    products run per K step: hi.hi, then the corrections hi.mid + mid.hi + hi.lo + mid.mid + lo.hi (the dropped
//    mid.lo, lo.mid, lo.lo are 2^-24 of the product and below);
//  - the tensor core's FP32 accumulation truncates, so a long accumulation chain drifts low by about half an ulp of
//    the chain's magnitude per instruction (1e-5 over 2305 patches as one chain). The chains are therefore short: each
//    64 of K (a chunk) accumulates from zero in TMEM (4 K steps), and the epilogue adds the chunk's sum into FP32
//    registers with Kahan compensation (chains of 8 K steps doubled the column error, 4e-7 to 7e-7 of the column's
//    maximum);
//  - the sun term (one direction per step, exact in the reference's float arithmetic) is added by k_series_sun, which
//    runs after the contraction on the same stream: E[i, t] = E[i, t] + term, the same float operations in the same
//    order as the reference's k_series tail.
//
// The six products take three MMAs per K step: the three S pieces are consecutive tiles in shared memory, so one B
// operand of N 192 is [S hi | S mid | S lo], and a chunk's accumulator [H | C1 | C2] (3 x 64 columns) receives
//    hi  x [hi | mid | lo]   (N 192, into H C1 C2)
//    mid x [hi | mid]        (N 128, into C1 C2)
//    lo  x [hi]              (N 64, into C2)
// so H = hi.hi, C1 = hi.mid + mid.hi, C2 = hi.lo + mid.mid + lo.hi, and the epilogue adds H + (C1 + C2) per chunk.
// An M 128 K 16 MMA costs about 29 cycles (its A operand's read from shared memory) plus 0.66 a column: six of N 64
// take some 426 cycles a K step, these three 340 (7.6 to 6.85 ms a 29,609-sensor chunk).
// With two chunk accumulators the MMA issuer runs one chunk ahead of the epilogue, so the epilogue's work per chunk
// bounds the kernel once it outlasts the chunk's MMAs: its compensated sums run on packed pairs of columns
// (add / sub .f32x2, the same roundings as the scalar form), which took a chunk from 6.85 to 5.59 ms (5.31 ms with no
// per-chunk epilogue work at all).
//
// Kernel k_series_tc, one CTA per SM, persistent over 128 x 64 output tiles (sensors x steps) in bands of 16 step-tiles
// (tile_coords), so that the CTAs running at once share a few V panels and the band's S panels in L2:
//   warp 0      TMA producer: per 64-wide K block, the three pieces of V (128 x 64) and of S (64 x 64), bf16,
//               128-byte swizzled, into a 3-stage shared-memory ring (72 KB a stage)
//   warp 1      MMA issuer (one thread): 12 tcgen05.mma per stage (M 128, K 16; N 192, 128, 64) into the chunk's
//               accumulator [H | C1 | C2] (two of them, at TMEM columns 0 and 256); tcgen05.commit frees the stage and
//               hands the finished chunk to the epilogue
//   warps 2-9   epilogue, two per TMEM lane quarter (warp w reads lanes 32 (w % 4) ..) with 32 of the tile's 64 columns
//               each, a thread per output row: per chunk, tcgen05.ld of H, C1, C2 (one wait per 16 columns),
//               H + (C1 + C2) added into the row's 32 Kahan-compensated FP32 sums (16 packed pairs each of sum and
//               compensation); per tile, those columns of the row of E stored 16 bytes at a time
// With two chunk accumulators the MMA issuer waits for the epilogue whenever the epilogue's tile-end work outlasts two
// chunks of MMAs. The sun term at the tile's end (per column its sun direction, then the sensor's visibility of it: two
// dependent global loads behind a branch, 64 times) did: it took a 29,609-sensor chunk from 5.1 to 8.8 ms at 1.95 GHz.
// k_series_sun adds it in a pass of its own over E (about 0.05 ms a band of 7424 sensors).
// The Kahan sums stay in registers: ten warps per CTA (one CTA per SM) leave each thread up to 204 registers.
// Every wait on an mbarrier is bounded: past the limit the kernel records kStatusTimeout and leaves its loops. Before the
// CTA releases its TMEM and exits, the producer waits for the last fill it issued into each stage (so no bulk copy still
// writes shared memory) and the MMA issuer commits to a drain barrier and waits for it (so no MMA still runs); both
// waits have their own 4 s limit. In a run that did not time out both return at once: every fill and every MMA has
// been consumed by then.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include "engine.h"

#include <algorithm>

namespace kgb {

constexpr int BM = 128, BN = 64, BK = 64, STAGES = 3, PIECES = 3;
constexpr uint32_t NH = 2;                           // chunk accumulators [H | C1 | C2]: the MMA issuer runs a chunk ahead
constexpr int V_TILE = BM * BK * 2;                  // 16 KB: one bf16 V tile (128 rows x 128 B)
constexpr int S_TILE = BN * BK * 2;                  // 8 KB: one bf16 S^T tile (64 rows x 128 B)
constexpr int STAGE_BYTES = PIECES * (V_TILE + S_TILE); // V hi mid lo, S hi mid lo
constexpr int EPI_WARPS = 8;                        // two per TMEM lane quarter, 32 of the tile's 64 columns each
constexpr int EPI_COLS = BN * 4 / EPI_WARPS;        // the columns of one epilogue warp
constexpr int THREADS = 32 * (2 + EPI_WARPS);
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 /* align */ + 256 /* barriers */;
static_assert((2 * STAGES + 2 * NH + 1) * 8 + 4 <= 256, "the barriers and the TMEM slot fit their 256 bytes");
constexpr uint32_t TMEM_COLS = 512;
constexpr uint32_t kChunkCols = 256;                 // chunk accumulator b at column 256 b: [H | C1 | C2] in 3 x BN of them
static_assert(3 * BN <= kChunkCols && NH * kChunkCols <= TMEM_COLS, "the chunk accumulators fit TMEM");
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
// Bounded wait for the phase of the given parity; false (and the status bit) once limitNs have passed.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t* status, uint64_t limitNs) {
  uint64_t t0 = 0;
  for (uint32_t k = 0;; ++k) {
    uint32_t ok;
    asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
                 : "=r"(ok) : "r"(smem_u32(bar)), "r"(parity) : "memory");
    if (ok) return true;
    if ((k & 255) == 0) {
      const uint64_t t = globaltimer();
      if (!t0) t0 = t;
      else if (t - t0 > limitNs) { atomicOr(status, kStatusTimeout); return false; }
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
// kind::f16 instruction descriptor: D f32, A and B bf16, both K-major, M = BM, N as given.
constexpr uint32_t idesc(uint32_t n) { return (1u << 4) | (1u << 7) | (1u << 10) | ((n >> 3) << 17) | (uint32_t(BM >> 4) << 24); }

template <uint32_t N>
__device__ __forceinline__ void mma_bf16(uint32_t dTmem, uint64_t aDesc, uint64_t bDesc, uint32_t accumulate) {
  static_assert(N % 16 == 0 && N >= 16 && N <= 256, "M 128 takes N in 16 .. 256, a multiple of 16");
  asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
               ::"r"(dTmem), "l"(aDesc), "l"(bDesc), "r"(idesc(N)), "r"(accumulate));
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}
// Columns [c, c + 16) of three accumulators (TMEM addresses h, c1, c2) for this warp's 32 lanes, one wait for all.
__device__ __forceinline__ void tmem_ld16x3(uint32_t h, uint32_t c1, uint32_t c2, uint32_t* a, uint32_t* b, uint32_t* c) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%48];\n"
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%49];\n"
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%32,%33,%34,%35,%36,%37,%38,%39,%40,%41,%42,%43,%44,%45,%46,%47}, [%50];\n"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(a[0]), "=r"(a[1]), "=r"(a[2]), "=r"(a[3]), "=r"(a[4]), "=r"(a[5]), "=r"(a[6]), "=r"(a[7]), "=r"(a[8]), "=r"(a[9]), "=r"(a[10]),
        "=r"(a[11]), "=r"(a[12]), "=r"(a[13]), "=r"(a[14]), "=r"(a[15]),
        "=r"(b[0]), "=r"(b[1]), "=r"(b[2]), "=r"(b[3]), "=r"(b[4]), "=r"(b[5]), "=r"(b[6]), "=r"(b[7]), "=r"(b[8]), "=r"(b[9]), "=r"(b[10]),
        "=r"(b[11]), "=r"(b[12]), "=r"(b[13]), "=r"(b[14]), "=r"(b[15]),
        "=r"(c[0]), "=r"(c[1]), "=r"(c[2]), "=r"(c[3]), "=r"(c[4]), "=r"(c[5]), "=r"(c[6]), "=r"(c[7]), "=r"(c[8]), "=r"(c[9]), "=r"(c[10]),
        "=r"(c[11]), "=r"(c[12]), "=r"(c[13]), "=r"(c[14]), "=r"(c[15])
      : "r"(h), "r"(c1), "r"(c2)
      : "memory");
}

// Packed pairs of floats (add / sub .f32x2, sm_100 and later): each half is rounded exactly as the scalar add.rn /
// sub.rn rounds it, so the compensated sums below equal their scalar form bit for bit, in half the instructions.
__device__ __forceinline__ unsigned long long f2(uint32_t lo, uint32_t hi) {
  unsigned long long r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "r"(lo), "r"(hi));
  return r;
}
__device__ __forceinline__ unsigned long long add2(unsigned long long a, unsigned long long b) {
  unsigned long long r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ unsigned long long sub2(unsigned long long a, unsigned long long b) {
  unsigned long long r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}

// One contraction of a launch: the rows of tiles mBase .. mBase + mTiles - 1 of one chunk's E (a band of a chunk, or a
// request's chunk in a serving batch), with its own operands, K extent and sun term.
struct TcSeg {
  CUtensorMap mapV;          // the three pieces of V stacked as rows [3 nc x Kp]
  CUtensorMap mapS;          // the pieces of S^T stacked as [3 T x Kp]
  // sun term of the epilogue (the reference's k_series tail, gpu.cu:145-148): column t's sun direction, if any
  const int32_t* sunOfCol;   // [T] -> j or -1
  const float* sunVec;       // [nSun x 3]
  const float* sunW;         // [nSun]
  const uint32_t* bits;      // visibility (bits, or bytes when non-null), rows of nc sensors
  const uint8_t* bytes;
  const float* N;            // chunk normals
  float* E;                  // [nc x T]
  uint32_t nc, T, Kp, sun0;
  uint32_t mBase, mTiles, nTiles;
  uint32_t tileBase;         // the launch's tiles tileBase .. tileBase + mTiles x nTiles - 1 are this contraction's
  uint32_t sunBase;          // k_series_sun's blocks sunBase .. sunBase + (row blocks x column blocks) - 1, likewise
};
constexpr uint32_t kMaxTcSegs = kMaxSeriesGroup;   // contractions of one launch: their tensor maps travel as kernel parameters
struct TcGroup {
  TcSeg seg[kMaxTcSegs];
  uint32_t nSegs, nTiles, nSunBlocks;
  uint32_t* status;
  uint64_t waitLimitNs;      // the pipeline's mbarrier waits give up past this (kWaitLimitNs, or lower)
  uint32_t withholdFills;    // 1: the producer issues no fills, so that the waits run out (a test of the bounded waits)
};
static_assert(sizeof(TcGroup) <= 32000, "the group fits the 32 KB of kernel parameters");

// the contraction that launch tile `tile` belongs to (tiles are numbered contraction after contraction)
__device__ __forceinline__ uint32_t tc_seg_of(const TcGroup& g, uint32_t tile) {
  uint32_t lo = 0, hi = g.nSegs - 1;
  while (lo < hi) {
    const uint32_t mid = (lo + hi + 1) / 2;
    if (g.seg[mid].tileBase <= tile) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Tile order: bands of kBand step-tiles; within a band every row of tiles, steps fastest. The CTAs running at once share
// a few V panels and the band's S panels (16 x 64 steps x K x 6 B, some 30 MB at K 4672), which stay in L2 for the
// band; S is read from DRAM about once and V once per band (a steps-fastest order over all steps re-read S per row).
// Measured on a precision chunk (29,609 sensors x 4456 steps, K 4672; kernel time of the chunk, DRAM read of one of its
// four launches, on the earlier kernel that added the sun term itself): bands of 4 / 8 / 16 / 32 / all step-tiles 8.71 / 8.67 / 8.60 / 8.84 / 9.23 ms, 2.33 GB at 8, 1.55 GB
// at 16, 1.92 GB at 32. The MMA issue bounds the kernel (DRAM at about a tenth of its rate), and 16 reads the least.
// On the kernel with its sun term in a pass of its own (six launches a chunk): 8 / 12 / 16 / 24 / 32 gave 5.325 / 5.320 /
// 5.318 / 5.317 / 5.327 ms, the same within the noise.
constexpr uint32_t kBand = 16;
__device__ __forceinline__ void tile_coords(uint32_t tile, uint32_t mTiles, uint32_t nTiles, uint32_t& m, uint32_t& n) {
  const uint32_t perBand = mTiles * kBand, band = tile / perBand, idx = tile - band * perBand;
  const uint32_t width = min(kBand, nTiles - band * kBand);
  m = idx / width;
  n = band * kBand + idx % width;
}

__device__ __forceinline__ float dotf_rn(const float* n, const float* d) {
  return __fadd_rn(__fadd_rn(__fmul_rn(n[0], d[0]), __fmul_rn(n[1], d[1])), __fmul_rn(n[2], d[2]));
}

// Per contraction, mapV holds the three pieces of V stacked as rows [3 nc x Kp] and mapS those of S^T as [3 T x Kp].
// Piece p of an operand tile at rows r0 is at rows r0 + p nc (p T); rows past a piece's end read the next piece's rows
// (or the zero fill), which only reach accumulator rows and columns that are never stored. Every role walks the same
// tiles in the same order, each tile with its contraction's K blocks, so the pipeline's phases stay in step across
// contractions of different K.
__global__ void __launch_bounds__(THREADS, 1) k_series_tc(const __grid_constant__ TcGroup g) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + STAGES * STAGE_BYTES);
  uint64_t* full = bars;                 // [STAGES] TMA -> MMA
  uint64_t* empty = bars + STAGES;       // [STAGES] MMA -> TMA
  uint64_t* hFull = bars + 2 * STAGES;   // [NH] MMA -> epilogue: a chunk's sums are complete
  uint64_t* hEmpty = hFull + NH;         // [NH] epilogue -> MMA
  uint64_t* drain = hEmpty + NH;         // the MMA issuer's last commit: every MMA it issued has completed
  uint32_t* tmemSlot = reinterpret_cast<uint32_t*>(drain + 1);
  __shared__ volatile uint32_t abortFlag;

  const uint32_t warp = threadIdx.x / 32, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) { mbar_init(&full[s], 1); mbar_init(&empty[s], 1); }
    for (uint32_t b = 0; b < NH; ++b) { mbar_init(&hFull[b], 1); mbar_init(&hEmpty[b], EPI_WARPS * 32); }
    mbar_init(drain, 1);
    abortFlag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {   // TMEM: NH chunk accumulators of 3 x BN fp32 columns x 128 lanes
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmemSlot)), "r"(TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmemBase = *tmemSlot;
  const uint32_t nTilesAll = g.nTiles;

  if (warp == 0) {
    if (lane == 0) {   // ---------------- TMA producer
      uint32_t stage = 0, phase = 0;
      uint32_t filled = 0, fillParity = 0;   // bit s: stage s received a fill; the phase parity of its last one
      for (uint32_t tile = blockIdx.x; tile < nTilesAll && !abortFlag; tile += gridDim.x) {
        const TcSeg& a = g.seg[tc_seg_of(g, tile)];
        uint32_t tm, tn;
        tile_coords(tile - a.tileBase, a.mTiles, a.nTiles, tm, tn);
        const int m0 = int(tm + a.mBase) * BM, n0 = int(tn) * BN;
        const uint32_t kBlocks = a.Kp / BK;
        for (uint32_t kb = 0; kb < kBlocks; ++kb) {
          if (!mbar_wait(&empty[stage], phase ^ 1, g.status, g.waitLimitNs)) { abortFlag = 1; break; }
          if (g.withholdFills) {   // nothing completes full[stage]: the MMA issuer's wait on it runs out
            if (++stage == STAGES) { stage = 0; phase ^= 1; }
            continue;
          }
          uint8_t* s = smem + stage * STAGE_BYTES;
          mbar_expect_tx(&full[stage], STAGE_BYTES);
          const int k0 = int(kb) * BK;
#pragma unroll
          for (int p = 0; p < PIECES; ++p) {
            tma_load_2d(s + p * V_TILE, &a.mapV, k0, m0 + p * int(a.nc), &full[stage]);
            tma_load_2d(s + PIECES * V_TILE + p * S_TILE, &a.mapS, k0, n0 + p * int(a.T), &full[stage]);
          }
          filled |= 1u << stage;
          fillParity = (fillParity & ~(1u << stage)) | (phase << stage);
          if (++stage == STAGES) { stage = 0; phase ^= 1; }
        }
      }
      // A stage's fill is issued only after the previous one was consumed, so only the last fill of each stage can be
      // in flight here: wait until it has landed.
      for (uint32_t st = 0; st < uint32_t(STAGES); ++st)
        if ((filled >> st) & 1u) mbar_wait(&full[st], (fillParity >> st) & 1u, g.status, kWaitLimitNs);
    }
    __syncwarp();
  } else if (warp == 1) {
    if (lane == 0) {   // ---------------- MMA issuer
      uint32_t stage = 0, phase = 0, chunk = 0;
      for (uint32_t tile = blockIdx.x; tile < nTilesAll && !abortFlag; tile += gridDim.x) {
        bool ok = true;
        const uint32_t kBlocks = g.seg[tc_seg_of(g, tile)].Kp / BK;
        for (uint32_t kb = 0; kb < kBlocks; ++kb, ++chunk) {   // a chunk: one K block, its sums from zero in [H | C1 | C2]
          const uint32_t hbuf = chunk % NH;
          if (!mbar_wait(&hEmpty[hbuf], ((chunk / NH) & 1) ^ 1, g.status, g.waitLimitNs)) { ok = false; break; }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t hT = tmemBase + hbuf * kChunkCols;
          if (!mbar_wait(&full[stage], phase, g.status, g.waitLimitNs)) { ok = false; break; }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint8_t* s = smem + stage * STAGE_BYTES;
          const uint64_t v0 = smem_desc(s), v1 = smem_desc(s + V_TILE), v2 = smem_desc(s + 2 * V_TILE);
          const uint64_t sAll = smem_desc(s + PIECES * V_TILE);   // S hi, mid, lo: consecutive tiles, one operand of N 192
#pragma unroll
          for (int k = 0; k < BK / 16; ++k) {   // 16 bf16 = 32 bytes along K: +2 in the descriptor's address field
            const uint64_t off = uint64_t(2 * k);
            mma_bf16<3 * BN>(hT, v0 + off, sAll + off, k != 0);   // hi.hi | hi.mid | hi.lo
            mma_bf16<2 * BN>(hT + BN, v1 + off, sAll + off, 1);   //         mid.hi | mid.mid
            mma_bf16<BN>(hT + 2 * BN, v2 + off, sAll + off, 1);   //                  lo.hi
          }
          mma_commit(&empty[stage]);   // the stage is free once these MMAs have read it
          mma_commit(&hFull[hbuf]);
          if (++stage == STAGES) { stage = 0; phase ^= 1; }
        }
        if (!ok) { abortFlag = 1; break; }
      }
      // tcgen05.commit tracks every MMA this thread issued before it: once the drain barrier completes, none runs
      mma_commit(drain);
      mbar_wait(drain, 0, g.status, kWaitLimitNs);
    }
    __syncwarp();
  } else {   // ---------------- epilogue: warps 2..9
    const uint32_t q = warp & 3;                       // the TMEM lane quarter this warp may read
    const uint32_t c0 = (warp - 2) / 4 * EPI_COLS;     // and its columns of the tile
    const uint32_t laneBase = (q * 32u) << 16;
    uint32_t chunk = 0;
    for (uint32_t tile = blockIdx.x; tile < nTilesAll; tile += gridDim.x) {
      const TcSeg& a = g.seg[tc_seg_of(g, tile)];
      const uint32_t kBlocks = a.Kp / BK;
      // each chunk's H + (C1 + C2), added with Kahan compensation (acc - cmp is the running sum); columns 2p and 2p + 1
      // share the packed pair p of acc and cmp
      unsigned long long acc[EPI_COLS / 2], cmp[EPI_COLS / 2];
#pragma unroll
      for (int c = 0; c < EPI_COLS / 2; ++c) { acc[c] = 0ull; cmp[c] = 0ull; }
      bool ok = true;
      for (uint32_t ch = 0; ch < kBlocks; ++ch, ++chunk) {
        const uint32_t hbuf = chunk % NH;
        ok = __all_sync(~0u, mbar_wait(&hFull[hbuf], (chunk / NH) & 1, g.status, g.waitLimitNs));
        if (!ok || abortFlag) { ok = false; break; }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t hAt = tmemBase + laneBase + hbuf * kChunkCols + c0;
#pragma unroll
        for (int g = 0; g < EPI_COLS / 16; ++g) {
          uint32_t v[16], c1[16], c2[16];
          tmem_ld16x3(hAt + g * 16, hAt + BN + g * 16, hAt + 2 * BN + g * 16, v, c1, c2);
#pragma unroll
          for (int c = 0; c < 16; c += 2) {
            const int j = (g * 16 + c) / 2;
            const unsigned long long y = sub2(add2(f2(v[c], v[c + 1]), add2(f2(c1[c], c1[c + 1]), f2(c2[c], c2[c + 1]))), cmp[j]);
            const unsigned long long t = add2(acc[j], y);
            cmp[j] = sub2(sub2(t, acc[j]), y);
            acc[j] = t;
          }
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        mbar_arrive(&hEmpty[hbuf]);
      }
      if (!ok || abortFlag) { abortFlag = 1; break; }
      uint32_t tm, tn;
      tile_coords(tile - a.tileBase, a.mTiles, a.nTiles, tm, tn);
      const uint32_t m0 = (tm + a.mBase) * BM, n0 = tn * BN;
      const uint32_t row = m0 + q * 32 + lane;         // this thread's sensor
      float* Erow = a.E + size_t(row) * a.T;
      const bool vec = (a.T & 3u) == 0;                  // 16-byte row stores when rows are 16-byte aligned
      if (row < a.nc) {
#pragma unroll
        for (int g = 0; g < EPI_COLS / 16; ++g) {
          float v[16];
#pragma unroll
          for (int c = 0; c < 16; c += 2) {
            const unsigned long long d = sub2(acc[(g * 16 + c) / 2], cmp[(g * 16 + c) / 2]);
            v[c] = __uint_as_float(uint32_t(d)); v[c + 1] = __uint_as_float(uint32_t(d >> 32));
          }
          const uint32_t t0 = n0 + c0 + g * 16;
          if (vec && t0 + 16 <= a.T) {
#pragma unroll
            for (int c = 0; c < 16; c += 4) *reinterpret_cast<float4*>(Erow + t0 + c) = make_float4(v[c], v[c + 1], v[c + 2], v[c + 3]);
          } else {
#pragma unroll
            for (int c = 0; c < 16; ++c) if (t0 + c < a.T) Erow[t0 + c] = v[c];
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmemBase), "r"(TMEM_COLS));
  }
}

// The sun term of the reference's k_series tail (gpu.cu:145-148), added to E after the contraction: for column t with a
// sun direction j (sunOfCol), E[i, t] + max(0, N_i . sun_j) at(i, sun0 + j) w_j when the sensor's visibility at of it
// is not zero, in float with the reference's operation order. A block covers 32 sensors x 64 columns: the terms are
// computed with lanes over sensors (the visibility reads coalesce) and added with lanes over columns (the E reads and
// writes coalesce), through shared memory.
constexpr uint32_t kSunRows = 32, kSunCols = 64;
constexpr uint32_t kNoTerm = 0xffffffffu;   // no sun term (a NaN pattern the term's arithmetic does not produce on the GPU)
__device__ __forceinline__ uint32_t sun_seg_of(const TcGroup& g, uint32_t block) {
  uint32_t lo = 0, hi = g.nSegs - 1;
  while (lo < hi) {
    const uint32_t mid = (lo + hi + 1) / 2;
    if (g.seg[mid].sunBase <= block) lo = mid; else hi = mid - 1;
  }
  return lo;
}
__global__ void __launch_bounds__(256) k_series_sun(const __grid_constant__ TcGroup g) {
  __shared__ uint32_t term[kSunCols][kSunRows + 1];
  __shared__ int32_t jOf[kSunCols];
  const TcSeg& a = g.seg[sun_seg_of(g, blockIdx.x)];
  const uint32_t colBlocks = (a.T + kSunCols - 1) / kSunCols, local = blockIdx.x - a.sunBase;
  const uint32_t r0 = a.mBase * BM + (local / colBlocks) * kSunRows, t0 = (local % colBlocks) * kSunCols;
  const uint32_t rowEnd = min(a.nc, (a.mBase + a.mTiles) * BM);
  if (threadIdx.x < kSunCols) jOf[threadIdx.x] = t0 + threadIdx.x < a.T ? __ldg(a.sunOfCol + t0 + threadIdx.x) : -1;
  __syncthreads();
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t row = r0 + lane;
  float nrm[3] = {0.f, 0.f, 0.f};
  if (row < rowEnd) { nrm[0] = a.N[3 * row]; nrm[1] = a.N[3 * row + 1]; nrm[2] = a.N[3 * row + 2]; }
  for (uint32_t c = warp; c < kSunCols; c += 8) {
    const int j = jOf[c];
    uint32_t u = kNoTerm;
    if (j >= 0 && row < rowEnd) {
      const uint32_t d = a.sun0 + uint32_t(j);
      float at;
      if (a.bytes) { const uint32_t b = a.bytes[size_t(d) * a.nc + row]; at = b ? float(b) / 255.f : 0.f; }
      else at = float((a.bits[size_t(d >> 5) * a.nc + row] >> (d & 31)) & 1u);
      if (at != 0.f) u = __float_as_uint(__fmul_rn(__fmul_rn(fmaxf(dotf_rn(nrm, a.sunVec + 3 * j), 0.f), at), a.sunW[j]));
    }
    term[c][lane] = u;
  }
  __syncthreads();
  for (uint32_t r = warp; r < kSunRows; r += 8) {
    const uint32_t i = r0 + r;
    if (i >= rowEnd) break;
    float* Erow = a.E + size_t(i) * a.T;
#pragma unroll
    for (uint32_t h = 0; h < kSunCols / 32; ++h) {
      const uint32_t c = h * 32 + lane, u = term[c][r];
      if (u != kNoTerm) Erow[t0 + c] = __fadd_rn(Erow[t0 + c], __uint_as_float(u));
    }
  }
}

// ------------------------------------------------------------------------------------------------ operand builds
// V per chunk: V[i, k] = sum over the sky directions d of patch k (in d order) of max(0, N_i . D_d) T_d wsky_d (float),
// then G_i (k = P), then dc(b, i) (k = P + 1 + b); split exactly into bf16 hi + mid + lo, rows of Kp (zero padded). A block computes 32
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
  const double* G64;           // used when G is null
  const float* dc;             // [nBins x nc] or null
  __nv_bfloat16* v;            // [3 x nc x Kp]: hi, mid, lo
};

// x = hi + mid + lo exactly (each difference is exact in FP32), each piece round-to-nearest bf16
__device__ __forceinline__ void split3(float x, __nv_bfloat16& hi, __nv_bfloat16& mid, __nv_bfloat16& lo) {
  hi = __float2bfloat16_rn(x);
  const float r = __fsub_rn(x, __bfloat162float(hi));
  mid = __float2bfloat16_rn(r);
  lo = __float2bfloat16_rn(__fsub_rn(r, __bfloat162float(mid)));
}

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
      } else if (k == a.P) v = a.G ? a.G[i] : __double2float_rn(a.G64[i]);
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
      __nv_bfloat16 hi, mid, lo;
      split3(tile[kk][r], hi, mid, lo);
      const size_t at = size_t(ii) * a.Kp + k0 + kk, piece = size_t(a.nc) * a.Kp;
      a.v[at] = hi;
      a.v[at + piece] = mid;
      a.v[at + 2 * piece] = lo;
    }
  }
}

// S^T per chunk (K-major rows of the steps): St[t, k] = S[k, t] (k < P), g[t] (k = P), Sdc[k - P - 1, t]; hi + mid + lo
// into [3 x T x Kp].
__global__ void __launch_bounds__(256) k_build_st(const float* S, const float* g, const float* Sdc, uint32_t P, uint32_t nBins, uint32_t T,
                                                  uint32_t Kp, __nv_bfloat16* st) {
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
    __nv_bfloat16 hi, mid, lo;
    split3(tile[tx][r], hi, mid, lo);
    const size_t at = size_t(t) * Kp + k, piece = size_t(T) * Kp;
    st[at] = hi;
    st[at + piece] = mid;
    st[at + 2 * piece] = lo;
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

// A [rows x Kp] bf16, K contiguous: boxes of 64 (128 B) x boxRows rows, 128-byte swizzle, zero fill past the rows.
static bool make_map(CUtensorMap* m, const void* base, uint64_t rows, uint64_t Kp, uint32_t boxRows) {
  auto fn = encode_fn();
  if (!fn) return false;
  const cuuint64_t dims[2] = {Kp, rows};
  const cuuint64_t strides[1] = {Kp * 2};
  const cuuint32_t box[2] = {BK, boxRows};
  const cuuint32_t estr[2] = {1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

const char* series_tc(const SeriesTcPlan& p, cudaStream_t st) { return series_tc_rows(p, 0, (p.nc + BM - 1) / BM, st); }

// a contraction's parameters (its tensor maps encoded here), tiles from tileBase on; null or what failed
static const char* tc_seg(const SeriesTcPlan& p, uint32_t mBase, uint32_t mCount, uint32_t tileBase, uint32_t sunBase, TcSeg& a,
                          uint32_t& sunBlocks) {
  if (uint64_t(mBase) + mCount > (p.nc + BM - 1) / BM) return "series_tc: rows of tiles beyond the chunk";
  if (p.Kp % BK || !p.Kp) return "series_tc: K not padded to 64";
  if (uint64_t(PIECES) * p.nc + BM > 0x7fffffffull || uint64_t(PIECES) * p.T + BN > 0x7fffffffull) return "series_tc: chunk too large";
  if (!make_map(&a.mapV, p.v, uint64_t(PIECES) * p.nc, p.Kp, BM) || !make_map(&a.mapS, p.s, uint64_t(PIECES) * p.T, p.Kp, BN))
    return "series_tc: cuTensorMapEncodeTiled failed";
  a.nc = p.nc; a.T = p.T; a.Kp = p.Kp;
  a.mTiles = mCount; a.mBase = mBase; a.nTiles = (p.T + BN - 1) / BN; a.tileBase = tileBase;
  const uint32_t rows = std::min<uint32_t>(p.nc, (mBase + mCount) * BM) - mBase * BM;
  a.sunBase = sunBase;
  sunBlocks = ((rows + kSunRows - 1) / kSunRows) * ((p.T + kSunCols - 1) / kSunCols);
  a.sunOfCol = p.sunOfCol; a.sunVec = p.sunVec; a.sunW = p.sunW; a.sun0 = p.sun0;
  a.bits = p.bits; a.bytes = p.bytes; a.N = p.N; a.E = p.E;
  return nullptr;
}

static const char* tc_launch(TcGroup& g, int numSMs, uint64_t waitLimitNs, bool withholdFills, cudaStream_t st) {
  static bool attr = false;
  if (!attr) {
    if (cudaFuncSetAttribute(k_series_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES) != cudaSuccess)
      return "series_tc: cannot reserve shared memory";
    attr = true;
  }
  g.waitLimitNs = waitLimitNs ? std::min(waitLimitNs, kWaitLimitNs) : kWaitLimitNs;
  g.withholdFills = withholdFills ? 1u : 0u;
  const int grid = int(std::min<uint32_t>(uint32_t(numSMs), g.nTiles));
  k_series_tc<<<grid, THREADS, SMEM_BYTES, st>>>(g);
  if (g.nSunBlocks) k_series_sun<<<g.nSunBlocks, 256, 0, st>>>(g);
  return nullptr;
}

const char* series_tc_rows(const SeriesTcPlan& p, uint32_t mBase, uint32_t mCount, cudaStream_t st) {
  if (p.nc == 0 || p.T == 0 || mCount == 0) return nullptr;
  thread_local TcGroup* tg = new TcGroup;   // 18 KB, off the stack; the launch copies it
  TcGroup& G = *tg;
  G.nSegs = 1;
  if (const char* why = tc_seg(p, mBase, mCount, 0, 0, G.seg[0], G.nSunBlocks)) return why;
  G.nTiles = mCount * G.seg[0].nTiles;
  G.status = p.status;
  return tc_launch(G, p.numSMs, p.waitLimitNs, p.withholdFills, st);
}

const char* series_tc_group(const SeriesTcPlan* plans, uint32_t n, cudaStream_t st) {
  if (!n) return nullptr;
  if (n > kMaxTcSegs) return "series_tc: more contractions than one launch holds";
  thread_local TcGroup* tg = new TcGroup;
  TcGroup& G = *tg;
  G.nSegs = 0;
  G.nTiles = 0;
  G.nSunBlocks = 0;
  for (uint32_t k = 0; k < n; ++k) {
    const SeriesTcPlan& p = plans[k];
    if (p.nc == 0 || p.T == 0) continue;
    const uint32_t mCount = (p.nc + BM - 1) / BM;
    uint32_t sunBlocks = 0;
    if (const char* why = tc_seg(p, 0, mCount, G.nTiles, G.nSunBlocks, G.seg[G.nSegs], sunBlocks)) return why;
    G.nTiles += mCount * G.seg[G.nSegs].nTiles;
    G.nSunBlocks += sunBlocks;
    ++G.nSegs;
  }
  if (!G.nSegs) return nullptr;
  G.status = plans[0].status;
  return tc_launch(G, plans[0].numSMs, plans[0].waitLimitNs, plans[0].withholdFills, st);
}

void build_series_operands(const SeriesTcPlan& p, const SeriesOperands& o, cudaStream_t st) {
  VBuildArgs v{};
  v.bits = p.bits; v.bytes = p.bytes; v.nc = p.nc; v.P = o.P; v.nBins = o.nBins; v.Kp = p.Kp; v.N = p.N; v.D = o.D;
  v.patchFirst = o.patchFirst; v.patchDirs = o.patchDirs; v.wsky = o.wsky; v.G = o.G; v.G64 = o.G64; v.dc = o.dc;
  v.v = static_cast<__nv_bfloat16*>(p.v);
  if (o.buildV && p.nc) k_build_v<<<dim3((p.nc + 31) / 32, p.Kp / 64), 256, 0, st>>>(v);
  if (o.rebuildS)
    k_build_st<<<dim3((p.T + 31) / 32, p.Kp / 32), 256, 0, st>>>(o.S, o.g, o.Sdc, o.P, o.nBins, p.T, p.Kp, static_cast<__nv_bfloat16*>(p.s));
}

}  // namespace kgb
