// Direction-major device buffers to sensor-major rows: out[i K + d] = in[d ld + i] for d < K, i < m.
//
// The engine keeps per-ray results direction-major ([K x nc]: view classes and distances, visibility bytes, bit words),
// the layout the reduces read coalesced. Callers that dump them want one row per sensor ([nc x K]): the reference
// transposes on the host (gpu.cu:720-734 for gpu_download_view, run.cpp:659-671 for --dump-bits), which at 50k sensors
// x 10,800 rays is seconds of strided host loops. Here the transpose is a tiled kernel: a block stages a TILE x TILE
// tile in shared memory, reading rows of the input and writing rows of the output, both contiguous; the padding keeps
// the column reads of the tile on distinct banks. It moves each byte once each way, so HBM bounds it (algorithmic
// bytes 2 x m x K x element size).
#include "engine.h"

namespace kgb {

template <typename T, int TILE, int PAD>
__global__ void __launch_bounds__(256) k_rows(const T* __restrict__ in, size_t ld, T* __restrict__ out, uint32_t K, uint32_t m) {
  __shared__ T tile[TILE][TILE + PAD];
  const uint32_t d0 = blockIdx.y * TILE, i0 = blockIdx.x * TILE;
  for (uint32_t idx = threadIdx.x; idx < TILE * TILE; idx += 256) {
    const uint32_t r = idx / TILE, c = idx % TILE;   // r: direction in the tile, c: sensor
    if (d0 + r < K && i0 + c < m) tile[r][c] = in[size_t(d0 + r) * ld + i0 + c];
  }
  __syncthreads();
  for (uint32_t idx = threadIdx.x; idx < TILE * TILE; idx += 256) {
    const uint32_t c = idx / TILE, r = idx % TILE;   // c: sensor, r: direction
    if (d0 + r < K && i0 + c < m) out[size_t(i0 + c) * K + d0 + r] = tile[r][c];
  }
}

// 1-byte elements: 64 x 64 tiles (rows of 64 B), 68-byte rows in shared memory (17 words: odd, so a warp's 32 column
// reads fall on 32 banks); 4-byte elements: 32 x 32 tiles (rows of 128 B), 33-word rows.
bool launch_rows(const void* in, size_t ld, void* out, size_t esize, uint32_t K, uint32_t m, cudaStream_t st) {
  const int tile = esize == 1 ? 64 : 32;
  const size_t gy = (size_t(K) + tile - 1) / tile, gx = (size_t(m) + tile - 1) / tile;
  if (!K || !m) return true;
  if (gy > 65535 || (esize != 1 && esize != 4)) return false;
  const dim3 grid{unsigned(gx), unsigned(gy), 1u};
  if (esize == 1) k_rows<uint8_t, 64, 4><<<grid, 256, 0, st>>>(static_cast<const uint8_t*>(in), ld, static_cast<uint8_t*>(out), K, m);
  else k_rows<uint32_t, 32, 1><<<grid, 256, 0, st>>>(static_cast<const uint32_t*>(in), ld, static_cast<uint32_t*>(out), K, m);
  return true;
}

}  // namespace kgb
