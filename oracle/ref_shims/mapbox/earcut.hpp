/* TEST INFRASTRUCTURE ONLY. Stand-in for mapbox earcut (v2.2.4, fetched by the reference's CMake and absent here) for
 * the reference's host code compiled by oracle/Makefile: the polygon's first ring through the engine's restatement of
 * earcut's algorithm (include/kgb_earcut.h, the code the device triangulation runs), so that the reference's own
 * n-gon tests (tests/check_mesh.cpp) run on it. Holes are not restated: the reference passes one ring
 * (src/mesh.cpp:161-162). */
#pragma once
#include <vector>
#include "kgb_earcut.h"
namespace mapbox {
template <typename N = unsigned, typename P>
std::vector<N> earcut(const P& poly) {
  if (poly.empty() || poly[0].size() < 3) return {};
  const int32_t n = int32_t(poly[0].size());
  std::vector<double> xy(2 * size_t(n));
  for (int32_t k = 0; k < n; ++k) { xy[2 * size_t(k)] = poly[0][size_t(k)][0]; xy[2 * size_t(k) + 1] = poly[0][size_t(k)][1]; }
  std::vector<kgb_earcut::Node> pool(2 * size_t(n) + 16);
  std::vector<int32_t> stack(2 * size_t(n) + 16);
  std::vector<uint32_t> tri(3 * size_t(2 * n + 8));
  const int made = kgb_earcut::earcut_ring(xy.data(), n, pool.data(), int32_t(pool.size()), stack.data(), int32_t(stack.size()), tri.data(),
                                           int32_t(tri.size() / 3));
  if (made <= 0) return {};
  return std::vector<N>(tri.begin(), tri.begin() + 3 * made);
}
}  // namespace mapbox
