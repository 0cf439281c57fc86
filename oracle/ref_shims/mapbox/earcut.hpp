/* TEST INFRASTRUCTURE ONLY. Stand-in for mapbox earcut (v2.2.4, fetched by the reference's CMake and absent here):
 * faces of 5 or more corners triangulate to nothing. Every workload of the oracle harness is triangles and quads,
 * which the reference triangulates without earcut (src/mesh.cpp:154-165). */
#pragma once
#include <vector>
namespace mapbox {
template <typename N = unsigned, typename P>
std::vector<N> earcut(const P&) { return {}; }
}
