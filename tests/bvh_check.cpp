// Test helper (compiled by tests/test_bvh_layout.py with the engine's host builder): checks the 8-wide BVH the GPU
// kernels walk, on the CPU, decoding the records exactly as kit-sim_daylight_gb300/csrc/rt.cuh does.
//  - every inner child index < nNodes and every node but the root is some node's child exactly once;
//  - every leaf's triangle range lies within the records, every triangle record appears exactly once;
//  - every child box (float planes) contains its subtree's triangles, and every empty slot holds the empty box;
//  - the depth fits the traversal stacks (48 node groups any-hit, 192 entries closest-hit).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../kit-sim_daylight_gb300/csrc/engine.h"

using namespace kgb;

extern "C" int bvh_check(const float* v, size_t nv, const uint32_t* tri, size_t nt, char* msg, size_t msgLen, uint32_t* depthOut) {
  BvhOut b;
  build_bvh8(v, nv, tri, nt, nullptr, nullptr, b);
  const auto bad = [&](const char* what, long a, long c) { std::snprintf(msg, msgLen, "%s (%ld, %ld)", what, a, c); return 1; };
  if (!nt) return b.nNodes == 0 ? 0 : bad("empty scene with nodes", b.nNodes, 0);
  const uint32_t N = b.nNodes, T = uint32_t(b.tris.size() / 12);
  if (b.nodes.size() != size_t(N) * kNodeWords) return bad("node words", long(b.nodes.size()), N);
  if (N >= kMaxNodes) return bad("node count beyond the 24-bit child index", long(N), 0);
  if (T != nt) return bad("triangle records", T, long(nt));
  std::vector<int> parentSeen(N, 0), triSeen(T, 0), primSeen(nt, 0);
  std::vector<uint32_t> depth(N, 0);
  uint32_t maxDepth = 0;
  // subtree triangle boxes, bottom-up is not needed: check each child box against each triangle it leads to
  std::vector<std::vector<uint32_t>> subtreeTris(N);
  // breadth-first order: children have larger indices, so walk from the last node to the first
  for (int64_t w = int64_t(N) - 1; w >= 0; --w) {
    const uint32_t* r = &b.nodes[size_t(w) * kNodeWords];
    const uint32_t imask = r[0] >> 24, childBase = r[0] & 0xffffffu, triBase = r[1];
    const uint32_t slots = 1 + (((r[2] >> 7) & 1u) | ((r[2] >> 14) & 2u) | ((r[2] >> 21) & 4u));
    uint32_t innerRank = 0;
    for (int k = 0; k < 8; ++k) {
      const uint32_t meta = ((k < 4 ? r[2] : r[3]) >> (8 * (k & 3))) & 0x7fu;   // bit 7: the slot count's
      const auto plane = [&](int f) { float x; std::memcpy(&x, &r[4 + 8 * f + k], 4); return double(x); };   // lo.x hi.x lo.y ..
      double lo[3], hi[3];
      for (int a = 0; a < 3; ++a) { lo[a] = plane(2 * a); hi[a] = plane(2 * a + 1); }
      const bool empty = !((imask >> k) & 1u) && !meta;
      if (!empty && uint32_t(k) >= slots) return bad("a child past the node's slot count", long(w), k);
      if (empty) {
        for (int a = 0; a < 3; ++a)
          if (!(std::isinf(lo[a]) && lo[a] > 0 && std::isinf(hi[a]) && hi[a] < 0)) return bad("empty slot with a box", long(w), k);
        continue;
      }
      std::vector<uint32_t> under;
      if ((imask >> k) & 1u) {
        const uint32_t c = childBase + innerRank++;
        if (c >= N || c <= uint32_t(w)) return bad("inner child index", long(w), long(c));
        if (parentSeen[c]++) return bad("node with two parents", long(c), 0);
        under = subtreeTris[c];
      } else if (meta) {
        const uint32_t cnt = meta >> 5, off = meta & 31u;
        if (cnt < 1 || cnt > 3 || off + cnt > 24) return bad("leaf meta", long(w), long(meta));
        for (uint32_t j = triBase + off; j < triBase + off + cnt; ++j) {
          if (j >= T) return bad("triangle record index", long(w), long(j));
          if (triSeen[j]++) return bad("triangle record in two leaves", long(j), 0);
          uint32_t prim;
          std::memcpy(&prim, &b.tris[size_t(j) * 12 + 3], 4);
          if (prim >= nt) return bad("primitive index", long(j), long(prim));
          if (primSeen[prim]++) return bad("primitive twice", long(prim), 0);
          under.push_back(j);
        }
      } else continue;
      for (uint32_t j : under)
        for (int vtx = 0; vtx < 3; ++vtx)
          for (int a = 0; a < 3; ++a) {
            const double x = b.tris[size_t(j) * 12 + 4 * vtx + a];
            if (x < lo[a] || x > hi[a]) return bad("child box misses a triangle", long(w), long(j));
          }
      subtreeTris[w].insert(subtreeTris[w].end(), under.begin(), under.end());
    }
  }
  for (uint32_t c = 1; c < N; ++c) if (parentSeen[c] != 1) return bad("orphan node", long(c), parentSeen[c]);
  for (uint32_t j = 0; j < T; ++j) if (triSeen[j] != 1) return bad("unreferenced triangle record", long(j), 0);
  for (uint32_t w = 0; w < N; ++w) {   // depth, top-down
    const uint32_t* r = &b.nodes[size_t(w) * kNodeWords];
    const uint32_t imask = r[0] >> 24;
    uint32_t k = 0;
    for (int c = 0; c < 8; ++c) if ((imask >> c) & 1u) depth[(r[0] & 0xffffffu) + k++] = depth[w] + 1;
    maxDepth = std::max(maxDepth, depth[w]);
  }
  *depthOut = maxDepth;
  if (maxDepth + 1 > 27) return bad("depth beyond the traversal stacks", long(maxDepth), 27);
  msg[0] = 0;
  return 0;
}
