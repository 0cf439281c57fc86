// Host builder of the engine's acceleration structure: a binned-SAH binary BVH (32 bins on the widest centroid axis,
// leaves of at most 3 triangles) collapsed to 8-wide nodes (each inner node adopts the children of its largest-area
// inner child until it has 8) with float child boxes, stored as the 208-byte node / 48-byte triangle records rt.cuh
// reads.
//
// Conservative by construction: every triangle box is expanded by 2^-16 x the scene's largest coordinate (256 ulps at
// that magnitude) before anything is built, so a box test never drops a triangle the watertight test would report;
// the traversal then equals the brute-force hit set on any input.
#include "engine.h"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace kgb {
namespace {

struct Box {
  float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  void grow(const Box& b) { for (int a = 0; a < 3; ++a) { lo[a] = std::min(lo[a], b.lo[a]); hi[a] = std::max(hi[a], b.hi[a]); } }
  float area() const {
    const float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
    return dx < 0.f ? 0.f : dx * dy + dy * dz + dz * dx;
  }
};
struct Node2 { Box box; int left = -1, right = -1; uint32_t first = 0, count = 0; };   // count > 0: leaf

struct Builder {
  std::vector<Box> tb;
  std::vector<float> cen;   // 3 per triangle
  std::vector<uint32_t> idx;
  std::vector<Node2> nodes;

  int build(uint32_t first, uint32_t count) {
    const int me = int(nodes.size());
    nodes.push_back(Node2{});
    Box box, cb;
    for (uint32_t j = first; j < first + count; ++j) {
      const uint32_t k = idx[j];
      box.grow(tb[k]);
      Box c;
      for (int a = 0; a < 3; ++a) c.lo[a] = c.hi[a] = cen[3 * k + a];
      cb.grow(c);
    }
    nodes[me].box = box;
    if (count <= 3) { nodes[me].first = first; nodes[me].count = count; return me; }
    int axis = 0;
    for (int a = 1; a < 3; ++a) if (cb.hi[a] - cb.lo[a] > cb.hi[axis] - cb.lo[axis]) axis = a;
    uint32_t split = 0;
    if (cb.hi[axis] > cb.lo[axis]) {
      constexpr int NB = 32;
      Box bb[NB];
      uint32_t bc[NB] = {};
      const float lo = cb.lo[axis], scale = float(NB) / (cb.hi[axis] - cb.lo[axis]);
      const auto bin = [&](uint32_t k) { return std::min(NB - 1, int((cen[3 * k + axis] - lo) * scale)); };
      for (uint32_t j = first; j < first + count; ++j) { const int b = bin(idx[j]); bc[b]++; bb[b].grow(tb[idx[j]]); }
      float rightA[NB];
      uint32_t rightN[NB];
      Box acc;
      uint32_t n = 0;
      for (int b = NB - 1; b > 0; --b) { acc.grow(bb[b]); n += bc[b]; rightA[b] = acc.area(); rightN[b] = n; }
      Box l;
      uint32_t nl = 0;
      float best = INFINITY;
      int bestB = -1;
      for (int b = 1; b < NB; ++b) {
        l.grow(bb[b - 1]); nl += bc[b - 1];
        if (!nl || !rightN[b]) continue;
        const float c = float(nl) * l.area() + float(rightN[b]) * rightA[b];
        if (c < best) { best = c; bestB = b; }
      }
      if (bestB > 0) {
        auto mid = std::partition(idx.begin() + first, idx.begin() + first + count, [&](uint32_t k) { return bin(k) < bestB; });
        split = uint32_t(mid - idx.begin()) - first;
      }
    }
    if (split == 0 || split == count) {   // no usable SAH split (coincident centroids): halves of the widest axis's order
      split = count / 2;
      std::nth_element(idx.begin() + first, idx.begin() + first + split, idx.begin() + first + count,
                       [&](uint32_t a, uint32_t b) { return cen[3 * a + axis] < cen[3 * b + axis]; });
    }
    const int L = build(first, split);
    const int R = build(first + split, count - split);
    nodes[me].left = L;
    nodes[me].right = R;
    return me;
  }
};

}  // namespace

void build_bvh8(const float* v, size_t nv, const uint32_t* tri, size_t nt, const uint32_t* slot, const uint8_t* translucent, BvhOut& out) {
  out = BvhOut{};
  if (!nt) return;
  Builder B;
  float M = 1.f;
  for (size_t k = 0; k < 3 * nv; ++k) M = std::max(M, std::fabs(v[k]));
  const float eps = M * (1.f / 65536.f);
  B.tb.resize(nt); B.cen.resize(3 * nt); B.idx.resize(nt);
  for (size_t k = 0; k < nt; ++k) {
    B.idx[k] = uint32_t(k);
    for (int a = 0; a < 3; ++a) {
      const float x0 = v[3 * tri[3 * k] + a], x1 = v[3 * tri[3 * k + 1] + a], x2 = v[3 * tri[3 * k + 2] + a];
      const float lo = std::min({x0, x1, x2}), hi = std::max({x0, x1, x2});
      B.tb[k].lo[a] = lo - eps; B.tb[k].hi[a] = hi + eps;
      B.cen[3 * k + a] = 0.5f * lo + 0.5f * hi;
    }
  }
  B.nodes.reserve(2 * nt);
  B.build(0, uint32_t(nt));

  // collapse: a wide node's children are BVH2 nodes (inner or leaf), at most 8
  struct Wide { int src; };   // the BVH2 node it was made from
  std::vector<int> wideSrc;   // wide node -> BVH2 node
  std::vector<uint32_t>& nodes = out.nodes;
  std::vector<float>& tris = out.tris;
  wideSrc.push_back(0);
  // children of wide node w, as BVH2 indices; computed on emission
  const auto children = [&](int src, int* ch) {
    int n = 0;
    const Node2& s = B.nodes[size_t(src)];
    if (s.count) { ch[n++] = src; return n; }   // a leaf root: one leaf child
    ch[n++] = s.left; ch[n++] = s.right;
    while (n < 8) {
      int bestK = -1;
      float bestA = -1.f;
      for (int k = 0; k < n; ++k) {
        const Node2& c = B.nodes[size_t(ch[k])];
        if (!c.count && c.box.area() > bestA) { bestA = c.box.area(); bestK = k; }
      }
      if (bestK < 0) break;
      const Node2& c = B.nodes[size_t(ch[bestK])];
      ch[bestK] = c.left;
      ch[n++] = c.right;
    }
    return n;
  };
  // breadth-first emission: wide node w's inner children are allocated as one consecutive block
  for (size_t w = 0; w < wideSrc.size(); ++w) {
    int ch[8];
    const int n = children(wideSrc[w], ch);
    uint32_t rec[kNodeWords] = {};
    uint32_t imask = 0, meta[8] = {};
    const uint32_t childBase = uint32_t(wideSrc.size()), triBase = uint32_t(tris.size() / 12);
    uint32_t triOff = 0;
    float plane[6][8];   // lo.x hi.x lo.y hi.y lo.z hi.z of each child; empty slots +inf / -inf
    for (int k = 0; k < 8; ++k)
      for (int a = 0; a < 3; ++a) { plane[2 * a][k] = INFINITY; plane[2 * a + 1][k] = -INFINITY; }
    for (int k = 0; k < n; ++k) {
      const Node2& c = B.nodes[size_t(ch[k])];
      for (int a = 0; a < 3; ++a) { plane[2 * a][k] = c.box.lo[a]; plane[2 * a + 1][k] = c.box.hi[a]; }
      if (!c.count) {
        imask |= 1u << k;
        wideSrc.push_back(ch[k]);
      } else {
        meta[k] = (c.count << 5) | triOff;
        for (uint32_t j = c.first; j < c.first + c.count; ++j) {
          const uint32_t t = B.idx[j];
          float r[12];
          for (int vtx = 0; vtx < 3; ++vtx)
            for (int a = 0; a < 3; ++a) r[4 * vtx + a] = v[3 * tri[3 * t + vtx] + a];
          uint32_t extra[3] = {t, translucent && translucent[t] ? 1u : 0u, slot ? slot[t] : 0u};
          for (int vtx = 0; vtx < 3; ++vtx) std::memcpy(&r[4 * vtx + 3], &extra[vtx], 4);
          tris.insert(tris.end(), r, r + 12);
        }
        triOff += c.count;
      }
    }
    rec[0] = childBase | (imask << 24);   // fewer than 2^24 nodes: the engine checks the triangle count first
    rec[1] = triBase;
    for (int b = 0; b < 3; ++b) meta[b] |= ((uint32_t(n - 1) >> b) & 1u) << 7;   // the slot count (n >= 1), on slots in use
    rec[2] = meta[0] | (meta[1] << 8) | (meta[2] << 16) | (meta[3] << 24);
    rec[3] = meta[4] | (meta[5] << 8) | (meta[6] << 16) | (meta[7] << 24);
    std::memcpy(&rec[4], plane, sizeof plane);   // n1 n2 lo.x, n3 n4 hi.x, n5 n6 lo.y, ...
    nodes.insert(nodes.end(), rec, rec + kNodeWords);
  }
  out.nNodes = uint32_t(wideSrc.size());
}

}  // namespace kgb
