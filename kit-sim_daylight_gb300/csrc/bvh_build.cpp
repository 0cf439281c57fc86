// Host builder of the engine's acceleration structure: a binned-SAH binary BVH (32 bins on the widest centroid axis,
// leaves of at most 3 triangles) collapsed to 8-wide nodes (each inner node adopts the children of its largest-area
// inner child until it has 8) with child boxes quantised to 8 bits against a power-of-two step per axis (the compressed
// wide BVH of Ylitie, Karras, Laine 2017), stored as the 80-byte node / 48-byte triangle records rt.cuh reads.
//
// Conservative by construction: every triangle box is expanded by 2^-16 x the scene's largest coordinate (256 ulps at
// that magnitude) before anything is built, and quantisation rounds outwards, so a box test never drops a triangle the
// watertight test would report; the traversal then equals the brute-force hit set on any input.
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

// One quantised axis: the step s = 2^(eb - 127) with p + 255 s covering the node's extent.
void quant_axis(float p, float hi, uint32_t& eb, float& s) {
  const double ext = std::max(double(hi) - double(p), 1e-30);
  int e = 0;
  std::frexp(ext / 255.0, &e);   // ext / 255 < 2^e
  e = std::max(-126, std::min(127, e));
  for (;;) {
    s = std::ldexp(1.f, e);
    if (double(p) + 255.0 * double(s) >= double(hi) || e >= 127) break;
    ++e;
  }
  eb = uint32_t(e + 127);
}

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
    Box box;
    for (int k = 0; k < n; ++k) box.grow(B.nodes[size_t(ch[k])].box);
    uint32_t rec[20] = {};
    float p[3];
    uint32_t eb[3];
    float s[3];
    for (int a = 0; a < 3; ++a) { p[a] = box.lo[a]; quant_axis(p[a], box.hi[a], eb[a], s[a]); }
    uint32_t imask = 0, meta[8] = {};
    const uint32_t childBase = uint32_t(wideSrc.size()), triBase = uint32_t(tris.size() / 12);
    uint32_t triOff = 0;
    uint8_t q[6][8];
    std::memset(q, 0, sizeof q);
    for (int k = 0; k < n; ++k) {
      const Node2& c = B.nodes[size_t(ch[k])];
      for (int a = 0; a < 3; ++a) {
        const double lo = std::floor((double(c.box.lo[a]) - double(p[a])) / double(s[a]));
        const double hi = std::ceil((double(c.box.hi[a]) - double(p[a])) / double(s[a]));
        q[a][k] = uint8_t(std::max(0.0, std::min(255.0, lo)));
        q[3 + a][k] = uint8_t(std::max(0.0, std::min(255.0, hi)));
      }
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
    std::memcpy(&rec[0], &p[0], 4); std::memcpy(&rec[1], &p[1], 4); std::memcpy(&rec[2], &p[2], 4);
    rec[3] = eb[0] | (eb[1] << 8) | (eb[2] << 16) | (imask << 24);
    rec[4] = childBase;
    rec[5] = triBase;
    rec[6] = meta[0] | (meta[1] << 8) | (meta[2] << 16) | (meta[3] << 24);
    rec[7] = meta[4] | (meta[5] << 8) | (meta[6] << 16) | (meta[7] << 24);
    // n2: qlo.x[8] qlo.y[8]; n3: qlo.z[8] qhi.x[8]; n4: qhi.y[8] qhi.z[8]
    const int order[6] = {0, 1, 2, 3, 4, 5};
    for (int f = 0; f < 6; ++f) {
      const int src = order[f];
      rec[8 + 2 * f] = uint32_t(q[src][0]) | (uint32_t(q[src][1]) << 8) | (uint32_t(q[src][2]) << 16) | (uint32_t(q[src][3]) << 24);
      rec[9 + 2 * f] = uint32_t(q[src][4]) | (uint32_t(q[src][5]) << 8) | (uint32_t(q[src][6]) << 16) | (uint32_t(q[src][7]) << 24);
    }
    nodes.insert(nodes.end(), rec, rec + 20);
  }
  out.nNodes = uint32_t(wideSrc.size());
}

}  // namespace kgb
