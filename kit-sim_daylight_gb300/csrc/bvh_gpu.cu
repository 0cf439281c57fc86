// Device builder of the engine's acceleration structure (the reference's gpu_build, gpu.cu:386-457, builds an OptiX
// GAS on the device; this is the GB300 counterpart): a linear BVH over Morton codes (Karras 2012), refined by treelet
// restructuring, collapsed to the
// 8-wide nodes with float child boxes and the 48-byte triangle records that rt.cuh reads, the same layout as the host
// builder (bvh_build.cpp) makes.
//
//   1. |coordinates| maximum -> eps = max(1, M) / 65536 (the host builder's expansion)
//   2. per triangle: box (expanded by eps), centroid; centroid bounds
//   3. 63-bit Morton codes of the centroids, radix-sorted with the triangle index (stable: ties keep index order)
//   4. binary radix tree (Karras 2012): internal node i's range and split from common prefixes of the sorted codes
//   5. boxes, triangle counts and SAH costs bottom-up (each leaf walks towards the root, the second arrival at a node
//      refits it from its children), then ten such passes that also restructure each node's treelet of up to 7
//      leaves to its least-SAH topology (Karras & Aila 2013)
//   6. SAH-optimal collapse to 8-wide nodes (Ylitie, Karras & Laine 2017): a bottom-up dynamic program gives each
//      binary node the least SAH cost of its subtree as at most i = 1..8 children of a wide node, and whether one slot
//      holds it as a leaf (at most 3 triangles) or as a wide node of its own; level by level, each wide node's children
//      follow those choices (leaf triangles gathered by a walk: restructured subtrees are no longer ranges of the
//      sorted order), and a prefix sum over the level gives each node its block of inner children and of triangle
//      records, so the layout is deterministic
//   7. each node's child boxes written as floats (the expanded boxes of step 2, merged), empty slots +inf / -inf
// Conservative exactly as the host builder: any conservative BVH gives the traversal the brute-force hit set, so the
// results do not depend on which builder made the scene.
#include "engine.h"

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

namespace kgb {
namespace {

constexpr uint32_t kLeafMax = 3;   // triangles per leaf, as the host builder
constexpr int kTreeletPasses = 10; // bottom-up passes of treelet restructuring (views city: 3 passes 3.2 G rays/s, 10 passes 3.7)

__device__ __forceinline__ uint32_t ord(float f) {   // order-preserving float -> uint
  const uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float unord(uint32_t u) { return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u); }

__global__ void k_maxabs(const float* v, size_t n, uint32_t* out) {
  uint32_t m = 0;
  for (size_t k = blockIdx.x * size_t(blockDim.x) + threadIdx.x; k < n; k += size_t(gridDim.x) * blockDim.x)
    m = max(m, __float_as_uint(fabsf(v[k])));   // non-negative floats order as their bits
  for (int s = 16; s; s >>= 1) m = max(m, __shfl_xor_sync(~0u, m, s));
  if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

// triangle boxes (expanded), centroids (of the unexpanded box, as the host), centroid bounds (ordered uints)
__global__ void k_prims(const float* v, const uint32_t* tri, uint32_t nt, float eps, float4* lo, float4* hi, float4* cen, uint32_t* cb) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t cmin[3] = {~0u, ~0u, ~0u}, cmax[3] = {0u, 0u, 0u};
  if (t < nt) {
    float l[3], h[3], c[3];
    for (int a = 0; a < 3; ++a) {
      const float x0 = v[3 * tri[3 * t] + a], x1 = v[3 * tri[3 * t + 1] + a], x2 = v[3 * tri[3 * t + 2] + a];
      const float mn = fminf(x0, fminf(x1, x2)), mx = fmaxf(x0, fmaxf(x1, x2));
      l[a] = __fsub_rn(mn, eps); h[a] = __fadd_rn(mx, eps);
      c[a] = __fadd_rn(__fmul_rn(0.5f, mn), __fmul_rn(0.5f, mx));
      cmin[a] = cmax[a] = ord(c[a]);
    }
    lo[t] = make_float4(l[0], l[1], l[2], 0.f);
    hi[t] = make_float4(h[0], h[1], h[2], 0.f);
    cen[t] = make_float4(c[0], c[1], c[2], 0.f);
  }
  for (int a = 0; a < 3; ++a) {
    for (int s = 16; s; s >>= 1) {
      cmin[a] = min(cmin[a], __shfl_xor_sync(~0u, cmin[a], s));
      cmax[a] = max(cmax[a], __shfl_xor_sync(~0u, cmax[a], s));
    }
    if ((threadIdx.x & 31) == 0) { atomicMin(&cb[a], cmin[a]); atomicMax(&cb[3 + a], cmax[a]); }
  }
}

__device__ __forceinline__ uint64_t spread21(uint64_t x) {   // 21 bits -> every third bit of 63
  x &= 0x1fffffull;
  x = (x | (x << 32)) & 0x1f00000000ffffull;
  x = (x | (x << 16)) & 0x1f0000ff0000ffull;
  x = (x | (x << 8)) & 0x100f00f00f00f00full;
  x = (x | (x << 4)) & 0x10c30c30c30c30c3ull;
  x = (x | (x << 2)) & 0x1249249249249249ull;
  return x;
}
__global__ void k_morton(const float4* cen, uint32_t nt, const uint32_t* cb, uint64_t* key, uint32_t* val) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nt) return;
  const float4 c = cen[t];
  const float cc[3] = {c.x, c.y, c.z};
  uint64_t code = 0;
  for (int a = 0; a < 3; ++a) {
    const float lo = unord(cb[a]), hi = unord(cb[3 + a]);
    const float ext = hi - lo;
    float u = ext > 0.f ? (cc[a] - lo) / ext : 0.f;
    u = fminf(fmaxf(u, 0.f), 1.f);
    code |= spread21(uint64_t(fminf(u * 2097152.f, 2097151.f))) << (2 - a);
  }
  key[t] = code;
  val[t] = t;
}

// Karras 2012: internal node i (0 <= i < n - 1) over sorted keys; ties broken by position. A child c >= 0 is an
// internal node, c < 0 the leaf ~c (a position in the sorted order).
__device__ __forceinline__ int delta(const uint64_t* k, int n, int i, long long j) {
  if (j < 0 || j >= n) return -1;
  const uint64_t a = k[i], b = k[size_t(j)];
  return a == b ? 64 + __clz(uint32_t(i) ^ uint32_t(j)) : __clzll(a ^ b);
}
__global__ void k_karras(const uint64_t* k, int n, int* left, int* right, int* parent, int* leafParent, int2* range) {
  const int i = int(blockIdx.x * blockDim.x + threadIdx.x);
  if (i >= n - 1) return;
  const int d = delta(k, n, i, i + 1) - delta(k, n, i, i - 1) >= 0 ? 1 : -1;
  const int dmin = delta(k, n, i, i - d);
  long long lmax = 2;
  while (lmax < 2ll * n && delta(k, n, i, i + lmax * d) > dmin) lmax *= 2;   // at most log2(2n) doublings
  long long l = 0;
  for (long long t = lmax / 2; t >= 1; t /= 2)
    if (delta(k, n, i, i + (l + t) * d) > dmin) l += t;
  const int j = int(i + l * d);
  const int dnode = delta(k, n, i, j);
  long long s = 0;
  for (long long div = 2;; div *= 2) {
    const long long t = (l + div - 1) / div;
    if (delta(k, n, i, i + (s + t) * d) > dnode) s += t;
    if (t <= 1) break;
  }
  const int gamma = int(i + s * d + min(d, 0));
  const int first = min(i, j), last = max(i, j);
  const int L = first == gamma ? ~gamma : gamma, R = last == gamma + 1 ? ~(gamma + 1) : gamma + 1;
  left[i] = L;
  right[i] = R;
  range[i] = make_int2(first, last);
  if (L >= 0) parent[L] = i; else leafParent[~L] = i;
  if (R >= 0) parent[R] = i; else leafParent[~R] = i;
  if (i == 0) parent[0] = -1;
}

// SAH constants of the binary tree's cost (relative): a box test, a triangle test
constexpr float kCi = 1.2f, kCt = 1.0f;

__device__ __forceinline__ float box_area(float4 lo, float4 hi) {
  const float dx = hi.x - lo.x, dy = hi.y - lo.y, dz = hi.z - lo.z;
  return dx < 0.f ? 0.f : dx * dy + dy * dz + dz * dx;
}

// the binary tree being built: child c >= 0 an internal node, c < 0 the leaf ~c (a sorted position)
struct Tree2 {
  int *left, *right, *parent, *leafParent;
  float4 *nlo, *nhi;
  uint32_t* count;   // triangles under an internal node
  float* cost;       // SAH cost of its subtree (a set of at most 3 triangles costs as one leaf)
  const uint32_t* order;
  const float4 *plo, *phi;
};
__device__ __forceinline__ void child_info(const Tree2& T, int c, float4& lo, float4& hi, uint32_t& cnt, float& cst) {
  if (c >= 0) { lo = __ldcg(&T.nlo[c]); hi = __ldcg(&T.nhi[c]); cnt = __ldcg(&T.count[c]); cst = __ldcg(&T.cost[c]); }
  else { lo = T.plo[T.order[~c]]; hi = T.phi[T.order[~c]]; cnt = 1; cst = kCt * box_area(lo, hi); }
}
// box, count and cost of internal node x from its children
__device__ __forceinline__ void refit(const Tree2& T, int x) {
  float4 a, b, c, d;
  uint32_t na, nb;
  float ca, cb;
  child_info(T, __ldcg(&T.left[x]), a, b, na, ca);
  child_info(T, __ldcg(&T.right[x]), c, d, nb, cb);
  const float4 lo = make_float4(fminf(a.x, c.x), fminf(a.y, c.y), fminf(a.z, c.z), 0.f);
  const float4 hi = make_float4(fmaxf(b.x, d.x), fmaxf(b.y, d.y), fmaxf(b.z, d.z), 0.f);
  const uint32_t n = na + nb;
  const float A = box_area(lo, hi);
  __stcg(&T.nlo[x], lo);
  __stcg(&T.nhi[x], hi);
  __stcg(&T.count[x], n);
  __stcg(&T.cost[x], n <= kLeafMax ? kCt * A * float(n) : kCi * A + ca + cb);
}

// Treelet restructuring (Karras & Aila 2013): the treelet of node x has up to 7 leaves (grown by opening the
// largest-area internal leaf); a dynamic program over the subsets of its leaves finds the binary topology of least SAH
// cost, and the treelet's internal nodes are rewired to it when that is cheaper. Subsets of at most 3 triangles cost
// as the one 8-wide leaf they become.
__device__ void optimize_treelet(const Tree2& T, int x) {
  int leaf[7], inner[6];
  int m = 0, ni = 0;
  inner[ni++] = x;
  leaf[m++] = __ldcg(&T.left[x]);
  leaf[m++] = __ldcg(&T.right[x]);
  while (m < 7) {
    int best = -1;
    float bestA = -1.f;
    for (int k = 0; k < m; ++k) {
      const int c = leaf[k];
      if (c < 0 || __ldcg(&T.count[c]) <= kLeafMax) continue;
      const float A = box_area(__ldcg(&T.nlo[c]), __ldcg(&T.nhi[c]));
      if (A > bestA) { bestA = A; best = k; }
    }
    if (best < 0) break;
    const int c = leaf[best];
    inner[ni++] = c;
    leaf[best] = __ldcg(&T.left[c]);
    leaf[m++] = __ldcg(&T.right[c]);
  }
  if (m < 4) return;
  float4 llo[7], lhi[7];
  uint32_t lcnt[7];
  float lcost[7];
  for (int k = 0; k < m; ++k) child_info(T, leaf[k], llo[k], lhi[k], lcnt[k], lcost[k]);
  float cst[128];
  uint8_t part[128];
  const uint32_t full = (1u << m) - 1u;
  for (uint32_t S = 1; S <= full; ++S) {   // a proper subset precedes its superset
    float4 lo = make_float4(INFINITY, INFINITY, INFINITY, 0.f), hi = make_float4(-INFINITY, -INFINITY, -INFINITY, 0.f);
    uint32_t n = 0;
    for (int k = 0; k < m; ++k)
      if (S >> k & 1u) {
        lo = make_float4(fminf(lo.x, llo[k].x), fminf(lo.y, llo[k].y), fminf(lo.z, llo[k].z), 0.f);
        hi = make_float4(fmaxf(hi.x, lhi[k].x), fmaxf(hi.y, lhi[k].y), fmaxf(hi.z, lhi[k].z), 0.f);
        n += lcnt[k];
      }
    const uint32_t low = S & (0u - S);
    if (S == low) { cst[S] = lcost[__ffs(S) - 1]; part[S] = 0; continue; }
    float best = INFINITY;
    uint32_t bp = low;
    for (uint32_t P = (S - 1) & S; P; P = (P - 1) & S)
      if (P & low) { const float c = cst[P] + cst[S ^ P]; if (c < best) { best = c; bp = P; } }
    const float A = box_area(lo, hi);
    cst[S] = n <= kLeafMax ? kCt * A * float(n) : kCi * A + best;
    part[S] = uint8_t(bp);
  }
  if (!(cst[full] < __ldcg(&T.cost[x]) * 0.9999f)) return;   // keep the tree unless the treelet improves
  // rewire top-down (x stays the root), then refit bottom-up in reverse order of assignment
  uint32_t setOf[6];
  int nodeOf[6], order[6];
  int sp = 0, next = 1, done = 0;
  setOf[0] = full; nodeOf[0] = x; sp = 1;
  while (sp) {
    --sp;
    const uint32_t S = setOf[sp];
    const int node = nodeOf[sp];
    order[done++] = node;
    const uint32_t P[2] = {part[S], S ^ part[S]};
    int id[2];
    for (int h = 0; h < 2; ++h) {
      if (__popc(P[h]) == 1) id[h] = leaf[__ffs(P[h]) - 1];
      else { id[h] = inner[next++]; setOf[sp] = P[h]; nodeOf[sp] = id[h]; ++sp; }
      if (id[h] >= 0) __stcg(&T.parent[id[h]], node); else __stcg(&T.leafParent[~id[h]], node);
    }
    __stcg(&T.left[node], id[0]);
    __stcg(&T.right[node], id[1]);
  }
  for (int k = done - 1; k >= 0; --k) refit(T, order[k]);
}

// bottom-up pass: the second thread to arrive at a node refits it from its children and, when asked, restructures
// its treelet (every node below is final by then); the first one stops: no thread waits
__global__ void k_bottom_up(Tree2 T, int n, uint32_t* arrivals, int optimize) {
  const int p = int(blockIdx.x * blockDim.x + threadIdx.x);
  if (p >= n) return;
  int node = __ldcg(&T.leafParent[p]);
  while (node >= 0) {
    __threadfence();
    if (atomicAdd(&arrivals[node], 1u) == 0) return;
    __threadfence();
    refit(T, node);
    if (optimize && __ldcg(&T.count[node]) > kLeafMax) optimize_treelet(T, node);
    __threadfence();
    node = __ldcg(&T.parent[node]);
  }
}

// SAH-optimal collapse. For binary node x and i = 1..8 slots, C(x, i) is the least SAH cost of x's subtree as at
// most i children of a wide node:
//   C(x, 1) = min(leaf: A(x) n kPrimCost, only for n <= 3 triangles; wide node: A(x) kNodeCost + D(x, 8)),
//   C(x, i) = min(C(x, i - 1), D(x, i)),  D(x, i) = min over 0 < k < i of C(left, k) + C(right, i - k),
// and a triangle costs A kPrimCost in any number of slots. eff[x][i] is the slot count whose choice C(x, i) takes,
// split[x][j] the left child's share of j slots (at j = 1: of the 8 slots of x's own wide node), leaf[x] the choice
// at one slot. The costs weigh a wide node's visit (eight box tests) against a triangle test as 1 : 0.3.
struct Dp {
  float* cost;      // [ni x 8], C(x, i) at i - 1
  uint8_t* eff;     // [ni x 8]
  uint8_t* split;   // [ni x 8]
  uint8_t* leaf;    // [ni]
};
constexpr float kNodeCost = 1.0f, kPrimCost = 0.3f;
__device__ __forceinline__ float dp_cost(const Tree2& T, const Dp& D, int c, int i) {
  if (c < 0) return kPrimCost * box_area(T.plo[T.order[~c]], T.phi[T.order[~c]]);
  return __ldcg(&D.cost[size_t(c) * 8 + i - 1]);
}
__device__ void dp_node(const Tree2& T, const Dp& D, int x) {
  const int L = __ldcg(&T.left[x]), R = __ldcg(&T.right[x]);
  float cl[9], cr[9], cd[9];
  uint8_t kb[9];
  for (int i = 1; i <= 8; ++i) { cl[i] = dp_cost(T, D, L, i); cr[i] = dp_cost(T, D, R, i); }
  for (int i = 2; i <= 8; ++i) {
    float best = INFINITY;
    int bk = 1;
    for (int k = 1; k < i; ++k) { const float c = cl[k] + cr[i - k]; if (c < best) { best = c; bk = k; } }
    cd[i] = best;
    kb[i] = uint8_t(bk);
  }
  const float A = box_area(__ldcg(&T.nlo[x]), __ldcg(&T.nhi[x]));
  const uint32_t n = __ldcg(&T.count[x]);
  const float cInner = kNodeCost * A + cd[8], cLeaf = n <= kLeafMax ? kPrimCost * A * float(n) : INFINITY;
  const size_t o = size_t(x) * 8;
  float c = fminf(cLeaf, cInner);
  uint8_t eff = 1;
  __stcg(&D.leaf[x], uint8_t(cLeaf <= cInner ? 1 : 0));
  __stcg(&D.cost[o], c);
  __stcg(&D.eff[o], uint8_t(1));
  __stcg(&D.split[o], kb[8]);
  for (int i = 2; i <= 8; ++i) {
    if (cd[i] < c) { c = cd[i]; eff = uint8_t(i); }
    __stcg(&D.cost[o + i - 1], c);
    __stcg(&D.eff[o + i - 1], eff);
    __stcg(&D.split[o + i - 1], kb[i]);
  }
}
// bottom-up as k_bottom_up: the second arrival at a node fills its row from its children's
__global__ void k_collapse_dp(Tree2 T, Dp D, int n, uint32_t* arrivals) {
  const int p = int(blockIdx.x * blockDim.x + threadIdx.x);
  if (p >= n) return;
  int node = __ldcg(&T.leafParent[p]);
  while (node >= 0) {
    __threadfence();
    if (atomicAdd(&arrivals[node], 1u) == 0) return;
    __threadfence();
    dp_node(T, D, node);
    __threadfence();
    node = __ldcg(&T.parent[node]);
  }
}

struct Tree {
  const uint32_t* order;   // sorted position -> triangle
  const float4 *plo, *phi, *nlo, *nhi;
  const int *left, *right;
  const uint32_t* count;
};
__device__ __forceinline__ uint32_t count_of(const Tree& T, int c) { return c >= 0 ? T.count[c] : 1u; }
// a child slot holds a leaf: a triangle, or a subtree the collapse's program made one
__device__ __forceinline__ bool dp_leaf(const Dp& D, int c) { return c < 0 || D.leaf[c] != 0; }
// the triangles under a subtree of at most kLeafMax triangles, left to right
__device__ __forceinline__ uint32_t gather(const Tree& T, int c, uint32_t* out) {
  int st[2 * kLeafMax];
  int sp = 0;
  uint32_t n = 0;
  st[sp++] = c;
  while (sp && n < kLeafMax) {
    const int x = st[--sp];
    if (x < 0) { out[n++] = T.order[~x]; continue; }
    if (sp + 2 > int(2 * kLeafMax)) break;
    st[sp++] = T.right[x];
    st[sp++] = T.left[x];
  }
  return n;
}
__device__ __forceinline__ void box_of(const Tree& T, int c, float4& lo, float4& hi) {
  if (c >= 0) { lo = T.nlo[c]; hi = T.nhi[c]; } else { lo = T.plo[T.order[~c]]; hi = T.phi[T.order[~c]]; }
}

// level pass 1: each wide node's children as the collapse's program chose them (left to right), inner-child and
// triangle counts
__global__ void k_collapse_count(Tree T, Dp D, const int* wideSrc, uint32_t b, uint32_t e, int* kids, uint32_t* nInner, uint32_t* nTri) {
  const uint32_t w = b + blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= e) return;
  const int src = wideSrc[w];
  int ch[8];
  int n = 0;
  if (dp_leaf(D, src)) ch[n++] = src;   // a leaf root: one leaf child
  else {   // the 8 slots split between src's children, each share expanded by its eff / split choices
    int stN[8], stI[8];
    int sp = 0;
    const int k8 = D.split[size_t(src) * 8];
    stN[sp] = T.right[src]; stI[sp++] = 8 - k8;
    stN[sp] = T.left[src]; stI[sp++] = k8;
    while (sp && n < 8) {   // the shares on the stack sum to at most 8 - n, each at least 1
      --sp;
      const int c = stN[sp], i = stI[sp];
      if (c < 0) { ch[n++] = c; continue; }
      const int j = D.eff[size_t(c) * 8 + i - 1];
      if (j <= 1) { ch[n++] = c; continue; }
      const int k = D.split[size_t(c) * 8 + j - 1];
      if (sp + 2 > 8) break;
      stN[sp] = T.right[c]; stI[sp++] = j - k;
      stN[sp] = T.left[c]; stI[sp++] = k;
    }
  }
  uint32_t ni = 0, nt = 0;
  for (int k = 0; k < 8; ++k) {
    kids[size_t(w - b) * 8 + k] = k < n ? ch[k] : INT32_MIN;
    if (k < n) { if (dp_leaf(D, ch[k])) nt += count_of(T, ch[k]); else ++ni; }
  }
  nInner[w - b] = ni;
  nTri[w - b] = nt;
}

// level pass 2: node records, triangle records, the next level's sources
__global__ void k_collapse_emit(Tree T, Dp D, const float* v, const uint32_t* tri, const uint32_t* slot, const uint8_t* translucent, uint32_t b,
                                uint32_t e, const int* kids, const uint32_t* innerOff, const uint32_t* triOff, uint32_t triBase0,
                                uint32_t* nodes, float* tris, int* wideSrc) {
  const uint32_t w = b + blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= e) return;
  int ch[8];
  int n = 0;
  for (int k = 0; k < 8; ++k) { ch[k] = kids[size_t(w - b) * 8 + k]; if (ch[k] != INT32_MIN) n = k + 1; }
  const uint32_t childBase = e + innerOff[w - b], triBase = triBase0 + triOff[w - b];
  uint32_t* rec = nodes + size_t(w) * kNodeWords;
  uint32_t imask = 0, meta[8] = {}, inner = 0, tOff = 0;
  for (int k = 0; k < 8; ++k) {   // lo.x hi.x lo.y hi.y lo.z hi.z of each child at word 4 + 8 plane + k; empty slots +inf / -inf
    float4 lo = make_float4(INFINITY, INFINITY, INFINITY, 0.f), hi = make_float4(-INFINITY, -INFINITY, -INFINITY, 0.f);
    if (k < n) box_of(T, ch[k], lo, hi);
    rec[4 + 0 * 8 + k] = __float_as_uint(lo.x); rec[4 + 1 * 8 + k] = __float_as_uint(hi.x);
    rec[4 + 2 * 8 + k] = __float_as_uint(lo.y); rec[4 + 3 * 8 + k] = __float_as_uint(hi.y);
    rec[4 + 4 * 8 + k] = __float_as_uint(lo.z); rec[4 + 5 * 8 + k] = __float_as_uint(hi.z);
  }
  for (int k = 0; k < n; ++k) {
    if (!dp_leaf(D, ch[k])) {
      imask |= 1u << k;
      wideSrc[childBase + inner++] = ch[k];
    } else {
      uint32_t tt[kLeafMax];
      const uint32_t cnt = gather(T, ch[k], tt);
      meta[k] = (cnt << 5) | tOff;
      for (uint32_t j = 0; j < cnt; ++j) {
        const uint32_t t = tt[j];
        float* r = tris + size_t(triBase + tOff + j) * 12;
        for (int vtx = 0; vtx < 3; ++vtx)
          for (int a = 0; a < 3; ++a) r[4 * vtx + a] = v[3 * tri[3 * t + vtx] + a];
        r[3] = __uint_as_float(t);
        r[7] = __uint_as_float(translucent && translucent[t] ? 1u : 0u);
        r[11] = __uint_as_float(slot ? slot[t] : 0u);
      }
      tOff += cnt;
    }
  }
  rec[0] = childBase | (imask << 24);   // fewer than 2^24 nodes: the engine checks the triangle count first
  rec[1] = triBase;
  for (int b = 0; b < 3; ++b) meta[b] |= ((uint32_t(n - 1) >> b) & 1u) << 7;   // slots up to the last child (n >= 1), on slots in use
  rec[2] = meta[0] | (meta[1] << 8) | (meta[2] << 16) | (meta[3] << 24);
  rec[3] = meta[4] | (meta[5] << 8) | (meta[6] << 16) | (meta[7] << 24);
}

struct DevBuf {
  void* p = nullptr;
  ~DevBuf() { if (p) cudaFree(p); }
  template <class T> T* as() { return static_cast<T*>(p); }
};
#define KGB_TRY(x) do { const cudaError_t e_ = (x); if (e_ != cudaSuccess) return std::string(#x ": ") + cudaGetErrorString(e_); } while (0)

}  // namespace

// Builds on the device from host arrays; *nodesOut / *trisOut are new device buffers (cudaMalloc) the caller owns,
// also when the build fails after allocating them. Returns "" or what failed.
std::string build_bvh8_gpu(const float* v, size_t nv, const uint32_t* tri, size_t nt, const uint32_t* slot, const uint8_t* translucent,
                           cudaStream_t st, void** nodesOut, void** trisOut, uint32_t* nNodesOut, uint64_t* tempBytes) {
  *nodesOut = *trisOut = nullptr;
  *nNodesOut = 0;
  if (!nt) return "";
  if (nt >= (size_t(1) << 31) - 1) return "more than 2^31 triangles";
  const int n = int(nt);
  DevBuf dv, dtri, dslot, dtr, plo, phi, cen, cb, keys, keys2, vals, vals2, left, right, parent, leafParent, range, nlo, nhi, arr, cnt, cost, wideSrc,
      kids, nInner, nTri, offI, offT, tmp, maxabs, dpCost, dpEff, dpSplit, dpLeaf;
  const size_t tiles = (nt + 255) / 256;
  KGB_TRY(cudaMalloc(&dv.p, nv * 12));
  KGB_TRY(cudaMalloc(&dtri.p, nt * 12));
  KGB_TRY(cudaMemcpyAsync(dv.p, v, nv * 12, cudaMemcpyDefault, st));
  KGB_TRY(cudaMemcpyAsync(dtri.p, tri, nt * 12, cudaMemcpyDefault, st));
  if (slot) { KGB_TRY(cudaMalloc(&dslot.p, nt * 4)); KGB_TRY(cudaMemcpyAsync(dslot.p, slot, nt * 4, cudaMemcpyDefault, st)); }
  if (translucent) { KGB_TRY(cudaMalloc(&dtr.p, nt)); KGB_TRY(cudaMemcpyAsync(dtr.p, translucent, nt, cudaMemcpyDefault, st)); }
  // 1. eps
  KGB_TRY(cudaMalloc(&maxabs.p, 4));
  KGB_TRY(cudaMemsetAsync(maxabs.p, 0, 4, st));
  k_maxabs<<<1024, 256, 0, st>>>(dv.as<float>(), nv * 3, maxabs.as<uint32_t>());
  uint32_t mbits = 0;
  KGB_TRY(cudaMemcpyAsync(&mbits, maxabs.p, 4, cudaMemcpyDeviceToHost, st));
  KGB_TRY(cudaStreamSynchronize(st));
  float M;
  std::memcpy(&M, &mbits, 4);
  M = std::max(1.f, M);
  const float eps = M * (1.f / 65536.f);
  // 2. boxes, centroids, centroid bounds
  KGB_TRY(cudaMalloc(&plo.p, nt * 16)); KGB_TRY(cudaMalloc(&phi.p, nt * 16)); KGB_TRY(cudaMalloc(&cen.p, nt * 16));
  KGB_TRY(cudaMalloc(&cb.p, 24));
  const uint32_t cbInit[6] = {~0u, ~0u, ~0u, 0u, 0u, 0u};
  KGB_TRY(cudaMemcpyAsync(cb.p, cbInit, 24, cudaMemcpyHostToDevice, st));
  k_prims<<<unsigned(tiles), 256, 0, st>>>(dv.as<float>(), dtri.as<uint32_t>(), uint32_t(nt), eps, plo.as<float4>(), phi.as<float4>(), cen.as<float4>(),
                                           cb.as<uint32_t>());
  // 3. Morton codes, sorted
  KGB_TRY(cudaMalloc(&keys.p, nt * 8)); KGB_TRY(cudaMalloc(&keys2.p, nt * 8));
  KGB_TRY(cudaMalloc(&vals.p, nt * 4)); KGB_TRY(cudaMalloc(&vals2.p, nt * 4));
  k_morton<<<unsigned(tiles), 256, 0, st>>>(cen.as<float4>(), uint32_t(nt), cb.as<uint32_t>(), keys.as<uint64_t>(), vals.as<uint32_t>());
  size_t sortBytes = 0, scanBytes = 0;
  KGB_TRY(cub::DeviceRadixSort::SortPairs(nullptr, sortBytes, keys.as<uint64_t>(), keys2.as<uint64_t>(), vals.as<uint32_t>(), vals2.as<uint32_t>(),
                                          n, 0, 63, st));
  KGB_TRY(cub::DeviceScan::ExclusiveSum(nullptr, scanBytes, static_cast<uint32_t*>(nullptr), static_cast<uint32_t*>(nullptr), n, st));
  const size_t tmpBytes = std::max(sortBytes, scanBytes);
  KGB_TRY(cudaMalloc(&tmp.p, tmpBytes));
  size_t sortUse = tmpBytes;
  KGB_TRY(cub::DeviceRadixSort::SortPairs(tmp.p, sortUse, keys.as<uint64_t>(), keys2.as<uint64_t>(), vals.as<uint32_t>(), vals2.as<uint32_t>(), n,
                                          0, 63, st));
  // 4. radix tree
  const size_t ni = std::max<size_t>(1, nt - 1);
  KGB_TRY(cudaMalloc(&left.p, ni * 4)); KGB_TRY(cudaMalloc(&right.p, ni * 4)); KGB_TRY(cudaMalloc(&parent.p, ni * 4));
  KGB_TRY(cudaMalloc(&leafParent.p, nt * 4)); KGB_TRY(cudaMalloc(&range.p, ni * 8));
  KGB_TRY(cudaMalloc(&nlo.p, ni * 16)); KGB_TRY(cudaMalloc(&nhi.p, ni * 16)); KGB_TRY(cudaMalloc(&arr.p, ni * 4));
  KGB_TRY(cudaMalloc(&cnt.p, ni * 4)); KGB_TRY(cudaMalloc(&cost.p, ni * 4));
  Tree2 T2{left.as<int>(), right.as<int>(), parent.as<int>(), leafParent.as<int>(), nlo.as<float4>(), nhi.as<float4>(), cnt.as<uint32_t>(),
           cost.as<float>(), vals2.as<uint32_t>(), plo.as<float4>(), phi.as<float4>()};
  if (n == 1) KGB_TRY(cudaMemsetAsync(leafParent.p, 0xff, 4, st));   // the single leaf is the root
  else {
    k_karras<<<unsigned((ni + 255) / 256), 256, 0, st>>>(keys2.as<uint64_t>(), n, left.as<int>(), right.as<int>(), parent.as<int>(), leafParent.as<int>(),
                                                         range.as<int2>());
    // 5. boxes, counts, costs; then passes of treelet restructuring
    for (int pass = 0; pass <= kTreeletPasses; ++pass) {
      KGB_TRY(cudaMemsetAsync(arr.p, 0, ni * 4, st));
      k_bottom_up<<<unsigned(tiles), 256, 0, st>>>(T2, n, arr.as<uint32_t>(), pass > 0 ? 1 : 0);
    }
  }
  // 6a. the collapse's program, bottom-up over the final tree
  KGB_TRY(cudaMalloc(&dpCost.p, ni * 32)); KGB_TRY(cudaMalloc(&dpEff.p, ni * 8)); KGB_TRY(cudaMalloc(&dpSplit.p, ni * 8));
  KGB_TRY(cudaMalloc(&dpLeaf.p, ni));
  const Dp D{dpCost.as<float>(), dpEff.as<uint8_t>(), dpSplit.as<uint8_t>(), dpLeaf.as<uint8_t>()};
  if (n > 1) {
    KGB_TRY(cudaMemsetAsync(arr.p, 0, ni * 4, st));
    k_collapse_dp<<<unsigned(tiles), 256, 0, st>>>(T2, D, n, arr.as<uint32_t>());
  }
  // 6-7. collapse level by level into the output buffers
  void* nodes = nullptr;
  void* tris = nullptr;
  const size_t maxNodes = std::max<size_t>(1, nt);   // a wide node has at least two children but the root
  KGB_TRY(cudaMalloc(&nodes, maxNodes * kNodeBytes));
  if (cudaMalloc(&tris, nt * 48) != cudaSuccess) { cudaFree(nodes); return "cudaMalloc(tris) failed"; }
  *nodesOut = nodes;
  *trisOut = tris;
  KGB_TRY(cudaMalloc(&wideSrc.p, maxNodes * 4));
  KGB_TRY(cudaMalloc(&kids.p, maxNodes * 32));
  KGB_TRY(cudaMalloc(&nInner.p, maxNodes * 4)); KGB_TRY(cudaMalloc(&nTri.p, maxNodes * 4));
  KGB_TRY(cudaMalloc(&offI.p, maxNodes * 4)); KGB_TRY(cudaMalloc(&offT.p, maxNodes * 4));
  const int root = n == 1 ? ~0 : 0;
  KGB_TRY(cudaMemcpyAsync(wideSrc.p, &root, 4, cudaMemcpyHostToDevice, st));
  Tree T{vals2.as<uint32_t>(), plo.as<float4>(), phi.as<float4>(), nlo.as<float4>(), nhi.as<float4>(), left.as<int>(), right.as<int>(),
         cnt.as<uint32_t>()};
  uint32_t b = 0, e = 1, triBase = 0;
  for (int level = 0; b < e; ++level) {
    if (level > 4096) return "bvh collapse: too many levels";
    const uint32_t cnt = e - b, blocks = (cnt + 127) / 128;
    k_collapse_count<<<blocks, 128, 0, st>>>(T, D, wideSrc.as<int>(), b, e, kids.as<int>(), nInner.as<uint32_t>(), nTri.as<uint32_t>());
    size_t sb = tmpBytes;
    KGB_TRY(cub::DeviceScan::ExclusiveSum(tmp.p, sb, nInner.as<uint32_t>(), offI.as<uint32_t>(), int(cnt), st));
    KGB_TRY(cub::DeviceScan::ExclusiveSum(tmp.p, sb, nTri.as<uint32_t>(), offT.as<uint32_t>(), int(cnt), st));
    uint32_t lastI[2], lastT[2];
    KGB_TRY(cudaMemcpyAsync(&lastI[0], offI.as<uint32_t>() + cnt - 1, 4, cudaMemcpyDeviceToHost, st));
    KGB_TRY(cudaMemcpyAsync(&lastI[1], nInner.as<uint32_t>() + cnt - 1, 4, cudaMemcpyDeviceToHost, st));
    KGB_TRY(cudaMemcpyAsync(&lastT[0], offT.as<uint32_t>() + cnt - 1, 4, cudaMemcpyDeviceToHost, st));
    KGB_TRY(cudaMemcpyAsync(&lastT[1], nTri.as<uint32_t>() + cnt - 1, 4, cudaMemcpyDeviceToHost, st));
    k_collapse_emit<<<blocks, 128, 0, st>>>(T, D, dv.as<float>(), dtri.as<uint32_t>(), dslot.as<uint32_t>(), dtr.as<uint8_t>(), b, e, kids.as<int>(),
                                            offI.as<uint32_t>(), offT.as<uint32_t>(), triBase, static_cast<uint32_t*>(nodes), static_cast<float*>(tris),
                                            wideSrc.as<int>());
    KGB_TRY(cudaGetLastError());
    KGB_TRY(cudaStreamSynchronize(st));
    const uint64_t next = uint64_t(e) + lastI[0] + lastI[1];
    if (next > maxNodes) return "bvh collapse: node count beyond its bound";
    triBase += lastT[0] + lastT[1];
    b = e;
    e = uint32_t(next);
  }
  if (triBase != nt) return "bvh collapse: " + std::to_string(triBase) + " triangle records for " + std::to_string(nt) + " triangles";
  *nNodesOut = e;
  *tempBytes = nt * (12 + 16 * 3 + 8 * 2 + 4 * 2 + 4 * 4 + 8 + 32 + 4 + 8 + 49) + maxNodes * (4 + 32 + 16) + tmpBytes;
  return "";
}

}  // namespace kgb
