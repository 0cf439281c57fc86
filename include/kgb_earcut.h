/*
 * kgb_earcut.h - ear-clipping triangulation of one polygon ring, for the GPU (one thread per polygon) and the host.
 *
 * The reference triangulates faces of five or more corners with mapbox earcut (v2.2.4, ISC licence, fetched by its
 * CMake and not vendored: src/mesh.cpp:154-165 projects the face onto its Newell plane and calls earcut on the one
 * ring). This file restates earcut's published algorithm, step for step, so that the engine's device triangulation
 * (kgb_triangulate) gives the triangles the reference gives:
 *  - the ring as a circular doubly linked list in clockwise order (reversed when its shoelace sum says otherwise), a
 *    last node equal to its successor dropped;
 *  - ear slicing: a node is an ear when the triangle (prev, node, next) is convex (signed area < 0) and no reflex
 *    node of the rest of the ring lies in it (point-in-triangle test, edges included); an ear emits (prev, node, next),
 *    is removed, and the search goes on from next's successor;
 *  - when a full turn finds no ear: pass 1 filters duplicate and collinear nodes and slices again; pass 2 also cures
 *    local self-intersections (an edge crossing the one after next: the triangle between them is emitted); pass 3
 *    splits the ring along the first valid diagonal and triangulates both halves, the first half first.
 * Earcut's z-order hash for rings of more than 80 points only changes the order in which the ear test looks at the
 * other nodes, never its answer, so it is left out: the triangles are the same (the search is quadratic instead).
 * All arithmetic is IEEE double with no contraction (compile with -fmad=false / -ffp-contract=off), as the
 * reference's build computes it.
 *
 * Storage is the caller's: pool >= 2 n + 16 nodes (a ring of n points, two more per split), stack >= 2 n + 16 work
 * items. earcut_ring returns the number of triangles written to tri (3 ring indices each, at most triCap), or -1 when
 * the pool or the stack ran out (the face is then skipped).
 */
#ifndef KGB_EARCUT_H
#define KGB_EARCUT_H

#include <stdint.h>

#if defined(__CUDACC__)
#define KGB_EC_FN __host__ __device__ inline
#else
#define KGB_EC_FN inline
#endif

namespace kgb_earcut {

struct Node {
  uint32_t i;        // the point's index in the ring
  double x, y;
  int32_t prev, next;
  int32_t steiner;   // always 0 here (earcut's Steiner points come from holes)
};

struct Ring {
  Node* nodes;
  int32_t n, cap;
  uint32_t* tri;
  int32_t nTri, triCap;
  bool full;
};

KGB_EC_FN double area(const Node& p, const Node& q, const Node& r) { return (q.y - p.y) * (r.x - q.x) - (q.x - p.x) * (r.y - q.y); }
KGB_EC_FN bool equals(const Node& a, const Node& b) { return a.x == b.x && a.y == b.y; }
KGB_EC_FN int sign(double v) { return (0.0 < v) - (v < 0.0); }
KGB_EC_FN bool point_in_triangle(double ax, double ay, double bx, double by, double cx, double cy, double px, double py) {
  return (cx - px) * (ay - py) >= (ax - px) * (cy - py) && (ax - px) * (by - py) >= (bx - px) * (ay - py) &&
         (bx - px) * (cy - py) >= (cx - px) * (by - py);
}
KGB_EC_FN bool on_segment(const Node& p, const Node& q, const Node& r) {
  const double mx = p.x > r.x ? p.x : r.x, nx = p.x < r.x ? p.x : r.x, my = p.y > r.y ? p.y : r.y, ny = p.y < r.y ? p.y : r.y;
  return q.x <= mx && q.x >= nx && q.y <= my && q.y >= ny;
}
KGB_EC_FN bool intersects(const Node& p1, const Node& q1, const Node& p2, const Node& q2) {
  const int o1 = sign(area(p1, q1, p2)), o2 = sign(area(p1, q1, q2)), o3 = sign(area(p2, q2, p1)), o4 = sign(area(p2, q2, q1));
  if (o1 != o2 && o3 != o4) return true;
  if (o1 == 0 && on_segment(p1, p2, q1)) return true;
  if (o2 == 0 && on_segment(p1, q2, q1)) return true;
  if (o3 == 0 && on_segment(p2, p1, q2)) return true;
  if (o4 == 0 && on_segment(p2, q1, q2)) return true;
  return false;
}

KGB_EC_FN int32_t insert_node(Ring& R, uint32_t i, double x, double y, int32_t last) {
  if (R.n >= R.cap) { R.full = true; return last; }
  const int32_t p = R.n++;
  Node& q = R.nodes[p];
  q.i = i; q.x = x; q.y = y; q.steiner = 0;
  if (last < 0) { q.prev = p; q.next = p; }
  else {
    q.next = R.nodes[last].next;
    q.prev = last;
    R.nodes[R.nodes[last].next].prev = p;
    R.nodes[last].next = p;
  }
  return p;
}
KGB_EC_FN void remove_node(Ring& R, int32_t p) {
  Node& q = R.nodes[p];
  R.nodes[q.next].prev = q.prev;
  R.nodes[q.prev].next = q.next;
}
KGB_EC_FN void emit(Ring& R, uint32_t a, uint32_t b, uint32_t c) {
  if (R.nTri >= R.triCap) return;
  R.tri[3 * R.nTri] = a; R.tri[3 * R.nTri + 1] = b; R.tri[3 * R.nTri + 2] = c;
  ++R.nTri;
}

// duplicate or collinear nodes removed, from start round to end (or start); returns the node the walk ended on
KGB_EC_FN int32_t filter_points(Ring& R, int32_t start, int32_t end) {
  if (end < 0) end = start;
  int32_t p = start;
  bool again;
  do {
    again = false;
    const Node& q = R.nodes[p];
    if (!q.steiner && (equals(q, R.nodes[q.next]) || area(R.nodes[q.prev], q, R.nodes[q.next]) == 0)) {
      remove_node(R, p);
      p = end = R.nodes[p].prev;
      if (p == R.nodes[p].next) break;
      again = true;
    } else {
      p = q.next;
    }
  } while (again || p != end);
  return end;
}

KGB_EC_FN bool is_ear(const Ring& R, int32_t ear) {
  const Node& a = R.nodes[R.nodes[ear].prev];
  const Node& b = R.nodes[ear];
  const Node& c = R.nodes[b.next];
  if (area(a, b, c) >= 0) return false;   // reflex
  for (int32_t p = c.next; p != b.prev; p = R.nodes[p].next) {
    const Node& q = R.nodes[p];
    if (point_in_triangle(a.x, a.y, b.x, b.y, c.x, c.y, q.x, q.y) && area(R.nodes[q.prev], q, R.nodes[q.next]) >= 0) return false;
  }
  return true;
}

KGB_EC_FN bool locally_inside(const Ring& R, int32_t ai, int32_t bi) {
  const Node& a = R.nodes[ai];
  const Node& b = R.nodes[bi];
  const Node& ap = R.nodes[a.prev];
  const Node& an = R.nodes[a.next];
  return area(ap, a, an) < 0 ? area(a, b, an) >= 0 && area(a, ap, b) >= 0 : area(a, b, ap) < 0 || area(a, an, b) < 0;
}
KGB_EC_FN bool middle_inside(const Ring& R, int32_t ai, int32_t bi) {
  const Node& a = R.nodes[ai];
  const Node& b = R.nodes[bi];
  bool inside = false;
  const double px = (a.x + b.x) / 2, py = (a.y + b.y) / 2;
  int32_t p = ai;
  do {
    const Node& q = R.nodes[p];
    const Node& n = R.nodes[q.next];
    if (((q.y > py) != (n.y > py)) && n.y != q.y && (px < (n.x - q.x) * (py - q.y) / (n.y - q.y) + q.x)) inside = !inside;
    p = q.next;
  } while (p != ai);
  return inside;
}
KGB_EC_FN bool intersects_polygon(const Ring& R, int32_t ai, int32_t bi) {
  const Node& a = R.nodes[ai];
  const Node& b = R.nodes[bi];
  int32_t p = ai;
  do {
    const Node& q = R.nodes[p];
    const Node& n = R.nodes[q.next];
    if (q.i != a.i && n.i != a.i && q.i != b.i && n.i != b.i && intersects(q, n, a, b)) return true;
    p = q.next;
  } while (p != ai);
  return false;
}
KGB_EC_FN bool is_valid_diagonal(const Ring& R, int32_t ai, int32_t bi) {
  const Node& a = R.nodes[ai];
  const Node& b = R.nodes[bi];
  return R.nodes[a.next].i != b.i && R.nodes[a.prev].i != b.i && !intersects_polygon(R, ai, bi) &&
         ((locally_inside(R, ai, bi) && locally_inside(R, bi, ai) && middle_inside(R, ai, bi) &&
           (area(R.nodes[a.prev], a, R.nodes[b.prev]) != 0.0 || area(a, R.nodes[b.prev], b) != 0.0)) ||
          (equals(a, b) && area(R.nodes[a.prev], a, R.nodes[a.next]) > 0 && area(R.nodes[b.prev], b, R.nodes[b.next]) > 0));
}
// the ring split along the diagonal a-b into two rings (a's copy and b's copy close the second); returns b's copy
KGB_EC_FN int32_t split_polygon(Ring& R, int32_t a, int32_t b) {
  if (R.n + 2 > R.cap) { R.full = true; return -1; }
  const int32_t a2 = R.n++, b2 = R.n++;
  R.nodes[a2] = Node{R.nodes[a].i, R.nodes[a].x, R.nodes[a].y, -1, -1, 0};
  R.nodes[b2] = Node{R.nodes[b].i, R.nodes[b].x, R.nodes[b].y, -1, -1, 0};
  const int32_t an = R.nodes[a].next, bp = R.nodes[b].prev;
  R.nodes[a].next = b; R.nodes[b].prev = a;
  R.nodes[a2].next = an; R.nodes[an].prev = a2;
  R.nodes[b2].next = a2; R.nodes[a2].prev = b2;
  R.nodes[bp].next = b2; R.nodes[b2].prev = bp;
  return b2;
}
KGB_EC_FN int32_t cure_local_intersections(Ring& R, int32_t start) {
  int32_t p = start;
  do {
    const int32_t a = R.nodes[p].prev, b = R.nodes[R.nodes[p].next].next;
    if (!equals(R.nodes[a], R.nodes[b]) && intersects(R.nodes[a], R.nodes[p], R.nodes[R.nodes[p].next], R.nodes[b]) && locally_inside(R, a, b) &&
        locally_inside(R, b, a)) {
      emit(R, R.nodes[a].i, R.nodes[p].i, R.nodes[b].i);
      remove_node(R, p);
      remove_node(R, R.nodes[p].next);
      p = start = b;
    }
    p = R.nodes[p].next;
  } while (p != start);
  return filter_points(R, p, -1);
}

// The ring's triangles (earcut's operator() for one ring, without the z-order hash). xy: 2 n doubles.
KGB_EC_FN int earcut_ring(const double* xy, int32_t n, Node* pool, int32_t poolCap, int32_t* stack, int32_t stackCap, uint32_t* tri, int32_t triCap) {
  Ring R{pool, 0, poolCap, tri, 0, triCap, false};
  if (n <= 0) return 0;
  // linkedList(ring, clockwise = true)
  double sum = 0;
  for (int32_t i = 0, j = n - 1; i < n; j = i++) sum += (xy[2 * j] - xy[2 * i]) * (xy[2 * i + 1] + xy[2 * j + 1]);
  int32_t last = -1;
  if (sum > 0) for (int32_t i = 0; i < n; ++i) last = insert_node(R, uint32_t(i), xy[2 * i], xy[2 * i + 1], last);
  else for (int32_t i = n; i-- > 0;) last = insert_node(R, uint32_t(i), xy[2 * i], xy[2 * i + 1], last);
  if (R.full) return -1;
  if (last >= 0 && equals(R.nodes[last], R.nodes[R.nodes[last].next])) {
    remove_node(R, last);
    last = R.nodes[last].next;
  }
  if (last < 0 || R.nodes[last].prev == R.nodes[last].next) return 0;
  // earcutLinked as a loop over work items (node, pass); a split pushes its second half, then its first, so the first
  // half's triangles come first, as the recursion's do
  int32_t sp = 0;
  stack[sp++] = last;   // pass 0
  stack[sp++] = 0;
  while (sp) {
    const int32_t pass = stack[--sp];
    int32_t ear = stack[--sp];
    if (ear < 0) continue;
    int32_t stop = ear;
    while (R.nodes[ear].prev != R.nodes[ear].next) {
      const int32_t prev = R.nodes[ear].prev, next = R.nodes[ear].next;
      if (is_ear(R, ear)) {
        emit(R, R.nodes[prev].i, R.nodes[ear].i, R.nodes[next].i);
        remove_node(R, ear);
        ear = R.nodes[next].next;
        stop = R.nodes[next].next;
        continue;
      }
      ear = next;
      if (ear == stop) {   // a full turn without an ear
        if (pass == 0) {
          if (sp + 2 > stackCap) return -1;
          stack[sp++] = filter_points(R, ear, -1); stack[sp++] = 1;
        } else if (pass == 1) {
          if (sp + 2 > stackCap) return -1;
          stack[sp++] = cure_local_intersections(R, filter_points(R, ear, -1)); stack[sp++] = 2;
        } else {   // splitEarcut: the first valid diagonal, then both halves
          int32_t a = ear;
          bool split = false;
          do {
            for (int32_t b = R.nodes[R.nodes[a].next].next; b != R.nodes[a].prev; b = R.nodes[b].next) {
              if (R.nodes[a].i != R.nodes[b].i && is_valid_diagonal(R, a, b)) {
                int32_t c = split_polygon(R, a, b);
                if (c < 0) return -1;
                a = filter_points(R, a, R.nodes[a].next);
                c = filter_points(R, c, R.nodes[c].next);
                if (sp + 4 > stackCap) return -1;
                stack[sp++] = c; stack[sp++] = 0;
                stack[sp++] = a; stack[sp++] = 0;
                split = true;
                break;
              }
            }
            if (split) break;
            a = R.nodes[a].next;
          } while (a != ear);
        }
        break;
      }
    }
  }
  return R.full ? -1 : R.nTri;
}

}  // namespace kgb_earcut

#endif /* KGB_EARCUT_H */
