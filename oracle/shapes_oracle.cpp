/*
 * TEST INFRASTRUCTURE ONLY — the CPU oracle for the shapes world step.
 *
 * This file restates, in plain sequential C++, the world step of ublubu/shapes
 * (`Physics.Engine.Main.updateWorld`, shapes/src/Physics/Engine/Main.hs:71-84)
 * and everything it calls, in the reference's exact floating-point operation
 * order.  It is the checker for the CUDA implementation and the timed CPU
 * baseline; nothing in the product links or calls it.
 *
 * Arithmetic contract: IEEE-754 binary64, every sum a left fold in source
 * order (shapes-math/src/Shapes/Linear/Template.hs:108-110 `dotE`), no fused
 * multiply-add (build with -ffp-contract=off), no fast-math.  Comparisons are
 * spelled exactly as the reference's (GHC's default `max x y = if x <= y then
 * y else x`, `min x y = if x <= y then x else y`), so NaN and signed-zero
 * behaviour follows the reference too.
 *
 * Deviations, all deliberate and shared with the CUDA path:
 *   - sin/cos come from shapes_sincos() (correctly rounded, see
 *     shapes_sincos.h) instead of libm; a world can be switched to the host
 *     libm's sin and cos (oracle_world_set_trig), which is what the reference
 *     calls, to measure how far the two choices drift apart;
 *   - the solver sweep count is a parameter (the reference hard-codes 2 sweeps,
 *     Engine/Main.hs:81-82; iterations=2 reproduces it);
 *   - warm starting can be switched off (the reference always warm-starts).
 *
 * Parity status: the reference is Haskell and cannot be built or run here, so
 * the oracle is pinned by known answers derived from the reference's own
 * fixtures (shapes/bench/Physics/Contact/Benchmark.hs:16-27 boxes,
 * shapes/bench/Physics/Constraint/Benchmark.hs:11-35 constraint pair,
 * shapes/test/Physics/Broadphase/AabbSpec.hs:8-16 pair count), not by running
 * the reference itself.
 */
#include <cmath>
#include <cstdint>
#include <cstring>
#include <algorithm>
#include <chrono>
#include <thread>
#include <vector>

#include "../shapes_gb300/csrc/shapes_sincos.h"

namespace {

/* PhysicalObj (Constraint.hs:52-57) + Material (World.hs:35-38), unboxed. */
struct Body {
  double vx, vy, w, px, py, th, iml, imr, mu, bounce;
};

/* ConvexHull (ConvexHull.hs:61-68): local vertices, precomputed local extents,
 * and the world-space vertices and unit edge normals of the current pose. */
struct Hull {
  int nv = 0;
  double radius = 0.0; /* > 0: a Circle (Contact/Circle.hs:19-22), nv = 1, local centre (0, 0) */
  std::vector<double> lx, ly;
  std::vector<int> emin, emax;
  std::vector<double> wx, wy, nx, ny;
};

/* ObjectFeatureKey (Constraints/Contact.hs:36-39), derived Ord = lexicographic. */
struct Key {
  int32_t i, j, fa, fb;
};
static inline bool key_lt(const Key& a, const Key& b) {
  if (a.i != b.i) return a.i < b.i;
  if (a.j != b.j) return a.j < b.j;
  if (a.fa != b.fa) return a.fa < b.fa;
  return a.fb < b.fb;
}
static inline bool key_eq(const Key& a, const Key& b) {
  return a.i == b.i && a.j == b.j && a.fa == b.fa && a.fb == b.fb;
}

/* Flipping Contact (Contact/Types.hs:30-36 + Utils.hs:147). */
struct Contact {
  Key key;
  int flip;
  double nx, ny, px, py, depth;
};

/* (ObjectFeatureKey, ContactLagrangian) cache entry (Engine/Main.hs:32). */
struct CacheEntry {
  Key key;
  double ln, lf;
};

/* ContactConstraint (Constraints/Types.hs:45-49): non-penetration J,b;
 * restitution radii + normal; friction J (b = 0). */
struct ContactConstraint {
  double jn[6], bn;
  double rax, ray, rbx, rby, rnx, rny;
  double jf[6];
};

struct World {
  double residual = 0.0; /* RMS of one non-applying sweep after the last step */
  bool trig_libm = false; /* rotations from the host libm's sin and cos instead of shapes_sincos */
  int64_t trig_mismatches = 0; /* libm mode: poses whose libm sin or cos differs from shapes_sincos */
  std::vector<Body> bodies;
  /* EmptiesVector (Utils/EmptiesVector.hs): filled slots, and the empty
   * slots as a stack (delete pushes, append pops: the last slot freed is the
   * next one filled) */
  std::vector<uint8_t> active;
  std::vector<int32_t> empties;
  std::vector<Hull> hulls;
  std::vector<CacheEntry> cache;
  std::vector<int32_t> pairs; /* flattened (i, j) */
  std::vector<Contact> contacts;
};

struct StepConfig {
  double dt, beta, slop, ax, ay;
  int iterations, warm_start, external;
};

/* ---- L1 math ------------------------------------------------------------ */

/* unitEdgeNormal (ConvexHull.hs:218-226) = normalizeV2 (Linear.hs:165-168)
 * of clockwiseV2 (Linear.hs:161-163) of (v' - v). */
static inline void unit_edge_normal(double x0, double y0, double x1, double y1,
                                    double* nx, double* ny) {
  double dx = x1 - x0, dy = y1 - y0;
  double ex = dy, ey = -dx;
  double n = std::sqrt(ex * ex + ey * ey);
  *nx = ex / n;
  *ny = ey / n;
}

/* extentAlong' (ConvexHull.hs:81-92): first strict minimum / maximum of the
 * projections vertex·dir, in vertex order. */
static inline void extent_along(const double* xs, const double* ys, int nv, double dx, double dy,
                                int* imin, int* imax, double* dmin, double* dmax) {
  double lo = xs[0] * dx + ys[0] * dy, hi = lo;
  int a = 0, b = 0;
  for (int k = 1; k < nv; ++k) {
    double d = xs[k] * dx + ys[k] * dy;
    if (d < lo) { lo = d; a = k; }
    if (d > hi) { hi = d; b = k; }
  }
  *imin = a; *imax = b; *dmin = lo; *dmax = hi;
}

/* listToHull (ConvexHull.hs:151-167): local normals from local vertices, then
 * the (min, max) extent indices of the hull along each of its own normals. */
static void init_hull(Hull& h, int nv, const double* xy) {
  if (nv == 1) { /* a circle: one local point (radius, 0) */
    h.nv = 1;
    h.radius = xy[0];
    h.lx.assign(1, 0.0); h.ly.assign(1, 0.0);
    h.emin.assign(1, 0); h.emax.assign(1, 0);
    h.wx.assign(1, 0.0); h.wy.assign(1, 0.0); h.nx.assign(1, 0.0); h.ny.assign(1, 0.0);
    return;
  }
  h.radius = 0.0;
  h.nv = nv;
  h.lx.resize(nv); h.ly.resize(nv);
  for (int k = 0; k < nv; ++k) { h.lx[k] = xy[2 * k]; h.ly[k] = xy[2 * k + 1]; }
  h.emin.resize(nv); h.emax.resize(nv);
  h.wx.resize(nv); h.wy.resize(nv); h.nx.resize(nv); h.ny.resize(nv);
  for (int e = 0; e < nv; ++e) {
    int n1 = e < nv - 1 ? e + 1 : 0;
    double nx, ny, lo, hi;
    unit_edge_normal(h.lx[e], h.ly[e], h.lx[n1], h.ly[n1], &nx, &ny);
    extent_along(h.lx.data(), h.ly.data(), nv, nx, ny, &h.emin[e], &h.emax[e], &lo, &hi);
  }
}

/* moveShape (World.hs:132-133) → setHullTransform (ConvexHull.hs:184-195) with
 * _physObjTransform (Constraint.hs:144-147) = toTransform (Transform.hs:34-38):
 * joinTransforms (Transform.hs:73-77) of translate (outer) and rotate (inner),
 * multiplied as 3x3 matrices (MatrixTemplate.hs:47-67), applied by afmul
 * (Linear.hs:217-220) to each local vertex; normals re-derived per edge. */
static void pose_hull(const Body& b, Hull& h, bool trig_libm, int64_t* mismatches) {
  double s, c;
  if (trig_libm) { /* rotate22 (Linear.hs:353-357): cosDouble# and sinDouble# are libm's cos and sin */
    c = std::cos(b.th);
    s = std::sin(b.th);
    double s2, c2;
    shapes_sincos(b.th, &s2, &c2);
    if (std::memcmp(&s, &s2, 8) != 0 || std::memcmp(&c, &c2, 8) != 0) ++*mismatches;
  } else {
    shapes_sincos(b.th, &s, &c);
  }
  const double T[3][3] = {{1.0, 0.0, b.px}, {0.0, 1.0, b.py}, {0.0, 0.0, 1.0}};
  const double R[3][3] = {{c, -s, 0.0}, {s, c, 0.0}, {0.0, 0.0, 1.0}};
  double M[3][3];
  for (int r = 0; r < 3; ++r)
    for (int q = 0; q < 3; ++q)
      M[r][q] = (T[r][0] * R[0][q] + T[r][1] * R[1][q]) + T[r][2] * R[2][q];
  for (int k = 0; k < h.nv; ++k) {
    double x = h.lx[k], y = h.ly[k];
    h.wx[k] = (M[0][0] * x + M[0][1] * y) + M[0][2] * 1.0;
    h.wy[k] = (M[1][0] * x + M[1][1] * y) + M[1][2] * 1.0;
  }
  if (h.radius > 0.0) return; /* setCircleTransform (Circle.hs:60-64): the centre only */
  for (int e = 0; e < h.nv; ++e) {
    int n1 = e < h.nv - 1 ? e + 1 : 0;
    unit_edge_normal(h.wx[e], h.wy[e], h.wx[n1], h.wy[n1], &h.nx[e], &h.ny[e]);
  }
}

/* ---- A3 broadphase ------------------------------------------------------- */

struct Aabb {
  double x0, x1, y0, y1;
};

/* hullToAabb (Aabb.hs:81-84): foldl1 mergeAabb over the vertex points, with
 * mergeRange (Aabb.hs:106-110) = (if a < c then a else c, if b > d then b else d). */
static Aabb hull_aabb(const Hull& h) {
  if (h.radius > 0.0) { /* circleToAabb (Aabb.hs:86-89) */
    const double x = h.wx[0], y = h.wy[0], r = h.radius;
    return Aabb{x - r, x + r, y - r, y + r};
  }
  Aabb a{h.wx[0], h.wx[0], h.wy[0], h.wy[0]};
  for (int k = 1; k < h.nv; ++k) {
    double x = h.wx[k], y = h.wy[k];
    a.x0 = a.x0 < x ? a.x0 : x;
    a.x1 = a.x1 > x ? a.x1 : x;
    a.y0 = a.y0 < y ? a.y0 : y;
    a.y1 = a.y1 > y ? a.y1 : y;
  }
  return a;
}

/* boundsOverlap (Aabb.hs:69-72): not (c > b || d < a). */
static inline bool bounds_overlap(double a, double b, double c, double d) {
  return !(c > b || d < a);
}

/* isStatic (Constraint.hs:123-125): InvMass2 == (0, 0). */
static inline bool is_static(const Body& b) { return b.iml == 0.0 && b.imr == 0.0; }

/* culledKeys (Aabb.hs:168-183) over unorderedPairs (Aabb.hs:155-163): every
 * (i, j), i > j, in descending order, not both static, AABBs overlapping.
 * The step calls Grid.culledKeys (Engine/Main.hs:75, Grid.hs:257-283), which
 * yields this same list: overlapping closed boxes share a point and therefore
 * a (possibly aliased) grid cell, aliasing only adds candidates that aabbCheck
 * removes, and sortBy-descending + uniq restores this order. */
static void broadphase(World& w) {
  const int n = (int)w.bodies.size();
  std::vector<Aabb> box(n);
  for (int i = 0; i < n; ++i) box[i] = hull_aabb(w.hulls[i]);
  w.pairs.clear();
  for (int i = n - 1; i >= 1; --i) {
    if (!w.active[i]) continue;
    for (int j = i - 1; j >= 0; --j) {
      if (!w.active[j]) continue;
      if (is_static(w.bodies[i]) && is_static(w.bodies[j])) continue;
      const Aabb& a = box[i];
      const Aabb& b = box[j];
      if (bounds_overlap(a.x0, a.x1, b.x0, b.x1) && bounds_overlap(a.y0, a.y1, b.y0, b.y1)) {
        w.pairs.push_back(i);
        w.pairs.push_back(j);
      }
    }
  }
}

/* Grid.toGrid + Grid.culledKeys (Broadphase/Grid.hs:67-141), the broadphase
 * the step calls (Engine/Main.hs:75) with gridAxes = GridAxis 20 1 (-10) on
 * both axes (Engine/Main.hs:40-41): each body goes into every cell its box
 * covers, cell (cx, cy) = (floor((x - (-10)) / 1), floor((y - (-10)) / 1)),
 * keyed cx + 20 * cy (keys alias, as in the reference's IntMap); every cell's
 * bodies in descending order give candidate pairs, aabbCheck and the
 * not-both-static test keep the real ones, and sortBy descending + uniq
 * makes the list.  The result equals the Aabb list above (see broadphase);
 * boxes with a non-finite or huge coordinate take that path instead. */
static void grid_broadphase(World& w) {
  const int n = (int)w.bodies.size();
  std::vector<Aabb> box(n);
  for (int i = 0; i < n; ++i) {
    box[i] = hull_aabb(w.hulls[i]);
    const Aabb& a = box[i];
    const double lim = 1e9;
    if (w.active[i] && !(std::fabs(a.x0) < lim && std::fabs(a.x1) < lim && std::fabs(a.y0) < lim && std::fabs(a.y1) < lim)) {
      broadphase(w);
      return;
    }
  }
  auto axial = [](double v) { return (int64_t)std::floor((v - (-10.0)) / 1.0); };
  std::vector<std::pair<int64_t, int>> entries; /* (cell key, body) */
  for (int i = 0; i < n; ++i) {
    if (!w.active[i]) continue; /* empty slots are not traversed (EmptiesVector.mapM_) */
    const Aabb& a = box[i];
    for (int64_t cx = axial(a.x0); cx <= axial(a.x1); ++cx)
      for (int64_t cy = axial(a.y0); cy <= axial(a.y1); ++cy) entries.emplace_back(cx + cy * 20, i);
  }
  /* cells in key order, bodies descending within a cell, one entry per body */
  std::sort(entries.begin(), entries.end(), [](const std::pair<int64_t, int>& p, const std::pair<int64_t, int>& q) {
    return p.first != q.first ? p.first < q.first : p.second > q.second;
  });
  entries.erase(std::unique(entries.begin(), entries.end()), entries.end());
  std::vector<std::pair<int, int>> found;
  for (size_t s0 = 0; s0 < entries.size();) {
    size_t s1 = s0;
    while (s1 < entries.size() && entries[s1].first == entries[s0].first) ++s1;
    for (size_t p = s0; p < s1; ++p)
      for (size_t q = p + 1; q < s1; ++q) {
        const int i = entries[p].second, j = entries[q].second; /* i > j */
        if (is_static(w.bodies[i]) && is_static(w.bodies[j])) continue;
        const Aabb& a = box[i];
        const Aabb& b = box[j];
        if (bounds_overlap(a.x0, a.x1, b.x0, b.x1) && bounds_overlap(a.y0, a.y1, b.y0, b.y1))
          found.emplace_back(i, j);
      }
    s0 = s1;
  }
  std::sort(found.begin(), found.end(), [](const std::pair<int, int>& p, const std::pair<int, int>& q) {
    return p > q;
  });
  found.erase(std::unique(found.begin(), found.end()), found.end());
  w.pairs.clear();
  for (const auto& pr : found) {
    w.pairs.push_back(pr.first);
    w.pairs.push_back(pr.second);
  }
}

/* ---- A6/A7 SAT and manifold ---------------------------------------------- */

struct SatResult {
  bool separated;
  int edge;     /* index of the penetrated edge's first vertex in sEdge */
  double depth;
  int pen;      /* index of the penetrating vertex in sPen */
};

/* overlap (SAT.hs:103-118) with extentAlongSelf (ConvexHull.hs:111-118),
 * extentAlong (ConvexHull.hs:94-100) and overlapAmount/overlapTest
 * (SAT.hs:74-95): depth = max(self) - min(pen) if the intervals overlap. */
static SatResult overlap_axis(const Hull& se, int e, const Hull& sp) {
  double dx = se.nx[e], dy = se.ny[e];
  int mi = se.emin[e], ma = se.emax[e];
  double sa = se.wx[mi] * dx + se.wy[mi] * dy;
  double sb = se.wx[ma] * dx + se.wy[ma] * dy;
  int pmin, pmax;
  double pa, pb;
  extent_along(sp.wx.data(), sp.wy.data(), sp.nv, dx, dy, &pmin, &pmax, &pa, &pb);
  SatResult r;
  r.edge = e;
  r.pen = pmin;
  if (pa > sb || pb < sa) {
    r.separated = true;
    r.depth = 0.0;
  } else {
    r.separated = false;
    r.depth = sb - pa;
  }
  return r;
}

/* minOverlap (SAT.hs:121-138): foldl1 keeping the first Separated axis, else
 * the first strictly smallest depth, over the edges in index order. */
static SatResult min_overlap(const Hull& se, const Hull& sp) {
  SatResult acc = overlap_axis(se, 0, sp);
  for (int e = 1; e < se.nv; ++e) {
    if (acc.separated) break; /* the fold can no longer change its result */
    SatResult o = overlap_axis(se, e, sp);
    if (o.separated) acc = o;
    else if (o.depth < acc.depth) acc = o;
  }
  return acc;
}

struct ClipPt {
  int idx;
  double x, y;
};

enum { CLIP_NONE = 0, CLIP_LEFT = 1, CLIP_RIGHT = 2, CLIP_BOTH = 3 };

/* clipSegment (Linear.hs:327-343) with intersect2 (Linear.hs:244-251) and
 * invM2x2 (Linear.hs:194-199).  Returns the clip kind; (*cx, *cy) = point. */
static int clip_segment(double bpx, double bpy, double bnx, double bny,  /* boundary */
                        double ipx, double ipy, double inx, double iny,  /* incident line */
                        double ax, double ay, double bx, double by,      /* segment */
                        double* cx, double* cy) {
  double b0 = bpx * bnx + bpy * bny;
  double b1 = ipx * inx + ipy * iny;
  double det = bnx * iny - bny * inx;
  double inv = 1.0 / det;
  double m00 = iny * inv, m01 = (-bny) * inv, m10 = (-inx) * inv, m11 = bnx * inv;
  double x = m00 * b0 + m01 * b1;
  double y = m10 * b0 + m11 * b1;
  *cx = x;
  *cy = y;
  double a_ = ax * bnx + ay * bny;
  double b_ = bx * bnx + by * bny;
  double c_ = x * bnx + y * bny;
  if (a_ < c_) return b_ < c_ ? CLIP_BOTH : CLIP_LEFT;
  if (b_ < c_) return CLIP_RIGHT;
  return CLIP_NONE;
}

/* contact_ (SAT.hs:261-267): penetratedEdge (SAT.hs:169-171), penetratingEdge
 * (SAT.hs:152-166), clipEdge (SAT.hs:190-218) with lApplyClip' / applyClip''
 * (Linear.hs:281-321), flattenContactPoints (SAT.hs:181-187).  Writes up to two
 * points in descending vertex-index order and returns their count (0 = the
 * manifold was clipped away). */
static int manifold(const Hull& se, int e, const Hull& sp, int pen, ClipPt out[2]) {
  const int ne = e < se.nv - 1 ? e + 1 : 0;
  const double ax = se.wx[e], ay = se.wy[e], bx = se.wx[ne], by = se.wy[ne];
  const double nx = se.nx[e], ny = se.ny[e];
  /* penetratingEdge */
  const int vb = pen, vc = pen < sp.nv - 1 ? pen + 1 : 0, va = pen > 0 ? pen - 1 : sp.nv - 1;
  double abn = std::fabs((sp.wx[vb] - sp.wx[va]) * nx + (sp.wy[vb] - sp.wy[va]) * ny);
  double bcn = std::fabs((sp.wx[vc] - sp.wx[vb]) * nx + (sp.wy[vc] - sp.wy[vb]) * ny);
  ClipPt c, d;
  if (bcn < abn) {
    c = {vb, sp.wx[vb], sp.wy[vb]};
    d = {vc, sp.wx[vc], sp.wy[vc]};
  } else {
    c = {va, sp.wx[va], sp.wy[va]};
    d = {vb, sp.wx[vb], sp.wy[vb]};
  }
  /* cd' = toLine2 c d (Linear.hs:233-236): point c, normal clockwise(d - c) */
  const double lpx = c.x, lpy = c.y;
  const double lnx = d.y - c.y, lny = -(d.x - c.x);
  double px, py;
  /* clip against perpLine2 a b (Linear.hs:238-241) */
  int k = clip_segment(ax, ay, bx - ax, by - ay, lpx, lpy, lnx, lny, c.x, c.y, d.x, d.y, &px, &py);
  if (k == CLIP_BOTH) return 0;
  if (k == CLIP_LEFT) { c.x = px; c.y = py; }
  if (k == CLIP_RIGHT) { d.x = px; d.y = py; }
  /* clip against perpLine2 b a */
  k = clip_segment(bx, by, ax - bx, ay - by, lpx, lpy, lnx, lny, c.x, c.y, d.x, d.y, &px, &py);
  if (k == CLIP_BOTH) return 0;
  if (k == CLIP_LEFT) { c.x = px; c.y = py; }
  if (k == CLIP_RIGHT) { d.x = px; d.y = py; }
  /* clip against Line2 a (negateV2 n); applyClip'' drops clipped points */
  k = clip_segment(ax, ay, -nx, -ny, lpx, lpy, lnx, lny, c.x, c.y, d.x, d.y, &px, &py);
  if (k == CLIP_BOTH) return 0;
  if (k == CLIP_LEFT) { out[0] = d; return 1; }
  if (k == CLIP_RIGHT) { out[0] = c; return 1; }
  if (c.idx > d.idx) { out[0] = c; out[1] = d; }
  else { out[0] = d; out[1] = c; }
  return 2;
}

/* HullVsHull.generateContacts (HullVsHull.hs:85-90) = flattenContactResult
 * (HullVsHull.hs:54-76) of SAT.contact (SAT.hs:238-258), with contactDepth_
 * (HullVsHull.hs:30-37) and eitherBranchBoth (Utils.hs:230-235): a Separated
 * axis either way gives nothing; otherwise Same if depth_ab < depth_ba, else
 * Flip (ties flip).  Appends keyed contacts for pair (i, j) in descending
 * feature order. */
static void hull_contacts(int32_t i, int32_t j, const Hull& a, const Hull& b,
                          std::vector<Contact>& out) {
  SatResult ab = min_overlap(a, b);
  if (ab.separated) return;
  SatResult ba = min_overlap(b, a);
  if (ba.separated) return;
  const bool flip = !(ab.depth < ba.depth);
  const SatResult& o = flip ? ba : ab;
  const Hull& se = flip ? b : a;
  const Hull& sp = flip ? a : b;
  ClipPt pts[2];
  int np = manifold(se, o.edge, sp, o.pen, pts);
  const double nx = se.nx[o.edge], ny = se.ny[o.edge];
  const double vx = se.wx[o.edge], vy = se.wy[o.edge];
  for (int q = 0; q < np; ++q) {
    Contact ct;
    ct.key.i = i;
    ct.key.j = j;
    if (flip) { ct.key.fa = pts[q].idx; ct.key.fb = o.edge; }
    else { ct.key.fa = o.edge; ct.key.fb = pts[q].idx; }
    ct.flip = flip ? 1 : 0;
    ct.nx = nx;
    ct.ny = ny;
    ct.px = pts[q].x;
    ct.py = pts[q].y;
    ct.depth = (vx * nx + vy * ny) - (pts[q].x * nx + pts[q].y * ny);
    out.push_back(ct);
  }
}

/* ---- circles (N2) --------------------------------------------------------- */

static inline double dot2(double ax, double ay, double bx, double by) { return ax * bx + ay * by; }

/* Circle.contact (Contact/Circle.hs:27-56): a is penetrated, b penetrates. */
static bool circle_circle(const Hull& a, const Hull& b, double* nx, double* ny, double* px, double* py,
                          double* depth) {
  const double ax = a.wx[0], ay = a.wy[0], bx = b.wx[0], by = b.wy[0];
  const double abx = bx - ax, aby = by - ay;
  const double ra = a.radius, rb = b.radius;
  const double rab = ra + rb;
  const double ab_sq = abx * abx + aby * aby;
  if (!(rab * rab >= ab_sq)) return false;
  const double len = std::sqrt(ab_sq);
  const double ux = abx / len, uy = aby / len;
  const double a1x = ux * ra + ax, a1y = uy * ra + ay;
  const double b1x = ux * (-rb) + bx, b1y = uy * (-rb) + by;
  *nx = ux;
  *ny = uy;
  *px = (a1x + b1x) / 2.0;
  *py = (a1y + b1y) / 2.0;
  *depth = ra + rb - len;
  return true;
}

/* crossV2V2 (Linear.hs:135-139): (a x b) x c. */
static inline void cross3(double ax, double ay, double bx, double by, double cx, double cy, double* x,
                          double* y) {
  const double abz = ax * by - ay * bx;
  *x = -(abz * cy);
  *y = abz * cx;
}

/* support (ConvexHull.hs:124-128): the first vertex of largest projection. */
static int support(const Hull& h, double dx, double dy) {
  int best = 0;
  double bd = dot2(h.wx[0], h.wy[0], dx, dy);
  for (int k = 1; k < h.nv; ++k) {
    const double t = dot2(h.wx[k], h.wy[k], dx, dy);
    if (t > bd) { bd = t; best = k; }
  }
  return best;
}

/* GJK.closestSimplex (GJK.hs:52-66) from vertex 0 toward the point (ox, oy).
 * Returns the simplex size (1, 2, or 3 = encloses the point) with s[0] the
 * vertex added last.  The reference loop has no bound; this one stops after
 * 4 nv + 8 extensions (treated as a failed search), a bound an ordinary
 * convex hull never reaches. */
static int closest_simplex(const Hull& h, double ox, double oy, int s[3]) {
  int n = 1;
  s[0] = 0;
  double dx = ox - h.wx[0], dy = oy - h.wy[0];
  for (int it = 0; it < 4 * h.nv + 8; ++it) {
    const int a = support(h, dx, dy);
    if (n == 1) { /* extendSimplex1 */
      if (a == s[0]) return 1;
      s[1] = s[0];
      s[0] = a;
      n = 2;
      /* shiftSimplex2 (GJK.hs:95-107) */
      const double abx = h.wx[s[1]] - h.wx[a], aby = h.wy[s[1]] - h.wy[a];
      const double aox = ox - h.wx[a], aoy = oy - h.wy[a];
      if (dot2(abx, aby, aox, aoy) > 0.0) {
        cross3(abx, aby, aox, aoy, abx, aby, &dx, &dy);
      } else {
        n = 1;
        dx = aox;
        dy = aoy;
      }
      continue;
    }
    /* extendSimplex2 */
    if (a == s[0] || a == s[1]) return 2;
    const int b = s[0], c = s[1];
    /* shiftSimplex3 (GJK.hs:109-135) on (a, b, c) */
    const double ax = h.wx[a], ay = h.wy[a];
    const double abx = h.wx[b] - ax, aby = h.wy[b] - ay;
    const double acx = h.wx[c] - ax, acy = h.wy[c] - ay;
    const double aox = ox - ax, aoy = oy - ay;
    const double abc = abx * acy - aby * acx;
    const double abcacx = -(abc * acy), abcacy = abc * acx;
    const double ababcx = aby * abc, ababcy = -(abx * abc);
    auto star = [&]() {
      if (dot2(abx, aby, aox, aoy) > 0.0) {
        s[0] = a; s[1] = b; n = 2;
        cross3(abx, aby, aox, aoy, abx, aby, &dx, &dy);
      } else {
        s[0] = a; n = 1;
        dx = aox; dy = aoy;
      }
    };
    if (dot2(abcacx, abcacy, aox, aoy) > 0.0) {
      if (dot2(acx, acy, aox, aoy) > 0.0) {
        s[0] = a; s[1] = c; n = 2;
        cross3(acx, acy, aox, aoy, acx, acy, &dx, &dy);
      } else {
        star();
      }
    } else if (dot2(ababcx, ababcy, aox, aoy) > 0.0) {
      star();
    } else {
      s[0] = a; s[1] = b; s[2] = c;
      return 3;
    }
  }
  return n;
}

/* CircleVsHull.generateContacts (CircleVsHull.hs:18-69): the circle
 * penetrates; one contact at the closest hull point, keyed by the feature
 * (vertex) the GJK simplex ended on; none for a 3-point simplex. */
static bool circle_hull(const Hull& circ, const Hull& hull, int* feature, double* nx, double* ny, double* px,
                        double* py, double* depth) {
  const double ox = circ.wx[0], oy = circ.wy[0];
  int s[3];
  const int n = closest_simplex(hull, ox, oy, s);
  if (n == 3) return false;
  double qx, qy;
  if (n == 1) {
    qx = hull.wx[s[0]];
    qy = hull.wy[s[0]];
  } else { /* closestAlong (CircleVsHull.hs:61-69) */
    const double ax = hull.wx[s[0]], ay = hull.wy[s[0]];
    const double aox = ox - ax, aoy = oy - ay;
    const double abx = hull.wx[s[1]] - ax, aby = hull.wy[s[1]] - ay;
    const double l = std::sqrt(abx * abx + aby * aby);
    const double ux = abx / l, uy = aby / l;
    const double t = dot2(aox, aoy, ux, uy);
    qx = ux * t + ax;
    qy = uy * t + ay;
  }
  /* processSimplex_ (CircleVsHull.hs:44-59) */
  const double r = circ.radius;
  const double bx = ox - qx, by = oy - qy;
  const double ab_sq = bx * bx + by * by;
  if (r * r < ab_sq) return false;
  const double len = std::sqrt(ab_sq);
  *feature = s[0];
  *nx = -(bx / len);
  *ny = -(by / len);
  *px = qx;
  *py = qy;
  *depth = r - len;
  return true;
}

/* Contact.generateContacts (Contact.hs:22-40) for pairs with a circle. */
static void circle_contacts(int32_t i, int32_t j, const Hull& a, const Hull& b, std::vector<Contact>& out) {
  Contact ct;
  ct.key.i = i;
  ct.key.j = j;
  int f = 0;
  bool hit;
  if (a.radius > 0.0 && b.radius > 0.0) {
    hit = circle_circle(a, b, &ct.nx, &ct.ny, &ct.px, &ct.py, &ct.depth);
    ct.key.fa = 0; ct.key.fb = 0; ct.flip = 0;
  } else if (a.radius > 0.0) {
    hit = circle_hull(a, b, &f, &ct.nx, &ct.ny, &ct.px, &ct.py, &ct.depth);
    ct.key.fa = 0; ct.key.fb = f; ct.flip = 0;
  } else {
    hit = circle_hull(b, a, &f, &ct.nx, &ct.ny, &ct.px, &ct.py, &ct.depth);
    ct.key.fa = f; ct.key.fb = 0; ct.flip = 1;
  }
  if (hit) out.push_back(ct);
}

/* prepareFrame (Solvers/Contact.hs:40-52) via keyedContacts
 * (Constraints/Contact.hs:49-57): contacts of every broadphase pair, in pair
 * order, concatenated. */
static void narrowphase(World& w) {
  w.contacts.clear();
  const size_t np = w.pairs.size() / 2;
  for (size_t p = 0; p < np; ++p) {
    int32_t i = w.pairs[2 * p], j = w.pairs[2 * p + 1];
    if (w.hulls[i].radius > 0.0 || w.hulls[j].radius > 0.0)
      circle_contacts(i, j, w.hulls[i], w.hulls[j], w.contacts);
    else
      hull_contacts(i, j, w.hulls[i], w.hulls[j], w.contacts);
  }
}

/* ---- A8 constraint generation -------------------------------------------- */

static inline double cross2(double ax, double ay, double bx, double by) { return ax * by - ay * bx; }

/* NonPenetration.jacobian (NonPenetration.hs:34-44) for (a penetrated by b). */
static inline void jac_nonpen(double nx, double ny, double px, double py, const Body& a,
                              const Body& b, double j[6]) {
  j[0] = -nx;
  j[1] = -ny;
  j[2] = cross2(a.px - px, a.py - py, nx, ny);
  j[3] = nx;
  j[4] = ny;
  j[5] = cross2(px - b.px, py - b.py, nx, ny);
}

/* Friction.jacobian (Friction.hs:31-44): tb = clockwise n, ta = -tb. */
static inline void jac_friction(double nx, double ny, double px, double py, const Body& a,
                                const Body& b, double j[6]) {
  double tbx = ny, tby = -nx;
  double tax = -tbx, tay = -tby;
  j[0] = tax;
  j[1] = tay;
  j[2] = cross2(px - a.px, py - a.py, tax, tay);
  j[3] = tbx;
  j[4] = tby;
  j[5] = cross2(px - b.px, py - b.py, tbx, tby);
}

/* constraintGen (Constraints/Contact.hs:60-72): NonPenetration.constraintGen
 * (NonPenetration.hs:16-23, baumgarte 48-56), Restitution.constraintGen
 * (Restitution.hs:21-31) and Friction.constraintGen (Friction.hs:18-23); a Flip
 * contact is solved with the bodies swapped and its Jacobian halves swapped
 * back (flipMap/flipExtract, Utils.hs:175-215; Flippable Constraint,
 * Constraint.hs:96-98). */
static ContactConstraint constraint_gen(const StepConfig& cfg, const Contact& ct, const Body& a,
                                        const Body& b) {
  ContactConstraint cc;
  double jn[6], jf[6];
  if (!ct.flip) {
    jac_nonpen(ct.nx, ct.ny, ct.px, ct.py, a, b, jn);
    jac_friction(ct.nx, ct.ny, ct.px, ct.py, a, b, jf);
    for (int k = 0; k < 6; ++k) { cc.jn[k] = jn[k]; cc.jf[k] = jf[k]; }
  } else {
    jac_nonpen(ct.nx, ct.ny, ct.px, ct.py, b, a, jn);
    jac_friction(ct.nx, ct.ny, ct.px, ct.py, b, a, jf);
    for (int k = 0; k < 3; ++k) {
      cc.jn[k] = jn[k + 3]; cc.jn[k + 3] = jn[k];
      cc.jf[k] = jf[k + 3]; cc.jf[k + 3] = jf[k];
    }
  }
  cc.bn = ct.depth > cfg.slop ? (cfg.beta / cfg.dt) * (cfg.slop - ct.depth) : 0.0;
  cc.rax = ct.px - a.px;
  cc.ray = ct.py - a.py;
  cc.rbx = ct.px - b.px;
  cc.rby = ct.py - b.py;
  cc.rnx = ct.flip ? -ct.nx : ct.nx;
  cc.rny = ct.flip ? -ct.ny : ct.ny;
  return cc;
}

/* ---- A9/A10 impulses ------------------------------------------------------ */

/* applyLagrangian (Constraint.hs:215-221) → applyLagrangian2 (Constraint.hs:197-204):
 * v += (J * lambda) * invMass, element-wise. */
static inline void apply_lagrangian(double l, const double j[6], Body& a, Body& b) {
  a.vx = a.vx + (j[0] * l) * a.iml;
  a.vy = a.vy + (j[1] * l) * a.iml;
  a.w = a.w + (j[2] * l) * a.imr;
  b.vx = b.vx + (j[3] * l) * b.iml;
  b.vy = b.vy + (j[4] * l) * b.iml;
  b.w = b.w + (j[5] * l) * b.imr;
}

/* applySln (Solvers/Contact.hs:55-65): non-penetration first, then friction. */
static inline void apply_sln(double ln, double lf, const ContactConstraint& cc, Body& a, Body& b) {
  apply_lagrangian(ln, cc.jn, a, b);
  apply_lagrangian(lf, cc.jf, a, b);
}

/* lagrangian2 (Constraint.hs:164-169) with velocity2 (152-158) and effMassM2
 * (173-179): lambda = (-(J·v + b)) / ((J ⊙ M⁻¹)·J). */
static inline double lagrangian2(const Body& a, const Body& b, const double j[6], double bias) {
  const double v[6] = {a.vx, a.vy, a.w, b.vx, b.vy, b.w};
  const double m[6] = {a.iml, a.iml, a.imr, b.iml, b.iml, b.imr};
  double jv = j[0] * v[0];
  for (int k = 1; k < 6; ++k) jv = jv + j[k] * v[k];
  double mc = (j[0] * m[0]) * j[0];
  for (int k = 1; k < 6; ++k) mc = mc + (j[k] * m[k]) * j[k];
  return (-(jv + bias)) / mc;
}

/* improveContactSln (Solvers/Contact.hs:124-143): contactLagrangian
 * (Constraints/Contact.hs:74-95) with bounceB (Restitution.hs:34-51), then
 * solutionProcessor (Constraints/Contact.hs:101-110) = positive for the normal
 * (SolutionProcessors.hs:33-35) and clampAbs by nonpen·pairMu for friction
 * (SolutionProcessors.hs:42-53, Friction.hs:46-56), then applySln. */
static inline void improve_amounts(const ContactConstraint& cc, const CacheEntry& cache, const Body& a,
                                   const Body& b, double* ln_apply_out, double* lf_apply_out, double* ln_cache_out,
                                   double* lf_cache_out) {
  /* bounceB */
  const double e = a.bounce <= b.bounce ? a.bounce : b.bounce;
  const double nwax = -((-a.w) * cc.ray), nway = (-a.w) * cc.rax;
  const double wbx = -(b.w * cc.rby), wby = b.w * cc.rbx;
  const double cvx = ((-a.vx + nwax) + b.vx) + wbx;
  const double cvy = ((-a.vy + nway) + b.vy) + wby;
  const double t = e * (cvx * cc.rnx + cvy * cc.rny);
  const double bounce = 0.0 <= t ? 0.0 : t;
  const double ln_new = lagrangian2(a, b, cc.jn, cc.bn + bounce);
  const double lf_new = lagrangian2(a, b, cc.jf, 0.0);
  /* positive */
  const double neg_cn = -cache.ln;
  const double ln_apply = ln_new <= neg_cn ? neg_cn : ln_new;
  const double ln_cache = cache.ln + ln_apply;
  /* clampAbs (nonpen * pairMu) */
  const double mu = (a.mu + b.mu) / 2.0;
  const double thr = ln_cache * mu;
  const double acc = cache.lf + lf_new;
  const double acc2 = acc > thr ? thr : (acc < -thr ? -thr : acc);
  *ln_apply_out = ln_apply;
  *lf_apply_out = acc2 - cache.lf;
  *ln_cache_out = ln_cache;
  *lf_cache_out = acc2;
}

static inline void improve_contact(const ContactConstraint& cc, CacheEntry& cache, Body& a, Body& b) {
  double ln_apply, lf_apply, ln_cache, lf_cache;
  improve_amounts(cc, cache, a, b, &ln_apply, &lf_apply, &ln_cache, &lf_cache);
  apply_sln(ln_apply, lf_apply, cc, a, b);
  cache.ln = ln_cache;
  cache.lf = lf_cache;
}

/* ---- A12 the step -------------------------------------------------------- */

/* updateWorld (Engine/Main.hs:71-84). */
static void step_world(World& w, const StepConfig& cfg) {
  /* 1. broadphase on the shapes posed at the end of the previous step */
  grid_broadphase(w);
  /* 2. applyExternal (World.hs:156-158) with constantAccel (External.hs:23-28) */
  if (cfg.external) {
    for (size_t i = 0; i < w.bodies.size(); ++i) {
      Body& b = w.bodies[i];
      if (w.active[i] && !(0.0 == b.iml)) {
        b.vx = b.vx + cfg.ax * cfg.dt;
        b.vy = b.vy + cfg.ay * cfg.dt;
      }
    }
  }
  /* 3. prepareFrame */
  narrowphase(w);
  /* 4. applyCachedSlns (Solvers/Contact.hs:74-121) merging with the previous
   *    cache by descZipVector (Utils/Descending.hs:47-71) */
  const size_t C = w.contacts.size();
  std::vector<ContactConstraint> cons(C);
  std::vector<CacheEntry> lag(C);
  size_t that = 0;
  const std::vector<CacheEntry>& old = w.cache;
  for (size_t k = 0; k < C; ++k) {
    const Contact& ct = w.contacts[k];
    Body& a = w.bodies[ct.key.i];
    Body& b = w.bodies[ct.key.j];
    cons[k] = constraint_gen(cfg, ct, a, b);
    bool hit = false;
    size_t hit_at = 0;
    if (cfg.warm_start) {
      while (that < old.size()) {
        if (key_lt(ct.key, old[that].key)) { ++that; continue; }
        if (key_eq(ct.key, old[that].key)) { hit = true; hit_at = that; ++that; }
        break;
      }
    }
    if (hit) {
      apply_sln(old[hit_at].ln, old[hit_at].lf, cons[k], a, b);
      lag[k] = old[hit_at];
    } else {
      lag[k].key = ct.key;
      lag[k].ln = 0.0;
      lag[k].lf = 0.0;
    }
  }
  /* 5. improveWorld (Solvers/Contact.hs:146-157), `iterations` sweeps */
  for (int it = 0; it < cfg.iterations; ++it) {
    for (size_t k = 0; k < C; ++k) {
      const Contact& ct = w.contacts[k];
      improve_contact(cons[k], lag[k], w.bodies[ct.key.i], w.bodies[ct.key.j]);
    }
  }
  /* Solver residual (no reference counterpart): the amounts one more sweep
   * would apply, every contact seeing the final velocities; RMS over the normal
   * and friction amounts of all contacts. */
  {
    double sum = 0.0;
    for (size_t k = 0; k < C; ++k) {
      const Contact& ct = w.contacts[k];
      double dn, df, cn, cf;
      improve_amounts(cons[k], lag[k], w.bodies[ct.key.i], w.bodies[ct.key.j], &dn, &df, &cn, &cf);
      sum += dn * dn + df * df;
    }
    w.residual = C ? std::sqrt(sum / (2.0 * (double)C)) : 0.0;
  }
  w.cache.swap(lag);
  /* 6. advance (World.hs:167-169) → advanceObj (Constraint.hs:225-229) */
  for (size_t i = 0; i < w.bodies.size(); ++i) {
    if (!w.active[i]) continue;
    Body& b = w.bodies[i];
    b.px = (b.vx * cfg.dt) + b.px;
    b.py = (b.vy * cfg.dt) + b.py;
    b.th = (cfg.dt * b.w) + b.th;
  }
  /* 7. moveShapes (World.hs:136-140) */
  for (size_t i = 0; i < w.bodies.size(); ++i)
    if (w.active[i]) pose_hull(w.bodies[i], w.hulls[i], w.trig_libm, &w.trig_mismatches);
}

static StepConfig make_cfg(const double* c5, int32_t iterations, int32_t warm_start, int32_t external) {
  StepConfig c;
  c.dt = c5[0]; c.beta = c5[1]; c.slop = c5[2]; c.ax = c5[3]; c.ay = c5[4];
  c.iterations = iterations; c.warm_start = warm_start; c.external = external;
  return c;
}

}  // namespace

extern "C" {

/* bodies10: n rows of (vx, vy, w, px, py, th, inv_mass_lin, inv_mass_rot, mu, bounce).
 * vert_off: n+1 offsets into local_xy (pairs).  Shapes are posed on creation
 * (makeWorldObj, World.hs:142-149) and the contact cache starts empty
 * (initEngine, Engine/Main.hs:43-46). */
void* oracle_world_create(int32_t n, const double* bodies10, const int32_t* vert_off,
                          const double* local_xy) {
  World* w = new World();
  w->bodies.resize(n);
  w->hulls.resize(n);
  w->active.assign(n, 1);
  for (int32_t i = 0; i < n; ++i) {
    const double* r = bodies10 + 10 * (size_t)i;
    w->bodies[i] = Body{r[0], r[1], r[2], r[3], r[4], r[5], r[6], r[7], r[8], r[9]};
    init_hull(w->hulls[i], vert_off[i + 1] - vert_off[i], local_xy + 2 * (size_t)vert_off[i]);
    pose_hull(w->bodies[i], w->hulls[i], w->trig_libm, &w->trig_mismatches);
  }
  return w;
}

void oracle_world_destroy(void* h) { delete static_cast<World*>(h); }

/* World.delete (World.hs:90-91) = EmptiesVector.safeDelete: the slot must be
 * filled; it becomes the top of the empty-slot stack.  Returns 0, or -1 for
 * an empty or out-of-range slot. */
int32_t oracle_world_delete(void* h, int32_t slot) {
  World& w = *static_cast<World*>(h);
  if (slot < 0 || slot >= (int32_t)w.bodies.size() || !w.active[slot]) return -1;
  w.active[slot] = 0;
  w.empties.push_back(slot);
  return 0;
}

/* World.append (World.hs:83-89) = EmptiesVector.append: fills the top of the
 * empty-slot stack; with no empty slot the world grows by one slot at the end
 * (the reference's vector would be full).  The shape is posed at once
 * (makeWorldObj, World.hs:142-149).  Returns the slot. */
int32_t oracle_world_append(void* h, const double* body10, int32_t nv, const double* local_xy) {
  World& w = *static_cast<World*>(h);
  int32_t slot;
  if (!w.empties.empty()) {
    slot = w.empties.back();
    w.empties.pop_back();
  } else {
    slot = (int32_t)w.bodies.size();
    w.bodies.emplace_back();
    w.hulls.emplace_back();
    w.active.push_back(0);
  }
  const double* r = body10;
  w.bodies[slot] = Body{r[0], r[1], r[2], r[3], r[4], r[5], r[6], r[7], r[8], r[9]};
  init_hull(w.hulls[slot], nv, local_xy);
  pose_hull(w.bodies[slot], w.hulls[slot], w.trig_libm, &w.trig_mismatches);
  w.active[slot] = 1;
  return slot;
}

/* Overwrites every body's ten fields (rows as in oracle_world_create) and
 * re-poses the shapes: updatePhysObj (World.hs:96-97) on every body, with the
 * shapes moved as the next step's moveShape would (World.hs:132-133). */
void oracle_world_set_bodies(void* h, const double* bodies10) {
  World& w = *static_cast<World*>(h);
  for (size_t i = 0; i < w.bodies.size(); ++i) {
    const double* r = bodies10 + 10 * i;
    w.bodies[i] = Body{r[0], r[1], r[2], r[3], r[4], r[5], r[6], r[7], r[8], r[9]};
    pose_hull(w.bodies[i], w.hulls[i], w.trig_libm, &w.trig_mismatches);
  }
}

void oracle_world_get_active(void* h, uint8_t* out) {
  World& w = *static_cast<World*>(h);
  for (size_t i = 0; i < w.active.size(); ++i) out[i] = w.active[i];
}

/* cfg5 = (dt, baumgarte, slop, accel_x, accel_y). */
void oracle_world_step(void* h, const double* cfg5, int32_t iterations, int32_t warm_start,
                       int32_t external, int32_t nsteps) {
  World& w = *static_cast<World*>(h);
  StepConfig cfg = make_cfg(cfg5, iterations, warm_start, external);
  for (int32_t s = 0; s < nsteps; ++s) step_world(w, cfg);
}

/* Broadphase + narrowphase on the current poses, nothing else (the demo's
 * worldContacts query, shapes-demo/src/Physics/Demo/IOWorld.hs:74-81). */
void oracle_world_collide(void* h) {
  World& w = *static_cast<World*>(h);
  grid_broadphase(w);
  narrowphase(w);
}

double oracle_world_residual(void* h) { return static_cast<World*>(h)->residual; }

int32_t oracle_world_num_bodies(void* h) { return (int32_t) static_cast<World*>(h)->bodies.size(); }

void oracle_world_get_bodies(void* h, double* out10) {
  World& w = *static_cast<World*>(h);
  for (size_t i = 0; i < w.bodies.size(); ++i) {
    const Body& b = w.bodies[i];
    double* r = out10 + 10 * i;
    r[0] = b.vx; r[1] = b.vy; r[2] = b.w; r[3] = b.px; r[4] = b.py;
    r[5] = b.th; r[6] = b.iml; r[7] = b.imr; r[8] = b.mu; r[9] = b.bounce;
  }
}

/* World vertices and unit normals of the current pose, in vertex order. */
void oracle_world_get_shapes(void* h, double* world_xy, double* normal_xy) {
  World& w = *static_cast<World*>(h);
  size_t o = 0;
  for (const Hull& hl : w.hulls) {
    for (int k = 0; k < hl.nv; ++k, ++o) {
      world_xy[2 * o] = hl.wx[k];
      world_xy[2 * o + 1] = hl.wy[k];
      normal_xy[2 * o] = hl.nx[k];
      normal_xy[2 * o + 1] = hl.ny[k];
    }
  }
}

void oracle_world_get_extents(void* h, int32_t* out2) {
  World& w = *static_cast<World*>(h);
  size_t o = 0;
  for (const Hull& hl : w.hulls)
    for (int k = 0; k < hl.nv; ++k, ++o) { out2[2 * o] = hl.emin[k]; out2[2 * o + 1] = hl.emax[k]; }
}

int64_t oracle_world_num_pairs(void* h) { return (int64_t) static_cast<World*>(h)->pairs.size() / 2; }

void oracle_world_get_pairs(void* h, int32_t* out2) {
  World& w = *static_cast<World*>(h);
  std::memcpy(out2, w.pairs.data(), w.pairs.size() * sizeof(int32_t));
}

int64_t oracle_world_num_contacts(void* h) { return (int64_t) static_cast<World*>(h)->contacts.size(); }

/* keys5: (i, j, feature_a, feature_b, flip); vals5: (nx, ny, px, py, depth). */
void oracle_world_get_contacts(void* h, int32_t* keys5, double* vals5) {
  World& w = *static_cast<World*>(h);
  for (size_t k = 0; k < w.contacts.size(); ++k) {
    const Contact& c = w.contacts[k];
    keys5[5 * k] = c.key.i; keys5[5 * k + 1] = c.key.j;
    keys5[5 * k + 2] = c.key.fa; keys5[5 * k + 3] = c.key.fb; keys5[5 * k + 4] = c.flip;
    vals5[5 * k] = c.nx; vals5[5 * k + 1] = c.ny; vals5[5 * k + 2] = c.px;
    vals5[5 * k + 3] = c.py; vals5[5 * k + 4] = c.depth;
  }
}

int64_t oracle_world_num_cache(void* h) { return (int64_t) static_cast<World*>(h)->cache.size(); }

void oracle_world_get_cache(void* h, int32_t* keys4, double* lam2) {
  World& w = *static_cast<World*>(h);
  for (size_t k = 0; k < w.cache.size(); ++k) {
    const CacheEntry& c = w.cache[k];
    keys4[4 * k] = c.key.i; keys4[4 * k + 1] = c.key.j;
    keys4[4 * k + 2] = c.key.fa; keys4[4 * k + 3] = c.key.fb;
    lam2[2 * k] = c.ln; lam2[2 * k + 1] = c.lf;
  }
}

void oracle_world_set_cache(void* h, int64_t n, const int32_t* keys4, const double* lam2) {
  World& w = *static_cast<World*>(h);
  w.cache.resize((size_t)n);
  for (int64_t k = 0; k < n; ++k) {
    CacheEntry& c = w.cache[k];
    c.key = Key{keys4[4 * k], keys4[4 * k + 1], keys4[4 * k + 2], keys4[4 * k + 3]};
    c.ln = lam2[2 * k];
    c.lf = lam2[2 * k + 1];
  }
}

/* Steps many independent worlds, `nthreads` host threads taking whole worlds
 * round-robin.  Returns wall seconds. */
double oracle_batch_step(int32_t nworlds, void** worlds, const double* cfg5, int32_t iterations,
                         int32_t warm_start, int32_t external, int32_t nsteps, int32_t nthreads) {
  StepConfig cfg = make_cfg(cfg5, iterations, warm_start, external);
  if (nthreads < 1) nthreads = 1;
  auto t0 = std::chrono::steady_clock::now();
  std::vector<std::thread> pool;
  for (int32_t t = 0; t < nthreads; ++t) {
    pool.emplace_back([&, t]() {
      for (int32_t wi = t; wi < nworlds; wi += nthreads) {
        World& w = *static_cast<World*>(worlds[wi]);
        for (int32_t s = 0; s < nsteps; ++s) step_world(w, cfg);
      }
    });
  }
  for (auto& th : pool) th.join();
  auto t1 = std::chrono::steady_clock::now();
  return std::chrono::duration<double>(t1 - t0).count();
}

/* SAT.contact on two hulls built by listToHull from the given (already posed)
 * vertices — the bench fixture path (shapes/bench/Physics/Contact/Benchmark.hs:16-30).
 * Writes (feature_a, feature_b, flip) and (nx, ny, px, py, depth) per contact. */
int32_t oracle_hull_contacts(int32_t nva, const double* xya, int32_t nvb, const double* xyb,
                             int32_t* keys3, double* vals5) {
  Hull a, b;
  init_hull(a, nva, xya);
  init_hull(b, nvb, xyb);
  for (int k = 0; k < nva; ++k) { a.wx[k] = a.lx[k]; a.wy[k] = a.ly[k]; }
  for (int k = 0; k < nvb; ++k) { b.wx[k] = b.lx[k]; b.wy[k] = b.ly[k]; }
  for (int e = 0; e < nva; ++e) {
    int n1 = e < nva - 1 ? e + 1 : 0;
    unit_edge_normal(a.wx[e], a.wy[e], a.wx[n1], a.wy[n1], &a.nx[e], &a.ny[e]);
  }
  for (int e = 0; e < nvb; ++e) {
    int n1 = e < nvb - 1 ? e + 1 : 0;
    unit_edge_normal(b.wx[e], b.wy[e], b.wx[n1], b.wy[n1], &b.nx[e], &b.ny[e]);
  }
  std::vector<Contact> out;
  hull_contacts(0, 0, a, b, out);
  for (size_t k = 0; k < out.size(); ++k) {
    keys3[3 * k] = out[k].key.fa; keys3[3 * k + 1] = out[k].key.fb; keys3[3 * k + 2] = out[k].flip;
    vals5[5 * k] = out[k].nx; vals5[5 * k + 1] = out[k].ny; vals5[5 * k + 2] = out[k].px;
    vals5[5 * k + 3] = out[k].py; vals5[5 * k + 4] = out[k].depth;
  }
  return (int32_t)out.size();
}

/* solveConstraint (Constraint.hs:207-212) on one pair; bodies as
 * (vx, vy, w, inv_mass_lin, inv_mass_rot), updated in place. */
void oracle_solve_constraint(const double* j6, double bias, double* a5, double* b5) {
  Body a{a5[0], a5[1], a5[2], 0, 0, 0, a5[3], a5[4], 0, 0};
  Body b{b5[0], b5[1], b5[2], 0, 0, 0, b5[3], b5[4], 0, 0};
  double l = lagrangian2(a, b, j6, bias);
  apply_lagrangian(l, j6, a, b);
  a5[0] = a.vx; a5[1] = a.vy; a5[2] = a.w;
  b5[0] = b.vx; b5[1] = b.vy; b5[2] = b.w;
}

/* length (unorderedPairs n) (Aabb.hs:155-163), counted by walking the list. */
int64_t oracle_unordered_pairs_count(int32_t n) {
  if (n < 2) return 0;
  int64_t c = 0;
  for (int32_t x = n - 1; x >= 1; --x)
    for (int32_t y = x - 1; y >= 0; --y) ++c;
  return c;
}

void oracle_sincos(const double* x, double* s, double* c, int64_t n) {
  for (int64_t k = 0; k < n; ++k) shapes_sincos(x[k], &s[k], &c[k]);
}

/* The two phases of shapes_sincos separately (tests of the function itself):
 * mode 0 the accurate phase alone; mode 1 the fast phase's unrounded
 * double-double results (s hi, s lo, c hi, c lo in out4, ok[k] = 0 where it
 * declines); mode 2 the host libm's sin and cos. */
void oracle_sincos_phase(int32_t mode, const double* x, double* out4, uint8_t* ok, int64_t n) {
  for (int64_t k = 0; k < n; ++k) {
    double* o = out4 + 4 * k;
    if (mode == 0) {
      shapes_sincos_accurate(x[k], &o[0], &o[2]);
      o[1] = o[3] = 0.0;
      ok[k] = 1;
    } else if (mode == 1) {
      ok[k] = (uint8_t)shapes_sincos_fast(x[k], o);
    } else {
      o[0] = std::sin(x[k]);
      o[2] = std::cos(x[k]);
      o[1] = o[3] = 0.0;
      ok[k] = 1;
    }
  }
}

/* Counts, over n arguments, how often shapes_sincos differs from the host
 * libm (sin and cos separately) and how often the fast phase could not decide
 * (counts3 = sin mismatches, cos mismatches, accurate-phase calls).  Stores
 * up to `cap` mismatching arguments. */
void oracle_sincos_vs_libm(const double* x, int64_t n, int64_t* counts3, double* bad, int64_t cap) {
  int64_t ns = 0, nc = 0, na = 0, nb = 0;
  for (int64_t k = 0; k < n; ++k) {
    double s, c, o[4];
    shapes_sincos(x[k], &s, &c);
    const double ax = std::fabs(x[k]);
    if (ax >= 0x1p-27 && ax < 0x1p16 &&
        !(shapes_sincos_fast(x[k], o) && shapes_sc_decided(o[0], o[1]) && shapes_sc_decided(o[2], o[3])))
      ++na;
    const double ls = std::sin(x[k]), lc = std::cos(x[k]);
    const bool ds = std::memcmp(&s, &ls, 8) != 0, dc = std::memcmp(&c, &lc, 8) != 0;
    ns += ds;
    nc += dc;
    if ((ds || dc) && nb < cap) bad[nb++] = x[k];
  }
  counts3[0] = ns;
  counts3[1] = nc;
  counts3[2] = na;
}

/* Selects the rotation source of one world (0: shapes_sincos, 1: the host
 * libm's sin and cos) and re-poses its shapes with it.  The world's count of
 * libm poses that differ from shapes_sincos restarts at 0. */
void oracle_world_set_trig(void* h, int32_t libm) {
  World& w = *static_cast<World*>(h);
  w.trig_libm = libm != 0;
  w.trig_mismatches = 0;
  for (size_t i = 0; i < w.bodies.size(); ++i)
    if (w.active[i]) pose_hull(w.bodies[i], w.hulls[i], w.trig_libm, &w.trig_mismatches);
}

/* libm mode: how many poses so far used a libm sin or cos that differs from
 * the correctly rounded shapes_sincos value (every pose counts once). */
int64_t oracle_world_trig_mismatches(void* h) { return static_cast<World*>(h)->trig_mismatches; }

}  // extern "C"
