// queries.cu -- point-query kernels: closest (embree/ray_tracer.cpp:328-345)
// and find_element (embree/ray_tracer.cpp:226-257).
//
// One thread owns one query point for its whole traversal of a 4- or 8-wide BVH
// with a private stack, visiting the nearest children first (closest) or
// every child whose box contains the point (find_element).  The FP32 node
// tests are conservative -- boxes are rounded outward at build time and a
// point rounded to FP32 stays inside any FP32 box that contains it -- and the
// per-primitive tests (closest point on a triangle, tet containment) are the
// reference's FP64 formulas from geom.cuh, so results are bit-identical.
#include <algorithm>

#include "queries.h"
#include "traverse.cuh"

namespace xdgcu {

namespace {

constexpr int kBlock = 128;

// ---------------------------------------------------------------------------
// closest (point query, embree/ray_tracer.cpp:328-345)
// ---------------------------------------------------------------------------

constexpr unsigned kFullMask = 0xffffffffu;

// The point a thread of a point-query launch takes: its position in the
// launch, or the entry of a.order there (a point index; an entry out of
// range takes no point).
__device__ __forceinline__ int64_t point_index(const PointArgs& a) {
  const int64_t pos = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (!a.order || pos >= a.n) return pos;
  const int32_t o = __ldg(&a.order[pos]);
  return o >= 0 ? (int64_t)o : a.n;
}
// closest: candidates a lane keeps for its exact tests after the traversal
constexpr int kCand = 8;

// The children of record `rec` of inner node `ref` that may hold a facet no
// farther than `best`: their references in cr and lower bounds of the
// point's distance to their boxes in ck (FP32, rounded down; 0 where FP32
// cannot prune), nearest first.  Returns their number.
template <bool MIXED>
__device__ __forceinline__ int closest_children(const TreeDev& T, int32_t ref, int rec, d3 p,
                                                float px, float py, float pz, float pabs,
                                                bool f32ok, double best, int32_t cr[4],
                                                float ck[4]) {
  const int nrec = T.width / kWidth;
  int nhit = 0;
  if (MIXED) {
    const Node32* np = T.n32 + (int64_t)ref * nrec + rec;
    const float4 lx = __ldg(&np->lox), hx = __ldg(&np->hix), ly = __ldg(&np->loy),
                 hy = __ldg(&np->hiy), lz = __ldg(&np->loz), hz = __ldg(&np->hiz);
    const int4 c = __ldg(&np->child);
    const float la[3][4] = {{lx.x, lx.y, lx.z, lx.w}, {ly.x, ly.y, ly.z, ly.w},
                            {lz.x, lz.y, lz.z, lz.w}};
    const float ha[3][4] = {{hx.x, hx.y, hx.z, hx.w}, {hy.x, hy.y, hy.z, hy.w},
                            {hz.x, hz.y, hz.z, hz.w}};
    const float pa[3] = {px, py, pz};
    const int32_t ca[4] = {c.x, c.y, c.z, c.w};
    // prune only when the FP32 distance, shrunk by its error bound,
    // exceeds the current best (rounded up to float)
    const float bestf = __double2float_ru(best);
    float key[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      float s2 = 0.0f;
      bool empty = false;
#pragma unroll
      for (int ax = 0; ax < 3; ++ax) {
        empty |= !(la[ax][k] <= ha[ax][k]);
        const float e = fmaxf(fmaxf(la[ax][k] - pa[ax], pa[ax] - ha[ax][k]), 0.0f);
        s2 += e * e;
      }
      const float dist = sqrtf(s2);
      const float lb = dist * (1.0f - 8.0f * kU32) - 4.0f * kU32 * pabs;
      // the key is the lower bound itself (0 where FP32 cannot prune)
      key[k] = (!empty && (lb <= bestf || !f32ok)) ? (f32ok ? fmaxf(lb, 0.0f) : 0.0f) : INFINITY;
      cr[k] = ca[k];
    }
    sort4(key, cr);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      nhit += key[k] < INFINITY ? 1 : 0;
      ck[k] = key[k];
    }
  } else {
    const Node64* np = T.n64 + (int64_t)ref * nrec + rec;
    const int4 c = __ldg(&np->child);
    const int32_t ca[4] = {c.x, c.y, c.z, c.w};
    double key[4];
    const double pa[3] = {p.x, p.y, p.z};
    const double* lo[3] = {np->lox, np->loy, np->loz};
    const double* hi[3] = {np->hix, np->hiy, np->hiz};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      double s2 = 0.0;
      bool empty = false;
#pragma unroll
      for (int ax = 0; ax < 3; ++ax) {
        const double l = __ldg(lo[ax] + k), u = __ldg(hi[ax] + k);
        empty |= !(l <= u);
        const double e = fmax(fmax(l - pa[ax], pa[ax] - u), 0.0);
        s2 += e * e;
      }
      const double dist = sqrt(s2);
      key[k] = (!empty && dist * (1.0 - 1e-12) <= best) ? dist : INFINITY;
      cr[k] = ca[k];
    }
    sort4d(key, cr);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      nhit += key[k] < INFINITY ? 1 : 0;
      // rounded down: a lower bound of dist * (1 - 1e-12)
      ck[k] = key[k] < INFINITY ? __double2float_rd(key[k] * (1.0 - 1e-12)) : INFINITY;
    }
  }
  return nhit;
}

// p's FP32 distances to the face plane (h, unsigned) and beyond the three
// edge planes (s0..s2, positive outside) of global triangle gtri
struct PlaneDists {
  float h, s0, s1, s2;
};
__device__ __forceinline__ PlaneDists closest_planes32(const float4* __restrict__ tri_cb,
                                                       int32_t gtri, float px, float py, float pz) {
  const float4* cb = tri_cb + 4 * (int64_t)gtri;
  const float4 pn = __ldg(cb), e0 = __ldg(cb + 1), e1 = __ldg(cb + 2), e2 = __ldg(cb + 3);
  PlaneDists r;
  r.h = fabsf(__fmaf_rn(pn.x, px, __fmaf_rn(pn.y, py, __fmaf_rn(pn.z, pz, -pn.w))));
  r.s0 = __fmaf_rn(e0.x, px, __fmaf_rn(e0.y, py, __fmaf_rn(e0.z, pz, -e0.w)));
  r.s1 = __fmaf_rn(e1.x, px, __fmaf_rn(e1.y, py, __fmaf_rn(e1.z, pz, -e1.w)));
  r.s2 = __fmaf_rn(e2.x, px, __fmaf_rn(e2.y, py, __fmaf_rn(e2.z, pz, -e2.w)));
  return r;
}

// closest_lower_of: the certified FP32 lower bound of the point's distance to
// a triangle, and closest_may_win: whether the triangle may be no farther than
// `bestf` (the best distance rounded up to FP32) by it.  From the planes of
// tri_cbound: sqrt(h^2 + m^2) with h the distance to its face plane and m the
// largest distance beyond one of its edge planes.  With p exact, the triangle
// lies within 8 u M of the face plane and inside the edge planes, and the rows
// are orthonormal to 4 u, so the distance is at least that root less 8 u M,
// over 1 + 6 u.  The FP32 evaluation (p's rounding and three FMAs) is within
// about 7 u (|p| + M) of h and of each edge distance (M = max_abs).  The
// bound, less 48 u (|p| + M) (cmargin) and the rounding of the root,
// undershoots the distance by at least 20 u (|p| + M), far beyond the FP64
// rounding of the exact test; the triangle is skipped only when it still
// exceeds the best distance rounded up, so neither the minimum nor its tie
// rule can change.
__device__ __forceinline__ float closest_lower_of(const PlaneDists& d, float cmargin) {
  const float mo = fmaxf(fmaxf(fmaxf(d.s0, d.s1), d.s2), 0.0f);
  const float lb = __fsqrt_rn(__fmaf_rn(d.h, d.h, mo * mo));
  return lb * (1.0f - 8.0f * kU32) - cmargin;
}

__device__ __forceinline__ float closest_lower32(const float4* __restrict__ tri_cb, int32_t gtri,
                                                 float px, float py, float pz, float cmargin) {
  return closest_lower_of(closest_planes32(tri_cb, gtri, px, py, pz), cmargin);
}

__device__ __forceinline__ bool closest_may_win(const float4* __restrict__ tri_cb, int32_t gtri,
                                                float px, float py, float pz, float cmargin,
                                                float bestf) {
  return !(closest_lower32(tri_cb, gtri, px, py, pz, cmargin) > bestf);
}

// closest_record_bounds: hi, a certified FP32 upper bound of the distance
// the exact test (closest_location_on_triangle, closest.cpp:54-183) gives
// for the leaf-ordered triangle qq, or +inf.  That routine returns the true
// closest point in its regions zero to five, but in region six (p beyond the edges
// v0v1 and v1v2 near v1, :155-177) it extrapolates along v1v2 past v1, so a
// geometric bound does not bound it there.  The bound is given only where
// the routine certainly does not take region six and computes accurately:
//  - the triangle is well shaped at v0: (v1-v0)x(v2-v0) squared is at least
//    1e-6 of |v1-v0|^2 |v2-v0|^2 (a flag in the FP32 record's fourth slot,
//    set from FP64 at build), so the routine's FP64 region tests and weights
//    are within about 1e-8 (|p| + M) of exact, in position, and the edge
//    planes' directions are accurate to about u;
//  - p's FP32 distance beyond edge plane 0 (v0v1) or 1 (v1v2) is below
//    -cmargin: with the planes' certificates (face slab 7 u M, the rows
//    orthonormal to 4 u), the foot of p on the plane is inside that edge's
//    line by at least 7 u (|p| + M), so the routine's t > 0 or s + t < det
//    holds in FP64 and region six is not taken.
// Its result is then the triangle's closest point up to those errors, and
// any point Q of the triangle bounds it: Q = v0 + s e1 + t e2 with s, t >= 0
// and s + t <= 1 exactly (the projection of p clamped into the triangle, so
// that the bound is tight).  The FP32 record holds v0, e1 = v1 - v0 and
// e2 = v2 - v0 rounded to nearest (each within u |x|, u = 2^-24, |v0| <= M,
// |e| <= 2M per coordinate, M = max_abs), so Q evaluated by two FMAs is
// within 9.1 u M of Q per coordinate (16 u M in norm); the FP32 distance is
// within 3.1 u of |p32 - q32|, and p32 within sqrt(3) u |p| of p.  So
// d32 (1 + 8u) + 48 u (|p| + M) (cmargin), rounded up, bounds the exact
// test's distance with about 30 u (|p| + M) to spare.
//
// And lo, a certified FP32 lower bound of the same distance from
// the triangle's bounding box, which the plane bound misses for triangles
// whose plane passes near p (the "horizon" of a sphere seen from outside:
// the plane bound there undershoots by a third).  The vertices rebuilt from
// the FP32 record (A, A + B, A + C) are within 4 u M of the triangle's per
// coordinate, p32 within u |p| of p, and the FP32 box distance within 3 u of
// its value, so dist32 (1 - 8u) - cmargin is at most the distance from p to
// the triangle; and the exact test's point is on the triangle, or in region
// six farther from p than v1 (the foot of p on the line v1v2 mirrored across
// v1), so its distance is no smaller.
struct RecordBounds {
  float lo, hi;
};
__device__ __forceinline__ RecordBounds closest_record_bounds(const PlaneDists& d,
                                                              const float4* __restrict__ prim32,
                                                              int32_t qq, float px, float py,
                                                              float pz, float cmargin) {
  const float4 A = __ldg(&prim32[3 * (int64_t)qq]);
  const float4 B = __ldg(&prim32[3 * (int64_t)qq + 1]);
  const float4 C = __ldg(&prim32[3 * (int64_t)qq + 2]);
  RecordBounds r;
  {
    const float b1x = A.x + B.x, b1y = A.y + B.y, b1z = A.z + B.z;
    const float b2x = A.x + C.x, b2y = A.y + C.y, b2z = A.z + C.z;
    // the point's distance beyond the box of the three vertices, per axis
    auto out = [](float a, float b, float c, float q) {
      return fmaxf(fmaxf(fminf(fminf(a, b), c) - q, q - fmaxf(fmaxf(a, b), c)), 0.0f);
    };
    const float ex = out(A.x, b1x, b2x, px);
    const float ey = out(A.y, b1y, b2y, py);
    const float ez = out(A.z, b1z, b2z, pz);
    r.lo = __fsqrt_rn(ex * ex + ey * ey + ez * ez) * (1.0f - 8.0f * kU32) - cmargin;
  }
  r.hi = INFINITY;
  // (a triangle without plane certificates has a NaN face distance)
  if (!(C.w > 0.0f) || !(d.h >= 0.0f) || !(fminf(d.s0, d.s1) <= -cmargin) || !(cmargin > 0.0f))
    return r;
  const float wx = px - A.x, wy = py - A.y, wz = pz - A.z;
  const float d11 = B.x * B.x + B.y * B.y + B.z * B.z;
  const float d12 = B.x * C.x + B.y * C.y + B.z * C.z;
  const float d22 = C.x * C.x + C.y * C.y + C.z * C.z;
  const float w1 = wx * B.x + wy * B.y + wz * B.z;
  const float w2 = wx * C.x + wy * C.y + wz * C.z;
  const float den = d11 * d22 - d12 * d12;
  // fmaxf of a NaN and 0 is 0
  float s = fmaxf((d22 * w1 - d12 * w2) / den, 0.0f);
  float t = fmaxf((d11 * w2 - d12 * w1) / den, 0.0f);
  // s + t rounded up: at most 1 means the exact sum is too
  if (!(__fadd_ru(s, t) <= 1.0f)) {
    s = fminf(s / (s + t), 1.0f);  // (inf / inf is NaN, and fminf gives 1)
    t = __fsub_rd(1.0f, s);
  }
  const float qx = __fmaf_rn(t, C.x, __fmaf_rn(s, B.x, A.x));
  const float qy = __fmaf_rn(t, C.y, __fmaf_rn(s, B.y, A.y));
  const float qz = __fmaf_rn(t, C.z, __fmaf_rn(s, B.z, A.z));
  const float dx = px - qx, dy = py - qy, dz = pz - qz;
  const float d32 = __fsqrt_rn(dx * dx + dy * dy + dz * dz);
  r.hi = __fmaf_ru(d32, 1.0f + 8.0f * kU32, cmargin);
  return r;
}

// Whether (d, face) replaces (best, best_face): triangle_intersect.cpp:126-133
// keeps a strictly nearer facet (strict <), and of facets at the same
// distance the lowest face id wins.  (best, best_face) starts at (INFTY, -1),
// so for face ids >= 0 the result is the lexicographic minimum, whatever the
// order the candidates come in.
__device__ __forceinline__ bool closest_better(double d, int32_t face, double best,
                                               int32_t best_face) {
  return d < best || (d == best && best_face >= 0 && face < best_face);
}

// One lane per point, the warp in step: each round, every lane without a
// leaf in hand takes up to a.node_steps inner-node steps, then the lanes
// holding a leaf bound its triangles in FP32 together, then the exact FP64
// tests of all the warp's lanes run together, one triangle per lane at a
// time.  A thread-per-point loop let the lanes of a warp drift apart (4.4 of
// 32 lanes per instruction); the phases keep the node tests, the bounds and
// the FP64 closest-point arithmetic each issued once for the warp.  Measured
// on the nested spheres (1e6 points, identical results): mixed 20.7 -> 25.8
// Mpoints/s with 8 node steps per round; the all-FP64 path, whose every
// triangle takes the exact test, is best with 1 (4.35 -> 4.5).  Entries
// popped beyond the best distance are skipped (node visits 74.7 -> 60.5
// per point).  In the mixed path a triangle's exact test waits, once a
// certified upper bound of the nearest exact distance is known, until the
// traversal ends, and runs only if its lower bound is still within the
// best: most triangles that would have improved the best for a while are
// never tested.  A lane keeps its point to the end, so a warp takes as long
// as its slowest point: large batches run in the [tree | Morton code] order
// a.order gives (point_index), whose neighbouring points take similar work.
template <bool MIXED>
__global__ void __launch_bounds__(kBlock) k_closest(PointArgs a) {
  const int64_t i = point_index(a);
  Counters cnt = {0, 0, 0, 0};
  double best = INFTY;
  int32_t best_face = -1;
  int32_t st = RAY_OK;
  TreeDev T{};
  d3 p = mk3(0.0, 0.0, 0.0);
  float px = 0.0f, py = 0.0f, pz = 0.0f, pabs = 0.0f, cmargin = 0.0f;
  bool f32ok = false, cbound = false;
  int32_t ref = CHILD_EMPTY;
  bool run = false, deferred = false;
  int32_t steps = 0;  // node records and triangles of this point (a.step_budget)
  if (i < a.n) {
    const int32_t tid = a.ray_trees ? a.ray_trees[i] : a.tree;
    p = load3(a.pts, i);
    if (tid < 1 || tid > a.n_trees || !finite3(p)) {
      st = RAY_INVALID;
    } else {
      T = a.trees[tid - 1];
      px = __double2float_rn(p.x);
      py = __double2float_rn(p.y);
      pz = __double2float_rn(p.z);
      pabs = fmaxf(fabsf(px), fmaxf(fabsf(py), fabsf(pz)));
      // FP32 box and triangle bounds only for coordinates far from FP32
      // overflow (a box distance squared stays finite); beyond, the FP32
      // box test prunes nothing and every triangle gets the exact test
      f32ok = pabs + T.max_abs < 1e18f;
      cbound = MIXED && a.tri_cb && f32ok;
      cmargin = 48.0f * kU32 * (pabs + T.max_abs);
      ref = T.root;
      run = ref != CHILD_EMPTY;
    }
  }
  int32_t stack[kStackSize];
  // each entry's lower bound of the point's distance to its box (FP32,
  // rounded down), checked again when the entry is popped: the best
  // distance has usually shrunk since it was pushed
  float skey[kStackSize];
  int sp = 0;
  // With the FP32 bounds, the exact tests wait once an upper bound is known:
  // a triangle whose lower bound is within the bound below joins the lane's
  // candidates (cl: lower bound, cq: leaf-ordered index), and the
  // candidates are tested after the traversal, nearest lower bound first.
  // best_hi, the least certified FP32 upper bound of the candidates' exact
  // distances (closest_record_bounds), prunes like a best distance: anything
  // whose lower bound exceeds it is strictly farther than some facet's exact
  // distance, so it is neither the minimum nor tied with it.  Before any
  // upper bound, and when the list is full, a triangle takes its exact test
  // at once.
  float best_hi = INFINITY;
  float cl[kCand];
  int32_t cq[kCand];
  int nc = 0;
  // the pruning bound: the best exact distance rounded up, or best_hi
  auto bound = [&]() { return fminf(__double2float_ru(best), best_hi); };
  // the exact closest-point test of leaf-ordered triangle qq
  auto exact = [&](int32_t qq) {
    if (MIXED) cnt.esc++;
    d3 v0, v1, v2;
    load_tri64(T.prim64 + kPrim64Stride * (int64_t)qq, v0, v1, v2);
    const d3 r = closest64(v0, v1, v2, p);
    const double dd = dist64(r, p);
    const int32_t fid = __ldg(&a.tri_face[__ldg(&T.prim_ref[qq])]);
    if (closest_better(dd, fid, best, best_face)) {
      best = dd;
      best_face = fid;
    }
  };
  // the next entry; one that can no longer hold a closer facet (its lower
  // bound above the bound: every facet inside is strictly farther) becomes
  // CHILD_EMPTY and is skipped
  auto pop = [&]() {
    if (sp == 0) {
      run = false;
      return;
    }
    --sp;
    ref = skey[sp] > bound() ? CHILD_EMPTY : stack[sp];
  };

  while (__any_sync(kFullMask, run)) {
    // a point past its step budget stops here; k_closest_coop finishes it
    if (run && a.step_budget > 0 && steps >= a.step_budget) {
      run = false;
      deferred = true;
    }
    // ---- inner nodes: lanes without a leaf in hand descend ----
    for (int it = 0; it < a.node_steps; ++it) {
      const bool want = run && (ref == CHILD_EMPTY || !ref_is_leaf(ref));
      if (!__any_sync(kFullMask, want)) break;
      if (!want) continue;
      if (ref == CHILD_EMPTY) {
        pop();
        continue;
      }
      // the node's records (one for 4-wide, two for 8-wide trees): the
      // hits of each are pushed nearest last, so the nearest is popped first
      const int nrec = T.width / kWidth;
      bool overflow = false;
      for (int rec = 0; rec < nrec; ++rec) {
        cnt.node++;
        cnt.box += 4;
        ++steps;
        int32_t cr[4];
        float ck[4];
        const int nhit = closest_children<MIXED>(T, ref, rec, p, px, py, pz, pabs, f32ok,
                                                 fmin(best, (double)best_hi), cr, ck);
        if (sp + nhit > kStackSize) {
          overflow = true;
          break;
        }
        for (int k = nhit - 1; k >= 0; --k) {
          stack[sp] = cr[k];
          skey[sp++] = ck[k];
        }
      }
      if (overflow) {
        st = RAY_STACK_OVERFLOW;
        run = false;
      } else {
        pop();
      }
    }

    // ---- leaves: FP32 bounds of each lane's triangles ----
    const bool leaf = run && ref != CHILD_EMPTY && ref_is_leaf(ref);
    int32_t first = 0;
    unsigned need = 0u;  // triangles of the leaf that take the exact test
    if (leaf) {
      first = leaf_first(ref);
      const int32_t count = leaf_count(ref);
      for (int32_t q = 0; q < count; ++q) {
        cnt.prim++;
        ++steps;
        if (cbound) {
          const int32_t qq = first + q;
          const PlaneDists pd = closest_planes32(a.tri_cb, __ldg(&T.prim_ref[qq]), px, py, pz);
          if (closest_lower_of(pd, cmargin) > bound()) continue;
          const RecordBounds rb = closest_record_bounds(pd, T.prim32, qq, px, py, pz, cmargin);
          const float lo = fmaxf(closest_lower_of(pd, cmargin), rb.lo);
          if (lo > bound()) continue;
          best_hi = fminf(best_hi, rb.hi);
          // without an upper bound yet the test runs at once: its distance
          // is the only bound the traversal would have
          if (best_hi < INFINITY) {
            if (nc == kCand) {  // drop the candidates the bound now excludes
              const float b = bound();
              int w = 0;
              for (int k = 0; k < kCand; ++k) {
                if (!(cl[k] > b)) {
                  cl[w] = cl[k];
                  cq[w] = cq[k];
                  ++w;
                }
              }
              nc = w;
            }
            if (nc < kCand) {
              cl[nc] = lo;
              cq[nc] = qq;
              ++nc;
              continue;
            }
          }
        }
        need |= 1u << q;
      }
    }
    // ---- the exact tests, every lane's next pending triangle at once ----
    while (__any_sync(kFullMask, need != 0u)) {
      if (need != 0u) {
        const int q = __ffs(need) - 1;
        need &= need - 1u;
        exact(first + q);
      }
    }
    if (leaf) pop();
  }
  // ---- the candidates' exact tests, nearest lower bound first, every
  // lane's next candidate at once; the rest of a lane's list is dropped at
  // the first lower bound above the bound ----
  if (MIXED && __any_sync(kFullMask, nc > 0)) {
    for (int k = 1; k < nc; ++k) {  // insertion sort by lower bound
      const float key = cl[k];
      const int32_t v = cq[k];
      int j = k - 1;
      while (j >= 0 && cl[j] > key) {
        cl[j + 1] = cl[j];
        cq[j + 1] = cq[j];
        --j;
      }
      cl[j + 1] = key;
      cq[j + 1] = v;
    }
    int nx = 0;
    while (__any_sync(kFullMask, nx < nc)) {
      if (nx < nc) {
        if (cl[nx] > bound()) {
          nx = nc;
        } else {
          exact(cq[nx]);
          ++nx;
        }
      }
    }
  }
  if (i < a.n) {
    if (a.deferred) a.deferred[i] = deferred ? 1 : 0;
    if (deferred) {
      a.def_best[i] = best;
      a.def_face[i] = best_face;
    } else {
      a.dist_out[i] = best_face >= 0 ? best : INFTY;
      if (a.id_out) a.id_out[i] = best_face;
      if (a.status) a.status[i] = st;
    }
  }
  if (a.counters) flush_counters(a.counters, cnt, i < a.n ? 1ull : 0ull);
}

// A point whose search passed k_closest's step budget (a.deferred[i] = 1),
// searched by a whole warp.  Each round the lanes take the top 32 entries of
// a shared stack of subtrees, push the children that may hold a facet no
// farther than the warp's best (closest_children), or bound and test their
// leaf's triangles (closest_may_win, then the exact FP64 closest point); the
// lanes' bests are then merged by closest_better.  The search starts from
// the best k_closest had found (a real candidate: nothing nearer is lost),
// and every facet that may be no farther than the final best takes the exact
// test, so the result is k_closest's: the strictly nearest facet, of equally
// near ones the lowest face id.  A point at the centre of a sphere is nearly
// equidistant from all its triangles and bounds most of them: one lane took
// about 20 ms on such a point of the nested spheres, the warp shares it.
constexpr int kCoopStack = 4096;

template <bool MIXED>
__global__ void __launch_bounds__(32) k_closest_coop(PointArgs a) {
  __shared__ int32_t sref[kCoopStack];
  __shared__ float skey[kCoopStack];
  const int lane = threadIdx.x;
  Counters cnt = {0, 0, 0, 0};
  for (int64_t base = (int64_t)blockIdx.x * 32; base < a.n; base += (int64_t)gridDim.x * 32) {
    const int64_t j = base + lane;
    unsigned todo = __ballot_sync(kFullMask, j < a.n && a.deferred[j] != 0);
    while (todo) {
      const int64_t i = base + __ffs(todo) - 1;
      todo &= todo - 1u;
      // (k_closest checked the tree id and the point)
      const int32_t tid = a.ray_trees ? a.ray_trees[i] : a.tree;
      const TreeDev T = a.trees[tid - 1];
      const d3 p = load3(a.pts, i);
      const float px = __double2float_rn(p.x), py = __double2float_rn(p.y),
                  pz = __double2float_rn(p.z);
      const float pabs = fmaxf(fabsf(px), fmaxf(fabsf(py), fabsf(pz)));
      const bool f32ok = pabs + T.max_abs < 1e18f;
      const bool cbound = MIXED && a.tri_cb && f32ok;
      const float cmargin = 48.0f * kU32 * (pabs + T.max_abs);
      double best = a.def_best[i];
      int32_t best_face = a.def_face[i];
      int32_t st = RAY_OK;
      int top = 0;
      if (T.root != CHILD_EMPTY) {
        if (lane == 0) {
          sref[0] = T.root;
          skey[0] = 0.0f;
        }
        top = 1;
      }
      __syncwarp();
      while (top > 0) {
        // the top entries, one per lane; an entry whose bound is above the
        // best (rounded up) holds no facet that could win
        const int take = min(top, 32);
        int32_t ref = CHILD_EMPTY;
        if (lane < take && !(skey[top - 1 - lane] > __double2float_ru(best)))
          ref = sref[top - 1 - lane];
        top -= take;
        __syncwarp();  // every entry read before the pushes below reuse the slots
        int32_t cr[8];
        float ck[8];
        int nc = 0;
        double lbest = best;
        int32_t lface = best_face;
        if (ref != CHILD_EMPTY && !ref_is_leaf(ref)) {
          const int nrec = T.width / kWidth;
          for (int rec = 0; rec < nrec; ++rec) {
            cnt.node++;
            cnt.box += 4;
            int32_t c4[4];
            float k4[4];
            const int nh = closest_children<MIXED>(T, ref, rec, p, px, py, pz, pabs, f32ok, best,
                                                   c4, k4);
#pragma unroll
            for (int k = 0; k < 4; ++k) {
              if (k < nh) {
                cr[rec * 4 + k] = c4[k];
                ck[rec * 4 + k] = k4[k];
              } else {
                cr[rec * 4 + k] = CHILD_EMPTY;
              }
            }
            nc = rec * 4 + 4;
          }
        } else if (ref != CHILD_EMPTY) {
          const int32_t first = leaf_first(ref), count = leaf_count(ref);
          const float bestf = __double2float_ru(best);
          for (int32_t q = 0; q < count; ++q) {
            cnt.prim++;
            const int32_t qq = first + q;
            if (cbound) {
              if (!closest_may_win(a.tri_cb, __ldg(&T.prim_ref[qq]), px, py, pz, cmargin, bestf))
                continue;
              cnt.esc++;
            }
            d3 v0, v1, v2;
            load_tri64(T.prim64 + kPrim64Stride * (int64_t)qq, v0, v1, v2);
            const double dd = dist64(closest64(v0, v1, v2, p), p);
            const int32_t fid = __ldg(&a.tri_face[__ldg(&T.prim_ref[qq])]);
            if (closest_better(dd, fid, lbest, lface)) {
              lbest = dd;
              lface = fid;
            }
          }
        }
        // the children to push (slots of cr holding CHILD_EMPTY are gaps)
        int mine = 0;
#pragma unroll
        for (int k = 0; k < 8; ++k) mine += (k < nc && cr[k] != CHILD_EMPTY) ? 1 : 0;
        int incl = mine;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
          const int y = __shfl_up_sync(kFullMask, incl, off);
          if (lane >= off) incl += y;
        }
        const int total = __shfl_sync(kFullMask, incl, 31);
        if (top + total > kCoopStack) {
          st = RAY_STACK_OVERFLOW;  // (warp-uniform)
        } else {
          // each record's children nearest last, so the nearest is taken first
          int pos = top + incl - mine;
#pragma unroll
          for (int k = 7; k >= 0; --k) {
            if (k < nc && cr[k] != CHILD_EMPTY) {
              sref[pos] = cr[k];
              skey[pos] = ck[k];
              ++pos;
            }
          }
          top += total;
        }
        __syncwarp();
        // the warp's best: the lanes' candidates merged, then lane 0's taken
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
          const double od = __shfl_xor_sync(kFullMask, lbest, off);
          const int32_t of = __shfl_xor_sync(kFullMask, lface, off);
          if (closest_better(od, of, lbest, lface)) {
            lbest = od;
            lface = of;
          }
        }
        best = __shfl_sync(kFullMask, lbest, 0);
        best_face = __shfl_sync(kFullMask, lface, 0);
        if (st != RAY_OK) break;
      }
      if (lane == 0) {
        a.dist_out[i] = best_face >= 0 ? best : INFTY;
        if (a.id_out) a.id_out[i] = best_face;
        if (a.status) a.status[i] = st;
      }
      __syncwarp();
    }
  }
  if (a.counters) flush_counters(a.counters, cnt, 0ull);
}

// ---------------------------------------------------------------------------
// find_element (embree/ray_tracer.cpp:226-257 + tetrahedron_contain.cpp:94-114)
// ---------------------------------------------------------------------------

// One thread per point, each on its own: the mixed path, whose FP32 filter
// decides nearly every tet of an interior point, runs faster this way (1409
// against 1249 Mpoints/s in warp-synchronous phases, 1e6 uniform points in
// the 750,000-tet cube).  For points on the cube's faces, where most tets
// take the exact test, the phases win: 445 against 198 Mpoints/s.
template <bool MIXED>
__global__ void __launch_bounds__(kBlock) k_find_element_lane(PointArgs a) {
  const int64_t i = point_index(a);
  Counters cnt = {0, 0, 0, 0};
  if (i < a.n) {
    const int32_t tid = a.ray_trees ? a.ray_trees[i] : a.tree;
    const d3 p = load3(a.pts, i);
    int32_t best_id = -1, best_idx = -1;
    int32_t st = RAY_OK;
    if (tid < 1 || tid > a.n_trees || !finite3(p)) {
      st = RAY_INVALID;
    } else {
      const TreeDev T = a.trees[tid - 1];
      // rounding a point to FP32 is monotone, so fl32(p) inside an outward
      // rounded box is implied by p inside the exact box: the test is
      // conservative
      const float px = __double2float_rn(p.x), py = __double2float_rn(p.y),
                  pz = __double2float_rn(p.z);
      const float pabs = fmaxf(fabsf(px), fmaxf(fabsf(py), fabsf(pz)));
      int32_t stack[kStackSize];
      int sp = 0;
      int32_t ref = T.root;
      bool run = ref != CHILD_EMPTY;
      while (run) {
        if (!ref_is_leaf(ref)) {
          const int nrec = T.width / kWidth;
          bool overflow = false;
          for (int rec = 0; rec < nrec; ++rec) {
          cnt.node++;
          cnt.box += 4;
          int32_t cr[4];
          int nhit = 0;
          if (MIXED) {
            const Node32* np = T.n32 + (int64_t)ref * nrec + rec;
            const float4 lx = __ldg(&np->lox), hx = __ldg(&np->hix), ly = __ldg(&np->loy),
                         hy = __ldg(&np->hiy), lz = __ldg(&np->loz), hz = __ldg(&np->hiz);
            const int4 c = __ldg(&np->child);
            const bool in[4] = {
                px >= lx.x && px <= hx.x && py >= ly.x && py <= hy.x && pz >= lz.x && pz <= hz.x,
                px >= lx.y && px <= hx.y && py >= ly.y && py <= hy.y && pz >= lz.y && pz <= hz.y,
                px >= lx.z && px <= hx.z && py >= ly.z && py <= hy.z && pz >= lz.z && pz <= hz.z,
                px >= lx.w && px <= hx.w && py >= ly.w && py <= hy.w && pz >= lz.w && pz <= hz.w};
            const int32_t ca[4] = {c.x, c.y, c.z, c.w};
            for (int k = 0; k < 4; ++k)
              if (in[k]) cr[nhit++] = ca[k];
          } else {
            const Node64* np = T.n64 + (int64_t)ref * nrec + rec;
            const int4 c = __ldg(&np->child);
            const int32_t ca[4] = {c.x, c.y, c.z, c.w};
            for (int k = 0; k < 4; ++k) {
              const bool in = p.x >= __ldg(np->lox + k) && p.x <= __ldg(np->hix + k) &&
                              p.y >= __ldg(np->loy + k) && p.y <= __ldg(np->hiy + k) &&
                              p.z >= __ldg(np->loz + k) && p.z <= __ldg(np->hiz + k);
              if (in) cr[nhit++] = ca[k];
            }
          }
          if (sp + nhit > kStackSize) {
            overflow = true;
            break;
          }
          for (int k = nhit - 1; k >= 0; --k) stack[sp++] = cr[k];
          }
          if (overflow) {
            st = RAY_STACK_OVERFLOW;
            break;
          }
        } else {
          const int32_t first = leaf_first(ref), count = leaf_count(ref);
          for (int32_t q = first; q < first + count; ++q) {
            cnt.prim++;
            if (MIXED) {
              const float4* f = T.prim32 + 4 * (int64_t)q;
              const int c = tet_filter32(px, py, pz, pabs, __ldg(f), __ldg(f + 1), __ldg(f + 2),
                                         __ldg(f + 3));
              if (c < 0) continue;
              if (c > 0) {
                const int32_t idx = __ldg(&T.prim_ref[q]);
                const int32_t id = __ldg(&a.elem_ids[idx]);
                if (best_idx < 0 || id < best_id) {
                  best_id = id;
                  best_idx = idx;
                }
                continue;
              }
              cnt.esc++;
            }
            const double* v = T.prim64 + 12 * (int64_t)q;
            const d3 v0 = mk3(__ldg(v + 0), __ldg(v + 1), __ldg(v + 2));
            const d3 v1 = mk3(__ldg(v + 3), __ldg(v + 4), __ldg(v + 5));
            const d3 v2 = mk3(__ldg(v + 6), __ldg(v + 7), __ldg(v + 8));
            const d3 v3 = mk3(__ldg(v + 9), __ldg(v + 10), __ldg(v + 11));
            if (!tet_contains64(p, v0, v1, v2, v3)) continue;
            const int32_t idx = __ldg(&T.prim_ref[q]);
            const int32_t id = __ldg(&a.elem_ids[idx]);
            if (best_idx < 0 || id < best_id) {  // tie rule: lowest element id
              best_id = id;
              best_idx = idx;
            }
          }
        }
        if (sp == 0) break;
        ref = stack[--sp];
      }
    }
    if (a.id_out) a.id_out[i] = best_id;
    if (a.index_out) a.index_out[i] = best_idx;
    if (a.status) a.status[i] = st;
  }
  if (a.counters) flush_counters(a.counters, cnt, i < a.n ? 1ull : 0ull);
}

// As closest: one lane per point, the warp in step -- up to a.node_steps
// inner-node steps for the lanes without a leaf in hand, then the leaves'
// tets (FP32 containment filter in the mixed path), then the exact FP64
// containment tests of all the warp's lanes together.  Every containing tet
// is visited (the lowest element id wins), so no entry is pruned.  The
// all-FP64 path, where every tet of a leaf takes the exact test, runs this
// way: 76.5 -> 114 Mpoints/s with 16 node steps (1e6 points, 750,000 tets);
// so does the mixed path for points on tet faces (launch_find_element).
template <bool MIXED>
__global__ void __launch_bounds__(kBlock) k_find_element(PointArgs a) {
  const int64_t i = point_index(a);
  Counters cnt = {0, 0, 0, 0};
  int32_t best_id = -1, best_idx = -1;
  int32_t st = RAY_OK;
  TreeDev T{};
  d3 p = mk3(0.0, 0.0, 0.0);
  float px = 0.0f, py = 0.0f, pz = 0.0f, pabs = 0.0f;
  int32_t ref = CHILD_EMPTY;
  bool run = false;
  if (i < a.n) {
    const int32_t tid = a.ray_trees ? a.ray_trees[i] : a.tree;
    p = load3(a.pts, i);
    if (tid < 1 || tid > a.n_trees || !finite3(p)) {
      st = RAY_INVALID;
    } else {
      T = a.trees[tid - 1];
      // rounding a point to FP32 is monotone, so fl32(p) inside an outward
      // rounded box is implied by p inside the exact box: the test is
      // conservative
      px = __double2float_rn(p.x);
      py = __double2float_rn(p.y);
      pz = __double2float_rn(p.z);
      pabs = fmaxf(fabsf(px), fmaxf(fabsf(py), fabsf(pz)));
      ref = T.root;
      run = ref != CHILD_EMPTY;
    }
  }
  int32_t stack[kStackSize];
  int sp = 0;
  auto pop = [&]() {
    if (sp == 0) {
      run = false;
      return;
    }
    ref = stack[--sp];
  };
  auto take = [&](int32_t idx) {
    const int32_t id = __ldg(&a.elem_ids[idx]);
    if (best_idx < 0 || id < best_id) {  // tie rule: lowest element id
      best_id = id;
      best_idx = idx;
    }
  };

  while (__any_sync(kFullMask, run)) {
    // ---- inner nodes ----
    for (int it = 0; it < a.node_steps; ++it) {
      const bool want = run && !ref_is_leaf(ref);
      if (!__any_sync(kFullMask, want)) break;
      if (!want) continue;
      const int nrec = T.width / kWidth;
      bool overflow = false;
      for (int rec = 0; rec < nrec; ++rec) {
        cnt.node++;
        cnt.box += 4;
        int32_t cr[4];
        int nhit = 0;
        if (MIXED) {
          const Node32* np = T.n32 + (int64_t)ref * nrec + rec;
          const float4 lx = __ldg(&np->lox), hx = __ldg(&np->hix), ly = __ldg(&np->loy),
                       hy = __ldg(&np->hiy), lz = __ldg(&np->loz), hz = __ldg(&np->hiz);
          const int4 c = __ldg(&np->child);
          const bool in[4] = {
              px >= lx.x && px <= hx.x && py >= ly.x && py <= hy.x && pz >= lz.x && pz <= hz.x,
              px >= lx.y && px <= hx.y && py >= ly.y && py <= hy.y && pz >= lz.y && pz <= hz.y,
              px >= lx.z && px <= hx.z && py >= ly.z && py <= hy.z && pz >= lz.z && pz <= hz.z,
              px >= lx.w && px <= hx.w && py >= ly.w && py <= hy.w && pz >= lz.w && pz <= hz.w};
          const int32_t ca[4] = {c.x, c.y, c.z, c.w};
          for (int k = 0; k < 4; ++k)
            if (in[k]) cr[nhit++] = ca[k];
        } else {
          const Node64* np = T.n64 + (int64_t)ref * nrec + rec;
          const int4 c = __ldg(&np->child);
          const int32_t ca[4] = {c.x, c.y, c.z, c.w};
          for (int k = 0; k < 4; ++k) {
            const bool in = p.x >= __ldg(np->lox + k) && p.x <= __ldg(np->hix + k) &&
                            p.y >= __ldg(np->loy + k) && p.y <= __ldg(np->hiy + k) &&
                            p.z >= __ldg(np->loz + k) && p.z <= __ldg(np->hiz + k);
            if (in) cr[nhit++] = ca[k];
          }
        }
        if (sp + nhit > kStackSize) {
          overflow = true;
          break;
        }
        for (int k = nhit - 1; k >= 0; --k) stack[sp++] = cr[k];
      }
      if (overflow) {
        st = RAY_STACK_OVERFLOW;
        run = false;
      } else {
        pop();
      }
    }

    // ---- leaves: the FP32 filter decides what it can ----
    const bool leaf = run && ref_is_leaf(ref);
    int32_t first = 0;
    unsigned need = 0u;  // tets of the leaf that take the exact test
    if (leaf) {
      first = leaf_first(ref);
      const int32_t count = leaf_count(ref);
      for (int32_t q = 0; q < count; ++q) {
        cnt.prim++;
        if (MIXED) {
          const float4* f = T.prim32 + 4 * (int64_t)(first + q);
          const int c = tet_filter32(px, py, pz, pabs, __ldg(f), __ldg(f + 1), __ldg(f + 2),
                                     __ldg(f + 3));
          if (c < 0) continue;
          if (c > 0) {
            take(__ldg(&T.prim_ref[first + q]));
            continue;
          }
          cnt.esc++;
        }
        need |= 1u << q;
      }
    }
    // ---- the exact tests, every lane's next pending tet at once ----
    while (__any_sync(kFullMask, need != 0u)) {
      if (need != 0u) {
        const int q = __ffs(need) - 1;
        need &= need - 1u;
        const double* v = T.prim64 + 12 * (int64_t)(first + q);
        const d3 v0 = mk3(__ldg(v + 0), __ldg(v + 1), __ldg(v + 2));
        const d3 v1 = mk3(__ldg(v + 3), __ldg(v + 4), __ldg(v + 5));
        const d3 v2 = mk3(__ldg(v + 6), __ldg(v + 7), __ldg(v + 8));
        const d3 v3 = mk3(__ldg(v + 9), __ldg(v + 10), __ldg(v + 11));
        if (tet_contains64(p, v0, v1, v2, v3)) take(__ldg(&T.prim_ref[first + q]));
      }
    }
    if (leaf) pop();
  }
  if (i < a.n) {
    if (a.id_out) a.id_out[i] = best_id;
    if (a.index_out) a.index_out[i] = best_idx;
    if (a.status) a.status[i] = st;
  }
  if (a.counters) flush_counters(a.counters, cnt, i < a.n ? 1ull : 0ull);
}

inline unsigned grid_for(int64_t n) { return (unsigned)((n + kBlock - 1) / kBlock); }

}  // namespace

cudaError_t launch_closest(bool mixed, const PointArgs& a, cudaStream_t st) {
  if (a.n <= 0) return cudaSuccess;
  PointArgs b = a;
  const bool coop = a.step_budget > 0 && a.deferred && a.def_best && a.def_face;
  if (!coop) b.step_budget = 0;
  if (mixed)
    k_closest<true><<<grid_for(a.n), kBlock, 0, st>>>(b);
  else
    k_closest<false><<<grid_for(a.n), kBlock, 0, st>>>(b);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || !coop) return e;
  // the deferred points, one warp each; blocks of one warp with a 32 KB
  // stack, at most 7 per SM, each scanning its share of the flags
  const int64_t need = (a.n + 31) / 32;
  const unsigned grid = (unsigned)std::max<int64_t>(
      1, std::min<int64_t>(need, (int64_t)device_sm_count() * 7));
  if (mixed)
    k_closest_coop<true><<<grid, 32, 0, st>>>(b);
  else
    k_closest_coop<false><<<grid, 32, 0, st>>>(b);
  return cudaGetLastError();
}

cudaError_t launch_find_element(bool mixed, const PointArgs& a, cudaStream_t st, bool phased) {
  if (a.n <= 0) return cudaSuccess;
  if (mixed && phased)
    k_find_element<true><<<grid_for(a.n), kBlock, 0, st>>>(a);
  else if (mixed)
    k_find_element_lane<true><<<grid_for(a.n), kBlock, 0, st>>>(a);
  else
    k_find_element<false><<<grid_for(a.n), kBlock, 0, st>>>(a);
  return cudaGetLastError();
}

}  // namespace xdgcu
