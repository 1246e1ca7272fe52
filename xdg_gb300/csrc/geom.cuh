// geom.cuh -- device geometry kernels of the XDG ray-query engine.
//
// Two families live here:
//
//  * FP64 routines that reproduce the reference's double-precision arithmetic
//    operation for operation (the translation unit is compiled with
//    -fmad=false, so no multiply-add is fused and every product and sum
//    rounds exactly as in the reference's C++):
//      plucker64      include/xdg/geometry/plucker.h:35-161
//      tet_contains64 src/tetrahedron_contain.cpp:11-43
//      closest64      src/geometry/closest.cpp:6-183
//      normalize64    include/xdg/vec3da.h:61-66
//
//  * an FP32 pre-filter for the Plucker test that returns a certified answer
//    ("this FP64 test would certainly reject") or "unknown", in which case the
//    caller escalates to plucker64.  The filter only ever skips candidates
//    that the FP64 test rejects, so results stay bit-identical.
#pragma once

#include <cfloat>
#include <cstdint>

namespace xdgcu {

// constants.h:15, 30 / dp_math.h:36
constexpr double INFTY = 1.7976931348623157e+308;
constexpr double ZERO_TOL = 20.0 * DBL_EPSILON;
// constants.h:90: float(FLT_MIN * 1e5); (double)FLT_MIN*1e5 rounded to float
constexpr float MIN_RCP_INPUT = 1.17549435e-33f;
constexpr double TINY_BIT = 1e-10;

struct d3 {
  double x, y, z;
};

__host__ __device__ __forceinline__ d3 mk3(double x, double y, double z) {
  d3 r;
  r.x = x;
  r.y = y;
  r.z = z;
  return r;
}
__host__ __device__ __forceinline__ d3 sub3(d3 a, d3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
__host__ __device__ __forceinline__ d3 add3(d3 a, d3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
__host__ __device__ __forceinline__ d3 scl3(double s, d3 a) { return mk3(s * a.x, s * a.y, s * a.z); }
__host__ __device__ __forceinline__ d3 neg3(d3 a) { return mk3(-a.x, -a.y, -a.z); }
// vec3da.h:80-83: (x*x' + y*y') + z*z'
__host__ __device__ __forceinline__ double dot3(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
// vec3da.h:85-90
__host__ __device__ __forceinline__ d3 cross3(d3 a, d3 b) {
  return mk3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__host__ __device__ __forceinline__ double comp3(d3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }

// vec3da.h:61-66 (Vec3da::normalize with the min_rcp_input clamp)
__host__ __device__ __forceinline__ d3 normalize64(d3 a) {
  double len = sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
  len = len < (double)MIN_RCP_INPUT ? (double)MIN_RCP_INPUT : len;
  a.x /= len;
  a.y /= len;
  a.z /= len;
  return a;
}

// mesh_manager_interface.cpp:216-220
__host__ __device__ __forceinline__ d3 face_normal64(d3 v0, d3 v1, d3 v2) {
  return normalize64(cross3(sub3(v1, v0), sub3(v2, v0)));
}


// ---------------------------------------------------------------------------
// Exact comparisons of doubles on the integer ALU.
//
// GB300 issues FP64 instructions (comparisons included) at 1/64 of the FP32
// rate.  For non-NaN doubles the map okey() below is strictly monotone and
// sends -0.0 and +0.0 to the same key, so every comparison of the reference's
// code can be evaluated on integer keys with identical outcome.  The engine
// rejects non-finite and huge (|x| >= 2^300) inputs at the C ABI, so no NaN
// can arise inside these routines.
// ---------------------------------------------------------------------------
__device__ __forceinline__ long long dbits(double x) { return __double_as_longlong(x); }
__device__ __forceinline__ long long okey(double x) {
  long long b = dbits(x);
  b = (b == (long long)0x8000000000000000ull) ? 0ll : b;
  return b >= 0 ? b : (b ^ 0x7fffffffffffffffll);
}
__device__ __forceinline__ bool gt0(double x) { return dbits(x) > 0; }
__device__ __forceinline__ bool lt0(double x) { return okey(x) < 0; }
__device__ __forceinline__ bool is0(double x) { return (dbits(x) << 1) == 0; }
__device__ __forceinline__ unsigned long long absbits(double x) {
  return (unsigned long long)dbits(x) & 0x7fffffffffffffffull;
}
__device__ __forceinline__ bool dlt(double a, double b) { return okey(a) < okey(b); }

// plucker.h:35-43
__device__ __forceinline__ bool first_lower(d3 a, d3 b) {
  const long long ax = okey(a.x), bx = okey(b.x);
  if (ax < bx) return true;
  if (ax > bx) return false;
  const long long ay = okey(a.y), by = okey(b.y);
  if (ay < by) return true;
  if (ay > by) return false;
  return okey(a.z) < okey(b.z);
}

// plucker.h:45-62.  The reference branches on the lexicographic order of the
// two vertices and evaluates the same formula with the operands swapped, then
// negates.  Here the operands are selected first and the sign is flipped on
// the integer bits, so the FP64 instructions are identical for every lane and
// a warp never runs both arms (the values are bit-identical to the branch).
__device__ __forceinline__ double plucker_edge64(d3 va, d3 vb, d3 ray, d3 rn) {
  const bool f = first_lower(va, vb);
  const d3 lo = f ? va : vb;
  const d3 hi = f ? vb : va;
  const d3 e = sub3(hi, lo);
  const d3 en = cross3(e, lo);
  double pip = dot3(ray, en) + dot3(rn, e);
  pip = __longlong_as_double(__double_as_longlong(pip) ^ (f ? 0ll : (long long)0x8000000000000000ull));
  // ZERO_TOL > fabs(pip)
  if (absbits(pip) < absbits(ZERO_TOL)) pip = 0.0;
  return pip;
}

// plucker.h:64-161.  `rn` is cross(direction, origin) (plucker.h:75), passed
// in so callers testing many triangles against one ray compute it once; the
// value is identical to recomputing it per call.  `orient` is +1 or -1 when
// use_or is set.
// index of the largest |d| component, first maximum wins (plucker.h:132-134)
__device__ __forceinline__ int plucker_axis(d3 d) {
  const unsigned long long ax = absbits(d.x), ay = absbits(d.y), az = absbits(d.z);
  int idx = 0;
  unsigned long long mx = 0ull;
  if (ax > mx) { idx = 0; mx = ax; }
  if (ay > mx) { idx = 1; mx = ay; }
  if (az > mx) { idx = 2; mx = az; }
  return idx;
}

// plucker.h:83-161 from the three edge coordinates c0 = (v0, v1), c1 =
// (v1, v2), c2 = (v2, v0) and component idx = plucker_axis(d) of the
// vertices, origin and direction.  Only that component of the intersection
// point is used; it is computed alone, with the reference's operations and
// order.
__device__ __forceinline__ bool plucker64_coords(double c0, double c1, double c2, double v0i,
                                                 double v1i, double v2i, double oi, double di,
                                                 double t_max, double t_min, bool use_or,
                                                 int orient, double* t_out) {
  // orientation * c > 0
  auto exits = [&](double c) { return orient > 0 ? gt0(c) : lt0(c); };
  const bool p0 = gt0(c0), n0 = lt0(c0), p1 = gt0(c1), n1 = lt0(c1), p2 = gt0(c2), n2 = lt0(c2);
  bool rej;
  if (use_or) {
    rej = exits(c0) || exits(c1) || exits(c2);
  } else {
    rej = (p0 && n1) || (n0 && p1) || (p1 && n2) || (n1 && p2) || (p0 && n2) || (n0 && p2);
  }
  if (rej || (is0(c0) && is0(c1) && is0(c2))) return false;
  const double inv = 1.0 / (c0 + c1 + c2);
  const double w0 = c0 * inv, w1 = c1 * inv, w2 = c2 * inv;
  const double hit_i = (w0 * v2i + w1 * v0i) + w2 * v1i;
  double dist = (hit_i - oi) / di;
  const double u = w2;
  const double v = w0;
  if (lt0(u) || lt0(v) || dlt(1.0, u + v)) dist = -1.0;
  if (dlt(dist, t_min) || dlt(t_max, dist)) return false;
  *t_out = dist;
  return true;
}

__device__ __forceinline__ bool plucker64(d3 v0, d3 v1, d3 v2, d3 o, d3 d, d3 rn, double t_max,
                                          double t_min, bool use_or, int orient, double* t_out) {
  // The three coordinates are evaluated unconditionally (the reference
  // returns after the first one that fails, :83-113); the decisions use the
  // same values, so the outcome is the same, and lanes of a warp do not
  // diverge in the FP64 part.
  const double c0 = plucker_edge64(v0, v1, d, rn);
  const double c1 = plucker_edge64(v1, v2, d, rn);
  const double c2 = plucker_edge64(v2, v0, d, rn);
  const int idx = plucker_axis(d);
  return plucker64_coords(c0, c1, c2, comp3(v0, idx), comp3(v1, idx), comp3(v2, idx),
                          comp3(o, idx), comp3(d, idx), t_max, t_min, use_or, orient, t_out);
}

// plucker.h:45-62 for an edge of a tet mesh whose edge vector e = hi - lo
// and edge normal en = e x lo (lo, hi: its vertices in first() order) were
// computed once when the mesh was set (6 doubles at E: e, then en).  The
// same operations on the same values give the same coordinate as
// plucker_edge64; `flip` is set when the test runs the edge from hi to lo.
__device__ __forceinline__ double plucker_edge_pre(const double* E, bool flip, d3 ray, d3 rn) {
  const double2 a = __ldg(reinterpret_cast<const double2*>(E));
  const double2 b = __ldg(reinterpret_cast<const double2*>(E + 2));
  const double2 c = __ldg(reinterpret_cast<const double2*>(E + 4));
  const d3 e = mk3(a.x, a.y, b.x), en = mk3(b.y, c.x, c.y);
  double pip = dot3(ray, en) + dot3(rn, e);
  pip = __longlong_as_double(__double_as_longlong(pip) ^ (flip ? (long long)0x8000000000000000ull : 0ll));
  if (absbits(pip) < absbits(ZERO_TOL)) pip = 0.0;
  return pip;
}

// plucker.h:45-62 for a triangle edge stored in test orientation: e and
// e x lo of the edge's first() order, both negated when the test runs the
// edge from hi to lo.  IEEE products and sums of negated operands are the
// negated results, so this is plucker_edge64's value (a zero may differ in
// sign before the snap to +0 below, not after).
__device__ __forceinline__ double plucker_edge_oriented(const double* E, d3 ray, d3 rn) {
  const double2 a = __ldg(reinterpret_cast<const double2*>(E));
  const double2 b = __ldg(reinterpret_cast<const double2*>(E + 2));
  const double2 c = __ldg(reinterpret_cast<const double2*>(E + 4));
  const d3 e = mk3(a.x, a.y, b.x), en = mk3(b.y, c.x, c.y);
  double pip = dot3(ray, en) + dot3(rn, e);
  if (absbits(pip) < absbits(ZERO_TOL)) pip = 0.0;
  return pip;
}

// Sign of dot(d, face_normal64(v0, v1, v2)) as the reference computes it
// (-1, 0, +1), without the square root and divisions of the normalisation
// when the rounding bound allows.  With c = (v1-v0) x (v2-v0) rounded as the
// reference rounds it, the reference's value is dot(d, c / len) evaluated
// with <= 4 roundings per term, so len * dot = sum d_i c_i (1 + th_i) with
// |th_i| <= gamma_4; the FP64 sum s = fl(sum d_i c_i) is within gamma_3
// sum |d_i c_i| of the exact sum.  If |s| > 8 eps sum |d_i c_i|, both have the
// sign of s and neither is zero; otherwise the exact normalised value decides.
__device__ __forceinline__ int normal_dot_sign_c(d3 d, d3 c) {
  const double p0 = d.x * c.x, p1 = d.y * c.y, p2 = d.z * c.z;
  const double s = p0 + p1 + p2;
  const double bound = (fabs(p0) + fabs(p1) + fabs(p2)) * (8.0 * DBL_EPSILON);
  // (the second test keeps the reference's value away from underflow)
  if (absbits(s) > absbits(bound) && absbits(s) > 0x0100000000000000ull) return gt0(s) ? 1 : -1;
  const double dp = dot3(d, normalize64(c));
  return gt0(dp) ? 1 : (lt0(dp) ? -1 : 0);
}

// the same from the vertices: c = (v1 - v0) x (v2 - v0) as the reference
// computes it (mesh_manager_interface.cpp:216-220)
__device__ __forceinline__ int normal_dot_sign(d3 d, d3 v0, d3 v1, d3 v2) {
  return normal_dot_sign_c(d, cross3(sub3(v1, v0), sub3(v2, v0)));
}

// tetrahedron_contain.cpp:11-43.  The reference solves T*lambda = p - v0 with
// T's columns e0 = v1-v0, e1 = v2-v0, e2 = v3-v0 through its linalg
// dependency: inverse = adjugate / determinant, then mul(inverse, rhs) summed
// over columns.  The same formula and order are used here.
__device__ __forceinline__ bool tet_contains64(d3 p, d3 v0, d3 v1, d3 v2, d3 v3) {
  const d3 X = sub3(v1, v0), Y = sub3(v2, v0), Z = sub3(v3, v0);
  const d3 ax = mk3(Y.y * Z.z - Z.y * Y.z, Z.y * X.z - X.y * Z.z, X.y * Y.z - Y.y * X.z);
  const d3 ay = mk3(Y.z * Z.x - Z.z * Y.x, Z.z * X.x - X.z * Z.x, X.z * Y.x - Y.z * X.x);
  const d3 az = mk3(Y.x * Z.y - Z.x * Y.y, Z.x * X.y - X.x * Z.y, X.x * Y.y - Y.x * X.y);
  const double det = X.x * (Y.y * Z.z - Z.y * Y.z) + X.y * (Y.z * Z.x - Z.z * Y.x) +
                     X.z * (Y.x * Z.y - Z.x * Y.y);
  const d3 ix = mk3(ax.x / det, ax.y / det, ax.z / det);
  const d3 iy = mk3(ay.x / det, ay.y / det, ay.z / det);
  const d3 iz = mk3(az.x / det, az.y / det, az.z / det);
  const d3 rhs = sub3(p, v0);
  const d3 l = add3(add3(scl3(rhs.x, ix), scl3(rhs.y, iy)), scl3(rhs.z, iz));
  const double l0 = 1.0 - (l.x + l.y + l.z);
  // bary < -PLUCKER_ZERO_TOL || bary > 1.0f + PLUCKER_ZERO_TOL, on integer keys
  const long long lo = okey(-ZERO_TOL), hi = okey(1.0 + ZERO_TOL);
  const long long k0 = okey(l0), k1 = okey(l.x), k2 = okey(l.y), k3 = okey(l.z);
  if (k0 < lo || k0 > hi) return false;
  if (k1 < lo || k1 > hi) return false;
  if (k2 < lo || k2 > hi) return false;
  if (k3 < lo || k3 > hi) return false;
  return true;
}

// closest.cpp:54-183 (Eberly's seven-region closest point, MOAB variant)
__host__ __device__ __forceinline__ d3 closest64(d3 v0, d3 v1, d3 v2, d3 p) {
  const d3 sv = sub3(v1, v0);
  const d3 tv = sub3(v2, v0);
  const d3 pv = sub3(v0, p);
  const double ss = dot3(sv, sv);
  const double st = dot3(sv, tv);
  const double tt = dot3(tv, tv);
  const double sp = dot3(sv, pv);
  const double tp = dot3(tv, pv);
  const double det = ss * tt - st * st;
  double s = st * tp - tt * sp;
  double t = st * sp - ss * tp;
  int region;  // closest.cpp:6-28
  if (s + t < det) {
    region = (s < 0) ? (t < 0 ? 4 : 3) : (t < 0 ? 5 : 0);
  } else {
    region = (s < 0) ? 2 : (t < 0 ? 6 : 1);
  }
  switch (region) {
    case 0: {
      const double inv_det = 1.0 / det;
      s *= inv_det;
      t *= inv_det;
      return add3(add3(v0, scl3(s, sv)), scl3(t, tv));
    }
    case 1: {
      const double num = tt + tp - st - sp;
      if (num <= 0) return v2;
      const double den = ss - 2 * st + tt;
      if (num >= den) return v1;
      const double q = num / den;
      return add3(scl3(q, v1), scl3(1 - q, v2));
    }
    case 2: {
      s = st + sp;
      t = tt + tp;
      if (t > s) {
        const double num = t - s;
        const double den = ss - 2 * st + tt;
        if (num > den) return v1;
        const double q = num / den;
        return add3(scl3(q, v1), scl3(1 - q, v2));
      } else if (t <= 0) {
        return v2;
      } else if (tp >= 0) {
        return v0;
      }
      return sub3(v0, scl3(tp / tt, tv));
    }
    case 3:
      if (tp >= 0) return v0;
      if (-tp >= tt) return v2;
      return sub3(v0, scl3(tp / tt, tv));
    case 4:
      if (sp < 0) {
        if (-sp > ss) return v1;
        return sub3(v0, scl3(sp / ss, sv));
      } else if (tp < 0) {
        if (-tp > tt) return v2;
        return sub3(v0, scl3(tp / tt, tv));
      }
      return v0;
    case 5:
      if (sp >= 0.0) return v0;
      if (-sp >= ss) return v1;
      return sub3(v0, scl3(sp / ss, sv));
    default: {
      t = st + tp;
      s = ss + sp;
      if (s > t) {
        const double num = t - s;
        const double den = tt - 2 * st + ss;
        if (num > den) return v2;
        t = num / den;
        s = 1 - t;
        return add3(scl3(s, v1), scl3(t, v2));
      } else if (s <= 0) {
        return v1;
      } else if (sp >= 0) {
        return v0;
      }
      return sub3(v0, scl3(sp / ss, sv));
    }
  }
}

// length of (a - p) as Vec3da::length (vec3da.h:58-59)
__host__ __device__ __forceinline__ double dist64(d3 a, d3 p) {
  const d3 w = sub3(a, p);
  return sqrt(w.x * w.x + w.y * w.y + w.z * w.z);
}

// ---------------------------------------------------------------------------
// FP32 pre-filter
// ---------------------------------------------------------------------------
//
// The exact Plucker coordinate of edge va->vb for the ray (o, d) is the triple
// product  pip = d . ((vb - va) x (va - o))  (expand plucker.h:45-62:
// d.(e x va) + (d x o).e = d.(e x va) - d.(e x o)).  The filter evaluates it
// in FP32 from
//    v0 = fl32(v0),  e1 = fl32(v1 - v0),  e2 = fl32(v2 - v0)   (stored per prim)
//    w0 = v0 - o32,  w1 = w0 + e1,  w2 = w0 + e2
//    pip01 = d.(e1 x w0), pip12 = d.((e2-e1) x w1), pip20 = d.((-e2) x w2)
// and bounds its distance to the exact value by standard rounding analysis
// (u = 2^-24; the stored vertex/edges are rounded to nearest (u|x|), the ray
// origin/direction are truncated (2u|x|), and each 6-term triple product is
// evaluated with at most 5 roundings per term, gamma_5 ~ 5u):
//    |pip32 - pip| <= u * D * E * (74 W0 + 77 E + 13 A)
// with D = |d|_inf, E = max edge |.|_inf, W0 = |w0|_inf, A = |v0|_inf + |o|_inf.
// The FP64 evaluation in plucker64 is within 2^-46 * D * E * (A + 2E) of the
// exact value, and values with |pip64| < 20*DBL_EPSILON are snapped to zero.
// Hence if |pip32| exceeds the sum of the three terms, pip64 is non-zero and
// has pip32's sign.  Inputs that overflow FP32 give inf/NaN, which never pass
// the comparison and therefore escalate.
// Double -> float conversions done with integer operations, so per-ray setup
// costs no FP64-pipe issue slots.  f32_trunc rounds toward zero (relative
// error < 2u = 2^-23), flushes magnitudes below FLT_MIN to zero (absolute
// error < 2^-126) and keeps inf/NaN (which then escalate or are rejected).
__device__ __forceinline__ float f32_trunc(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned hi = (unsigned)(b >> 32);
  const unsigned sign = hi & 0x80000000u;
  const int e = (int)((hi >> 20) & 0x7ffu);
  const unsigned m23 = (unsigned)((b >> 29) & 0x7fffffull);
  if (e == 0x7ff) return __uint_as_float(sign | 0x7f800000u | (m23 ? 0x400000u : 0u));
  const int fe = e - 1023 + 127;
  if (fe >= 255) return __uint_as_float(sign | 0x7f800000u);
  if (fe <= 0) return __uint_as_float(sign);
  return __uint_as_float(sign | ((unsigned)fe << 23) | m23);
}

// An FP32 value >= x for finite x >= 0 (the next float above the truncation),
// used for the culling distance; +inf for DBL_MAX or inf.
__device__ __forceinline__ float f32_up(double x) {
  const float t = f32_trunc(x);
  if (!(x > 0.0)) return t;
  const unsigned tb = __float_as_uint(t);
  return (tb >= 0x7f800000u) ? __uint_as_float(0x7f800000u) : __uint_as_float(tb + 1u);
}

__device__ __forceinline__ bool nan_bits(double x) {
  return ((unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull) > 0x7ff0000000000000ull;
}

// finite and |x| < 2^300, so no product of three inputs can overflow
__device__ __forceinline__ bool sane_bits(double x) {
  return ((unsigned)((unsigned long long)__double_as_longlong(x) >> 52) & 0x7ffu) < 1023u + 300u;
}

__device__ __forceinline__ bool finite_bits(double x) {
  return ((unsigned)((unsigned long long)__double_as_longlong(x) >> 52) & 0x7ffu) != 0x7ffu;
}

struct Ray32 {
  float ox, oy, oz;     // f32_trunc(o)
  float dx, dy, dz;     // f32_trunc(d)
  float du;             // u * |d|_inf * (1 + 2^-20)
  float oabs;           // |o32|_inf
};

__device__ __forceinline__ Ray32 make_ray32(d3 o, d3 d) {
  Ray32 r;
  r.ox = f32_trunc(o.x);
  r.oy = f32_trunc(o.y);
  r.oz = f32_trunc(o.z);
  r.dx = f32_trunc(d.x);
  r.dy = f32_trunc(d.y);
  r.dz = f32_trunc(d.z);
  const float dmax = fmaxf(fabsf(r.dx), fmaxf(fabsf(r.dy), fabsf(r.dz)));
  r.du = dmax * (5.9604645e-08f * 1.000001f);
  r.oabs = fmaxf(fabsf(r.ox), fmaxf(fabsf(r.oy), fabsf(r.oz)));
  return r;
}

// Returns a 3-bit sign code per coordinate: for coordinate k, bit pos[k] set
// means "certainly > 0" and bit neg[k] "certainly < 0".  v0/e1/e2 as above;
// emax = max |edge|_inf (stored per prim, rounded up); v0abs = |v0|_inf.
struct SignCert {
  unsigned pos, neg;
};

__device__ __forceinline__ float triple32(float dx, float dy, float dz, float ex, float ey,
                                          float ez, float wx, float wy, float wz) {
  const float cx = ey * wz - ez * wy;
  const float cy = ez * wx - ex * wz;
  const float cz = ex * wy - ey * wx;
  return dx * cx + dy * cy + dz * cz;
}

__device__ __forceinline__ SignCert plucker_filter32(const Ray32& r, float v0x, float v0y,
                                                     float v0z, float e1x, float e1y, float e1z,
                                                     float e2x, float e2y, float e2z, float emax,
                                                     float v0abs) {
  const float w0x = v0x - r.ox, w0y = v0y - r.oy, w0z = v0z - r.oz;
  const float w1x = w0x + e1x, w1y = w0y + e1y, w1z = w0z + e1z;
  const float w2x = w0x + e2x, w2y = w0y + e2y, w2z = w0z + e2z;
  const float p01 = triple32(r.dx, r.dy, r.dz, e1x, e1y, e1z, w0x, w0y, w0z);
  const float p12 = triple32(r.dx, r.dy, r.dz, e2x - e1x, e2y - e1y, e2z - e1z, w1x, w1y, w1z);
  const float p20 = triple32(r.dx, r.dy, r.dz, -e2x, -e2y, -e2z, w2x, w2y, w2z);
  const float w0a = fmaxf(fabsf(w0x), fmaxf(fabsf(w0y), fabsf(w0z)));
  const float A = v0abs + r.oabs;
  // u*D*E*(74 W0 + 77 E + 13 A) + 2^-46 D E (A + 2E) + 20 DBL_EPSILON, rounded up
  const float de = r.du * emax;
  const float thr = de * (74.0f * w0a + 77.0f * emax + 13.0f * A) * 1.0001f + 4.5e-15f;
  SignCert c;
  c.pos = (p01 > thr ? 1u : 0u) | (p12 > thr ? 2u : 0u) | (p20 > thr ? 4u : 0u);
  c.neg = (p01 < -thr ? 1u : 0u) | (p12 < -thr ? 2u : 0u) | (p20 < -thr ? 4u : 0u);
  return c;
}

// FP32 pre-filter of tet containment (tetrahedron_contain.cpp:11-43).
// Returns +1 when the FP64 test certainly accepts, -1 when it certainly
// rejects, 0 when only the FP64 test can tell.
//
// With the per-tet data of k_tet_gather (M = T^{-1} rounded to FP32, m >= the
// max row 1-norm of M, e64 >= the error of the reference's FP64 barycentric
// coordinates anywhere in the tet's box), the FP32 coordinates
//    l = M32 (p32 - v0_32),  l0 = 1 - (l1 + l2 + l3)
// are within E32 = u (16 m (R + |p| + |v0|) + 4 (1 + sum |l|)) of the exact
// barycentric coordinates (R = |p32 - v0_32|_inf; p, v0 and M rounded to
// nearest (u; the bound allows 2u for p), 3-term dot products gamma_3), and the FP64 coordinates are
// within e64 of them.  The reference accepts iff every coordinate lies in
// [-20 eps, 1 + 20 eps]; so l_k < -(E32 + e64 + 20 eps) for some k certifies a
// rejection, and E32 + e64 <= l_k <= 1 - (E32 + e64) for all k an acceptance.
__device__ __forceinline__ int tet_filter32(float px, float py, float pz, float pabs, float4 f0,
                                            float4 f1, float4 f2, float4 f3) {
  const float m = f0.w;
  if (!(m < INFINITY)) return 0;
  const float rx = px - f0.x, ry = py - f0.y, rz = pz - f0.z;
  const float R = fmaxf(fabsf(rx), fmaxf(fabsf(ry), fabsf(rz)));
  const float l1 = f1.x * rx + f1.y * ry + f1.z * rz;
  const float l2 = f2.x * rx + f2.y * ry + f2.z * rz;
  const float l3 = f3.x * rx + f3.y * ry + f3.z * rz;
  const float l0 = 1.0f - (l1 + l2 + l3);
  const float sl = fabsf(l1) + fabsf(l2) + fabsf(l3);
  const float E = (5.9604645e-08f * (16.0f * m * (R + pabs + f1.w) + 4.0f * (1.0f + sl))) * 1.0001f +
                  f2.w + 4.5e-15f;
  const float lmin = fminf(fminf(l0, l1), fminf(l2, l3));
  const float lmax = fmaxf(fmaxf(l0, l1), fmaxf(l2, l3));
  if (lmin < -E || lmax > 1.0f + E) return -1;
  if (lmin >= E && lmax <= 1.0f - E) return 1;
  return 0;
}

// Non-oriented test (ray_fire, point_in_volume, occluded): the FP64 test
// rejects whenever two coordinates have strictly opposite signs
// (plucker.h:99-121), so a certified opposite pair is a certified miss.
__device__ __forceinline__ bool certified_miss(SignCert c) { return c.pos != 0u && c.neg != 0u; }

}  // namespace xdgcu
