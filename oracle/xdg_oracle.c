/*
 * xdg_oracle.c -- CPU restatement of the reference's double-precision ray-query
 * semantics (see xdg_oracle.h).
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA engine and the timed
 * CPU baseline of bench.py.  Nothing in the product path loads it.
 *
 * Compile with -ffp-contract=off: every expression below is written in the
 * reference's evaluation order (C evaluates a*b + c*d + e*f as
 * ((a*b + c*d) + e*f), exactly like Vec3da::dot in vec3da.h:80-83), and no
 * fused multiply-add may change the last bit.
 */
#include "xdg_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

/* constants.h:30 (PLUCKER_ZERO_TOL) == dp_math.h:36 (DBL_ZERO_TOL) */
static const double ZERO_TOL = 20.0 * DBL_EPSILON;
/* constants.h:90: float(FLT_MIN * 1e5), evaluated in double then narrowed */
static const float MIN_RCP_INPUT = (float)((double)FLT_MIN * 1E5);

typedef struct { double x, y, z; } v3;

static inline v3 mk(const double* p) { v3 r = {p[0], p[1], p[2]}; return r; }
static inline v3 sub(v3 a, v3 b) { v3 r = {a.x - b.x, a.y - b.y, a.z - b.z}; return r; }
static inline v3 add(v3 a, v3 b) { v3 r = {a.x + b.x, a.y + b.y, a.z + b.z}; return r; }
static inline v3 scl(double s, v3 a) { v3 r = {s * a.x, s * a.y, s * a.z}; return r; }
static inline v3 neg(v3 a) { v3 r = {-a.x, -a.y, -a.z}; return r; }
/* vec3da.h:80-83 */
static inline double dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
/* vec3da.h:85-90 */
static inline v3 cross(v3 a, v3 b) {
  v3 r = {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
  return r;
}
static inline double comp(v3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }
/* vec3da.h:58-59 */
static inline double length(v3 a) { return sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
/* vec3da.h:61-66 */
static inline v3 normalize(v3 a) {
  double len = length(a);
  len = len < MIN_RCP_INPUT ? MIN_RCP_INPUT : len;
  a.x /= len; a.y /= len; a.z /= len;
  return a;
}

/* ------------------------------------------------------------------------ */
/* Plucker ray-triangle test                                                */
/* ------------------------------------------------------------------------ */

/* plucker.h:35-43: lexicographic "a is lower than b" */
static inline int first_lower(v3 a, v3 b) {
  if (a.x < b.x) return 1;
  if (a.x > b.x) return 0;
  if (a.y < b.y) return 1;
  if (a.y > b.y) return 0;
  return a.z < b.z;
}

/* plucker.h:45-62 */
static inline double edge_test(v3 va, v3 vb, v3 ray, v3 rn) {
  double pip;
  if (first_lower(va, vb)) {
    v3 e = sub(vb, va);
    v3 en = cross(e, va);
    pip = dot(ray, en) + dot(rn, e);
  } else {
    v3 e = sub(va, vb);
    v3 en = cross(e, vb);
    pip = dot(ray, en) + dot(rn, e);
    pip = -pip;
  }
  if (ZERO_TOL > fabs(pip)) pip = 0.0;
  return pip;
}

/* plucker.h:64-161 */
static int plucker(v3 v0, v3 v1, v3 v2, v3 o, v3 d, double t_max, double t_min,
                   int use_or, int orient, double* t_out) {
  const v3 raya = d;
  const v3 rayb = cross(d, o);
  double c0 = edge_test(v0, v1, raya, rayb);
  if (use_or && orient * c0 > 0) return 0;
  double c1 = edge_test(v1, v2, raya, rayb);
  if (use_or) {
    if (orient * c1 > 0) return 0;
  } else if ((0.0 < c0 && 0.0 > c1) || (0.0 > c0 && 0.0 < c1)) {
    return 0;
  }
  double c2 = edge_test(v2, v0, raya, rayb);
  if (use_or) {
    if (orient * c2 > 0) return 0;
  } else if ((0.0 < c1 && 0.0 > c2) || (0.0 > c1 && 0.0 < c2) ||
             (0.0 < c0 && 0.0 > c2) || (0.0 > c0 && 0.0 < c2)) {
    return 0;
  }
  if (0.0 == c0 && 0.0 == c1 && 0.0 == c2) return 0;

  const double inv = 1.0 / (c0 + c1 + c2);
  /* (c0*inv)*v2 + (c1*inv)*v0 + (c2*inv)*v1, summed left to right */
  const v3 hit = add(add(scl(c0 * inv, v2), scl(c1 * inv, v0)), scl(c2 * inv, v1));

  int idx = 0;
  double max_abs = 0;
  for (int i = 0; i < 3; ++i) {
    if (fabs(comp(d, i)) > max_abs) { idx = i; max_abs = fabs(comp(d, i)); }
  }
  double dist = (comp(hit, idx) - comp(o, idx)) / comp(d, idx);

  double u = c2 * inv;
  double v = c0 * inv;
  if (u < 0.0 || v < 0.0 || (u + v) > 1.0) dist = -1.0;
  if (dist < t_min || dist > t_max) return 0;
  *t_out = dist;
  return 1;
}

double xo_plucker_edge_test(const double va[3], const double vb[3],
                            const double ray[3], const double ray_normal[3]) {
  return edge_test(mk(va), mk(vb), mk(ray), mk(ray_normal));
}

int xo_plucker_ray_tri(const double v[9], const double origin[3], const double dir[3],
                       double t_max, double t_min, int use_orientation, int orientation,
                       double* t_out) {
  double t = 0.0;
  int hit = plucker(mk(v), mk(v + 3), mk(v + 6), mk(origin), mk(dir), t_max, t_min,
                    use_orientation, orientation, &t);
  if (hit && t_out) *t_out = t;
  return hit;
}

/* ------------------------------------------------------------------------ */
/* Tet containment                                                          */
/* ------------------------------------------------------------------------ */

/* tetrahedron_contain.cpp:11-43.  The 3x3 solve uses the reference's linalg
 * dependency (sgorsten/linalg, submodule absent): T's *columns* are
 * e0 = v1-v0, e1 = v2-v0, e2 = v3-v0 (linalg matrices are column-major and
 * brace-initialised by column); inverse(T) = adjugate(T) / determinant(T);
 * mul(A, b) = A.x*b.x + A.y*b.y + A.z*b.z over columns.  The element-level
 * op order is linalg's published adjugate/determinant formula; last-ulp
 * agreement with the unpinned submodule version is not verified. */
int xo_tet_contains(const double p[3], const double vv[12]) {
  v3 v0 = mk(vv), v1 = mk(vv + 3), v2 = mk(vv + 6), v3_ = mk(vv + 9);
  v3 X = sub(v1, v0), Y = sub(v2, v0), Z = sub(v3_, v0); /* columns */
  /* adjugate, column by column */
  v3 ax = {Y.y * Z.z - Z.y * Y.z, Z.y * X.z - X.y * Z.z, X.y * Y.z - Y.y * X.z};
  v3 ay = {Y.z * Z.x - Z.z * Y.x, Z.z * X.x - X.z * Z.x, X.z * Y.x - Y.z * X.x};
  v3 az = {Y.x * Z.y - Z.x * Y.y, Z.x * X.y - X.x * Z.y, X.x * Y.y - Y.x * X.y};
  double det = X.x * (Y.y * Z.z - Z.y * Y.z) + X.y * (Y.z * Z.x - Z.z * Y.x) +
               X.z * (Y.x * Z.y - Z.x * Y.y);
  v3 ix = {ax.x / det, ax.y / det, ax.z / det};
  v3 iy = {ay.x / det, ay.y / det, ay.z / det};
  v3 iz = {az.x / det, az.y / det, az.z / det};
  v3 rhs = sub(mk(p), v0);
  v3 l = add(add(scl(rhs.x, ix), scl(rhs.y, iy)), scl(rhs.z, iz));
  double l0 = 1.0 - (l.x + l.y + l.z);
  double bary[4] = {l0, l.x, l.y, l.z};
  for (int i = 0; i < 4; ++i) {
    if (bary[i] < -ZERO_TOL || bary[i] > 1.0 + ZERO_TOL) return 0;
  }
  return 1;
}

/* ------------------------------------------------------------------------ */
/* Closest point on a triangle                                              */
/* ------------------------------------------------------------------------ */

/* closest.cpp:6-28 (Region::Zero..Six as 0..6) */
static int region_of(double s, double t, double det) {
  if (s + t < det) {
    if (s < 0) return t < 0 ? 4 : 3;
    if (t < 0) return 5;
    return 0;
  }
  if (s < 0) return 2;
  if (t < 0) return 6;
  return 1;
}

/* closest.cpp:54-183 */
static v3 closest_on_tri(v3 v0, v3 v1, v3 v2, v3 p) {
  const v3 sv = sub(v1, v0);
  const v3 tv = sub(v2, v0);
  const v3 pv = sub(v0, p);
  const double ss = dot(sv, sv);
  const double st = dot(sv, tv);
  const double tt = dot(tv, tv);
  const double sp = dot(sv, pv);
  const double tp = dot(tv, pv);
  const double det = ss * tt - st * st;
  double s = st * tp - tt * sp;
  double t = st * sp - ss * tp;
  switch (region_of(s, t, det)) {
    case 0: {
      const double inv_det = 1.0 / det;
      s *= inv_det;
      t *= inv_det;
      return add(add(v0, scl(s, sv)), scl(t, tv));
    }
    case 1: {
      const double num = tt + tp - st - sp;
      if (num <= 0) return v2;
      const double den = ss - 2 * st + tt;
      if (num >= den) return v1;
      const double q = num / den;
      return add(scl(q, v1), scl(1 - q, v2));
    }
    case 2: {
      s = st + sp;
      t = tt + tp;
      if (t > s) {
        const double num = t - s;
        const double den = ss - 2 * st + tt;
        if (num > den) return v1;
        const double q = num / den;
        return add(scl(q, v1), scl(1 - q, v2));
      } else if (t <= 0) {
        return v2;
      } else if (tp >= 0) {
        return v0;
      }
      return sub(v0, scl(tp / tt, tv));
    }
    case 3:
      if (tp >= 0) return v0;
      if (-tp >= tt) return v2;
      return sub(v0, scl(tp / tt, tv));
    case 4:
      if (sp < 0) {
        if (-sp > ss) return v1;
        return sub(v0, scl(sp / ss, sv));
      } else if (tp < 0) {
        if (-tp > tt) return v2;
        return sub(v0, scl(tp / tt, tv));
      }
      return v0;
    case 5:
      if (sp >= 0.0) return v0;
      if (-sp >= ss) return v1;
      return sub(v0, scl(sp / ss, sv));
    default: { /* 6 */
      t = st + tp;
      s = ss + sp;
      if (s > t) {
        const double num = t - s;
        const double den = tt - 2 * st + ss;
        if (num > den) return v2;
        t = num / den;
        s = 1 - t;
        return add(scl(s, v1), scl(t, v2));
      } else if (s <= 0) {
        return v1;
      } else if (sp >= 0) {
        return v0;
      }
      return sub(v0, scl(sp / ss, sv));
    }
  }
}

int xo_closest_region(const double v[9], const double pp[3]) {
  v3 v0 = mk(v), v1 = mk(v + 3), v2 = mk(v + 6), p = mk(pp);
  v3 sv = sub(v1, v0), tv = sub(v2, v0), pv = sub(v0, p);
  double ss = dot(sv, sv), st = dot(sv, tv), tt = dot(tv, tv);
  double sp = dot(sv, pv), tp = dot(tv, pv);
  double det = ss * tt - st * st;
  double s = st * tp - tt * sp;
  double t = st * sp - ss * tp;
  return region_of(s, t, det);
}

void xo_closest_on_tri(const double v[9], const double p[3], double out[3]) {
  v3 r = closest_on_tri(mk(v), mk(v + 3), mk(v + 6), mk(p));
  out[0] = r.x; out[1] = r.y; out[2] = r.z;
}

void xo_normalize(double v[3]) {
  v3 r = normalize(mk(v));
  v[0] = r.x; v[1] = r.y; v[2] = r.z;
}

/* mesh_manager_interface.cpp:216-220 */
static inline v3 face_normal(v3 v0, v3 v1, v3 v2) {
  return normalize(cross(sub(v1, v0), sub(v2, v0)));
}

void xo_face_normal(const double v[9], double n[3]) {
  v3 r = face_normal(mk(v), mk(v + 3), mk(v + 6));
  n[0] = r.x; n[1] = r.y; n[2] = r.z;
}

/* ------------------------------------------------------------------------ */
/* Trees: primitive storage + a binned-SAH BVH over bumped double boxes     */
/* ------------------------------------------------------------------------ */

typedef struct {
  double lo[3], hi[3];
  int64_t a;     /* leaf: first index into order[]; internal: left child */
  int32_t count; /* >0 leaf */
} node_t;

struct xo_tree {
  int kind; /* 0 triangles, 1 tets */
  int64_t n;
  int stride; /* 9 or 12 doubles */
  double* xyz;
  int32_t* ids;
  int32_t* surf;
  uint8_t* flip;
  double* box; /* 6 per prim */
  int use_bvh;
  node_t* nodes;
  int64_t n_nodes;
  int64_t* order;
};

static void prim_box(const double* v, int nv, double bump, double* box) {
  /* bbox.h:104-111 from_points, then +-bump (triangle_intersect.cpp:36-50) */
  double lo[3] = {XO_INFTY, XO_INFTY, XO_INFTY};
  double hi[3] = {-XO_INFTY, -XO_INFTY, -XO_INFTY};
  for (int k = 0; k < nv; ++k)
    for (int c = 0; c < 3; ++c) {
      double x = v[3 * k + c];
      lo[c] = x < lo[c] ? x : lo[c];
      hi[c] = x > hi[c] ? x : hi[c];
    }
  for (int c = 0; c < 3; ++c) {
    box[c] = lo[c] - bump;
    box[3 + c] = hi[c] + bump;
  }
}

/* bbox.h:85-102: dilation = max_chord_length * FP_BOX_TOL */
static double dilation_of(const double* v, int nv) {
  double lo[3] = {XO_INFTY, XO_INFTY, XO_INFTY};
  double hi[3] = {-XO_INFTY, -XO_INFTY, -XO_INFTY};
  for (int k = 0; k < nv; ++k)
    for (int c = 0; c < 3; ++c) {
      double x = v[3 * k + c];
      lo[c] = x < lo[c] ? x : lo[c];
      hi[c] = x > hi[c] ? x : hi[c];
    }
  v3 w = {hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]};
  return sqrt(dot(w, w)) * 1e-6;
}

typedef struct { int64_t node, first, count; } build_item;

static double half_area(const double* lo, const double* hi) {
  double dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
  return dx * dy + dy * dz + dz * dx;
}

static void build_bvh(xo_tree* t) {
  const int64_t n = t->n;
  t->order = (int64_t*)malloc(sizeof(int64_t) * (n > 0 ? n : 1));
  for (int64_t i = 0; i < n; ++i) t->order[i] = i;
  t->nodes = (node_t*)malloc(sizeof(node_t) * (n > 0 ? 2 * n : 1));
  t->n_nodes = 0;
  if (n == 0) return;
  double* cen = (double*)malloc(sizeof(double) * 3 * n);
  for (int64_t i = 0; i < n; ++i)
    for (int c = 0; c < 3; ++c) cen[3 * i + c] = 0.5 * (t->box[6 * i + c] + t->box[6 * i + 3 + c]);
  build_item* stack = (build_item*)malloc(sizeof(build_item) * 2 * n + 64);
  int64_t sp = 0;
  t->n_nodes = 1;
  stack[sp++] = (build_item){0, 0, n};
  enum { NB = 16 };
  while (sp > 0) {
    build_item it = stack[--sp];
    node_t* nd = &t->nodes[it.node];
    double lo[3] = {XO_INFTY, XO_INFTY, XO_INFTY}, hi[3] = {-XO_INFTY, -XO_INFTY, -XO_INFTY};
    double clo[3] = {XO_INFTY, XO_INFTY, XO_INFTY}, chi[3] = {-XO_INFTY, -XO_INFTY, -XO_INFTY};
    for (int64_t k = it.first; k < it.first + it.count; ++k) {
      int64_t p = t->order[k];
      for (int c = 0; c < 3; ++c) {
        if (t->box[6 * p + c] < lo[c]) lo[c] = t->box[6 * p + c];
        if (t->box[6 * p + 3 + c] > hi[c]) hi[c] = t->box[6 * p + 3 + c];
        if (cen[3 * p + c] < clo[c]) clo[c] = cen[3 * p + c];
        if (cen[3 * p + c] > chi[c]) chi[c] = cen[3 * p + c];
      }
    }
    memcpy(nd->lo, lo, sizeof lo);
    memcpy(nd->hi, hi, sizeof hi);
    if (it.count <= 4) {
      nd->a = it.first;
      nd->count = (int32_t)it.count;
      continue;
    }
    int axis = 0;
    double ext = chi[0] - clo[0];
    for (int c = 1; c < 3; ++c)
      if (chi[c] - clo[c] > ext) { ext = chi[c] - clo[c]; axis = c; }
    int64_t mid = -1;
    if (ext > 0) {
      int64_t cnt[NB] = {0};
      double blo[NB][3], bhi[NB][3];
      for (int b = 0; b < NB; ++b)
        for (int c = 0; c < 3; ++c) { blo[b][c] = XO_INFTY; bhi[b][c] = -XO_INFTY; }
      const double scale = NB / ext;
      for (int64_t k = it.first; k < it.first + it.count; ++k) {
        int64_t p = t->order[k];
        int b = (int)((cen[3 * p + axis] - clo[axis]) * scale);
        if (b >= NB) b = NB - 1;
        if (b < 0) b = 0;
        cnt[b]++;
        for (int c = 0; c < 3; ++c) {
          if (t->box[6 * p + c] < blo[b][c]) blo[b][c] = t->box[6 * p + c];
          if (t->box[6 * p + 3 + c] > bhi[b][c]) bhi[b][c] = t->box[6 * p + 3 + c];
        }
      }
      double best = XO_INFTY;
      int best_b = -1;
      for (int s = 1; s < NB; ++s) {
        double llo[3] = {XO_INFTY, XO_INFTY, XO_INFTY}, lhi[3] = {-XO_INFTY, -XO_INFTY, -XO_INFTY};
        double rlo[3] = {XO_INFTY, XO_INFTY, XO_INFTY}, rhi[3] = {-XO_INFTY, -XO_INFTY, -XO_INFTY};
        int64_t nl = 0, nr = 0;
        for (int b = 0; b < NB; ++b) {
          double* L = b < s ? llo : rlo;
          double* H = b < s ? lhi : rhi;
          if (b < s) nl += cnt[b]; else nr += cnt[b];
          for (int c = 0; c < 3; ++c) {
            if (blo[b][c] < L[c]) L[c] = blo[b][c];
            if (bhi[b][c] > H[c]) H[c] = bhi[b][c];
          }
        }
        if (nl == 0 || nr == 0) continue;
        double cost = half_area(llo, lhi) * nl + half_area(rlo, rhi) * nr;
        if (cost < best) { best = cost; best_b = s; }
      }
      if (best_b > 0) {
        /* partition by bin */
        int64_t i = it.first, j = it.first + it.count - 1;
        while (i <= j) {
          int64_t p = t->order[i];
          int b = (int)((cen[3 * p + axis] - clo[axis]) * scale);
          if (b >= NB) b = NB - 1;
          if (b < 0) b = 0;
          if (b < best_b) {
            ++i;
          } else {
            int64_t tmp = t->order[i];
            t->order[i] = t->order[j];
            t->order[j] = tmp;
            --j;
          }
        }
        mid = i;
      }
    }
    if (mid <= it.first || mid >= it.first + it.count) mid = it.first + it.count / 2;
    int64_t left = t->n_nodes;
    t->n_nodes += 2;
    nd = &t->nodes[it.node];
    nd->a = left;
    nd->count = 0;
    stack[sp++] = (build_item){left, it.first, mid - it.first};
    stack[sp++] = (build_item){left + 1, mid, it.first + it.count - mid};
  }
  free(stack);
  free(cen);
}

static xo_tree* tree_alloc(int kind, int64_t n, int stride, const double* xyz,
                           const int32_t* ids) {
  xo_tree* t = (xo_tree*)calloc(1, sizeof(xo_tree));
  t->kind = kind;
  t->n = n;
  t->stride = stride;
  size_t m = (size_t)(n > 0 ? n : 1);
  t->xyz = (double*)malloc(sizeof(double) * stride * m);
  t->ids = (int32_t*)malloc(sizeof(int32_t) * m);
  t->box = (double*)malloc(sizeof(double) * 6 * m);
  if (n > 0) {
    memcpy(t->xyz, xyz, sizeof(double) * stride * n);
    memcpy(t->ids, ids, sizeof(int32_t) * n);
  }
  return t;
}

xo_tree* xo_tree_create_tris(int64_t n, const double* tri_xyz, const int32_t* face_ids,
                             const int32_t* surf_ids, const uint8_t* flip, double bump,
                             int use_bvh) {
  xo_tree* t = tree_alloc(0, n, 9, tri_xyz, face_ids);
  size_t m = (size_t)(n > 0 ? n : 1);
  t->surf = (int32_t*)malloc(sizeof(int32_t) * m);
  t->flip = (uint8_t*)malloc(m);
  if (n > 0) {
    memcpy(t->surf, surf_ids, sizeof(int32_t) * n);
    if (flip) memcpy(t->flip, flip, n); else memset(t->flip, 0, n);
  }
  for (int64_t i = 0; i < n; ++i) prim_box(t->xyz + 9 * i, 3, bump, t->box + 6 * i);
  t->use_bvh = use_bvh;
  if (use_bvh) build_bvh(t);
  return t;
}

xo_tree* xo_tree_create_tets(int64_t n, const double* tet_xyz, const int32_t* elem_ids,
                             int use_bvh) {
  xo_tree* t = tree_alloc(1, n, 12, tet_xyz, elem_ids);
  for (int64_t i = 0; i < n; ++i) {
    double d = dilation_of(t->xyz + 12 * i, 4);
    prim_box(t->xyz + 12 * i, 4, d, t->box + 6 * i);
  }
  t->use_bvh = use_bvh;
  if (use_bvh) build_bvh(t);
  return t;
}

void xo_tree_destroy(xo_tree* t) {
  if (!t) return;
  free(t->xyz); free(t->ids); free(t->surf); free(t->flip); free(t->box);
  free(t->nodes); free(t->order);
  free(t);
}

/* ------------------------------------------------------------------------ */
/* Traversal helpers                                                        */
/* ------------------------------------------------------------------------ */

/* conservative double slab test of a ray segment [0, tmax] against a box */
static inline int ray_box(const double* lo, const double* hi, v3 o, v3 d, double tmax) {
  double tn = 0.0, tf = tmax;
  for (int c = 0; c < 3; ++c) {
    double oc = comp(o, c), dc = comp(d, c);
    if (dc == 0.0) {
      if (oc < lo[c] || oc > hi[c]) return 0;
      continue;
    }
    double t0 = (lo[c] - oc) / dc, t1 = (hi[c] - oc) / dc;
    if (t0 > t1) { double tmp = t0; t0 = t1; t1 = tmp; }
    t0 -= 1e-12 * fabs(t0);
    t1 += 1e-12 * fabs(t1);
    if (t0 > tn) tn = t0;
    if (t1 < tf) tf = t1;
    if (tn > tf) return 0;
  }
  return 1;
}

static inline int point_box(const double* lo, const double* hi, v3 p) {
  return p.x >= lo[0] && p.x <= hi[0] && p.y >= lo[1] && p.y <= hi[1] && p.z >= lo[2] &&
         p.z <= hi[2];
}

static inline double box_dist2(const double* lo, const double* hi, v3 p) {
  double s = 0;
  for (int c = 0; c < 3; ++c) {
    double x = comp(p, c), e = 0;
    if (x < lo[c]) e = lo[c] - x; else if (x > hi[c]) e = x - hi[c];
    s += e * e;
  }
  return s;
}

/* Generic iteration over the candidate primitives of one query.  The visitor
 * returns 1 to stop early.  `bound` reports the current pruning bound. */
typedef struct {
  int mode; /* 0 ray segment, 1 point-in-box, 2 point distance */
  v3 o, d;
  double tmax;   /* ray mode: current segment end */
  double dist2;  /* distance mode: current best squared (with slack) */
} query_t;

typedef int (*visit_fn)(const xo_tree* t, int64_t prim, query_t* q, void* state);

static void for_candidates(const xo_tree* t, query_t* q, visit_fn fn, void* state) {
  if (!t->use_bvh) {
    for (int64_t i = 0; i < t->n; ++i) {
      const double* b = t->box + 6 * i;
      int ok = q->mode == 0 ? ray_box(b, b + 3, q->o, q->d, q->tmax)
               : q->mode == 1 ? point_box(b, b + 3, q->o)
                              : box_dist2(b, b + 3, q->o) <= q->dist2;
      if (ok && fn(t, i, q, state)) return;
    }
    return;
  }
  if (t->n_nodes == 0) return;
  int64_t stack[256];
  int sp = 0;
  stack[sp++] = 0;
  while (sp > 0) {
    const node_t* nd = &t->nodes[stack[--sp]];
    int ok = q->mode == 0 ? ray_box(nd->lo, nd->hi, q->o, q->d, q->tmax)
             : q->mode == 1 ? point_box(nd->lo, nd->hi, q->o)
                            : box_dist2(nd->lo, nd->hi, q->o) <= q->dist2;
    if (!ok) continue;
    if (nd->count > 0) {
      for (int64_t k = nd->a; k < nd->a + nd->count; ++k)
        if (fn(t, t->order[k], q, state)) return;
    } else {
      if (sp + 2 > 256) abort(); /* depth beyond any tree this oracle builds */
      stack[sp++] = nd->a + 1;
      stack[sp++] = nd->a;
    }
  }
}

/* ------------------------------------------------------------------------ */
/* ray_fire / point_in_volume                                               */
/* ------------------------------------------------------------------------ */

typedef struct {
  int orientation; /* XO_ANY / EXITING / ENTERING */
  const int32_t* excl;
  int32_t n_excl;
  int has_hit;
  double t;
  int32_t face, surf;
  int dot_positive;
} rf_state;

/* triangle_intersect.cpp:12-24 */
static inline int orientation_cull(v3 d, v3 n, int orientation) {
  if (orientation == XO_ANY) return 0;
  double dp = dot(d, n);
  if (orientation == XO_EXITING && dp < 0.0) return 1;
  if (orientation == XO_ENTERING && dp >= 0.0) return 1;
  return 0;
}

/* triangle_intersect.cpp:52-109 for a RayFireType::VOLUME ray */
static int rf_visit(const xo_tree* t, int64_t p, query_t* q, void* vs) {
  rf_state* s = (rf_state*)vs;
  const double* v = t->xyz + 9 * p;
  v3 v0 = mk(v), v1 = mk(v + 3), v2 = mk(v + 6);
  double tt;
  if (!plucker(v0, v1, v2, q->o, q->d, q->tmax, 0.0, 0, 0, &tt)) return 0;
  if (tt > q->tmax) return 0;
  int32_t fid = t->ids[p];
  if (s->has_hit && tt == s->t && fid >= s->face) return 0; /* tie rule */
  v3 n = face_normal(v0, v1, v2);
  if (t->flip[p]) n = neg(n);
  if (orientation_cull(q->d, n, s->orientation)) return 0;
  for (int32_t k = 0; k < s->n_excl; ++k)
    if (s->excl[k] == fid) return 0; /* primitive_mask_cull, :26-34 */
  s->has_hit = 1;
  s->t = tt;
  s->face = fid;
  s->surf = t->surf[p];
  s->dot_positive = dot(q->d, n) > 0.0;
  q->tmax = tt;
  return 0;
}

void xo_ray_fire(const xo_tree* t, int64_t n, const double* org, const double* dir,
                 const double* dist_limit, int orientation, const int32_t* excl_off,
                 const int32_t* excl_ids, double* t_out, int32_t* surf_out,
                 int32_t* face_out, int n_threads) {
#pragma omp parallel for schedule(dynamic, 64) num_threads(n_threads > 0 ? n_threads : 1)
  for (int64_t i = 0; i < n; ++i) {
    query_t q;
    q.mode = 0;
    q.o = mk(org + 3 * i);
    q.d = mk(dir + 3 * i);
    q.tmax = dist_limit ? dist_limit[i] : XO_INFTY;
    rf_state s;
    memset(&s, 0, sizeof s);
    s.orientation = orientation;
    if (excl_off) {
      s.excl = excl_ids + excl_off[i];
      s.n_excl = excl_off[i + 1] - excl_off[i];
    }
    for_candidates(t, &q, rf_visit, &s);
    if (s.has_hit) {
      t_out[i] = s.t;
      surf_out[i] = s.surf;
      if (face_out) face_out[i] = s.face;
    } else {
      t_out[i] = XO_INFTY;
      surf_out[i] = XO_ID_NONE;
      if (face_out) face_out[i] = XO_ID_NONE;
    }
  }
}

void xo_point_in_volume(const xo_tree* t, int64_t n, const double* pts, const double* dir,
                        const int32_t* excl_off, const int32_t* excl_ids, int32_t* inside,
                        int n_threads) {
  /* embree/ray_tracer.cpp:268: {1. / std::sqrt(2.0), 1 / std::sqrt(2.0), 0.0} */
  const double dd[3] = {1. / sqrt(2.0), 1 / sqrt(2.0), 0.0};
#pragma omp parallel for schedule(dynamic, 64) num_threads(n_threads > 0 ? n_threads : 1)
  for (int64_t i = 0; i < n; ++i) {
    query_t q;
    q.mode = 0;
    q.o = mk(pts + 3 * i);
    q.d = dir ? mk(dir + 3 * i) : mk(dd);
    q.tmax = XO_INFTY;
    rf_state s;
    memset(&s, 0, sizeof s);
    s.orientation = XO_ANY;
    if (excl_off) {
      s.excl = excl_ids + excl_off[i];
      s.n_excl = excl_off[i + 1] - excl_off[i];
    }
    for_candidates(t, &q, rf_visit, &s);
    inside[i] = s.has_hit ? s.dot_positive : 0;
  }
}

/* ------------------------------------------------------------------------ */
/* occluded                                                                 */
/* ------------------------------------------------------------------------ */

static int occ_visit(const xo_tree* t, int64_t p, query_t* q, void* vs) {
  const double* v = t->xyz + 9 * p;
  double tt;
  if (plucker(mk(v), mk(v + 3), mk(v + 6), q->o, q->d, XO_INFTY, 0.0, 0, 0, &tt)) {
    *(int*)vs = 1;
    return 1;
  }
  return 0;
}

void xo_occluded(const xo_tree* t, int64_t n, const double* org, const double* dir,
                 int32_t* occ, double* dist, int n_threads) {
#pragma omp parallel for schedule(dynamic, 64) num_threads(n_threads > 0 ? n_threads : 1)
  for (int64_t i = 0; i < n; ++i) {
    query_t q;
    q.mode = 0;
    q.o = mk(org + 3 * i);
    q.d = mk(dir + 3 * i);
    q.tmax = XO_INFTY;
    int hit = 0;
    for_candidates(t, &q, occ_visit, &hit);
    occ[i] = hit;
    if (dist) dist[i] = hit ? -XO_INFTY : XO_INFTY;
  }
}

/* ------------------------------------------------------------------------ */
/* closest                                                                  */
/* ------------------------------------------------------------------------ */

typedef struct { double d; int32_t face; } cl_state;

static int cl_visit(const xo_tree* t, int64_t p, query_t* q, void* vs) {
  cl_state* s = (cl_state*)vs;
  const double* v = t->xyz + 9 * p;
  v3 r = closest_on_tri(mk(v), mk(v + 3), mk(v + 6), q->o);
  double d = length(sub(r, q->o));
  int32_t fid = t->ids[p];
  if (d < s->d || (d == s->d && s->face != XO_ID_NONE && fid < s->face)) {
    s->d = d;
    s->face = fid;
    q->dist2 = d * d * (1.0 + 1e-9) + 1e-300;
  }
  return 0;
}

void xo_closest(const xo_tree* t, int64_t n, const double* pts, double* dist_out,
                int32_t* face_out, int n_threads) {
#pragma omp parallel for schedule(dynamic, 64) num_threads(n_threads > 0 ? n_threads : 1)
  for (int64_t i = 0; i < n; ++i) {
    query_t q;
    q.mode = 2;
    q.o = mk(pts + 3 * i);
    q.d = q.o;
    q.dist2 = XO_INFTY;
    cl_state s = {XO_INFTY, XO_ID_NONE};
    for_candidates(t, &q, cl_visit, &s);
    dist_out[i] = s.d;
    face_out[i] = s.face;
  }
}

/* ------------------------------------------------------------------------ */
/* find_element                                                             */
/* ------------------------------------------------------------------------ */

typedef struct { int32_t id; int64_t idx; } fe_state;

static int fe_visit(const xo_tree* t, int64_t p, query_t* q, void* vs) {
  fe_state* s = (fe_state*)vs;
  double pp[3] = {q->o.x, q->o.y, q->o.z};
  if (!xo_tet_contains(pp, t->xyz + 12 * p)) return 0;
  int32_t id = t->ids[p];
  if (s->idx < 0 || id < s->id) { s->id = id; s->idx = p; }
  return 0;
}

void xo_find_element(const xo_tree* t, int64_t n, const double* pts, int32_t* elem_id,
                     int32_t* elem_idx, int n_threads) {
#pragma omp parallel for schedule(dynamic, 64) num_threads(n_threads > 0 ? n_threads : 1)
  for (int64_t i = 0; i < n; ++i) {
    query_t q;
    q.mode = 1;
    q.o = mk(pts + 3 * i);
    q.d = q.o;
    fe_state s = {XO_ID_NONE, -1};
    for_candidates(t, &q, fe_visit, &s);
    if (elem_id) elem_id[i] = s.idx < 0 ? XO_ID_NONE : s.id;
    if (elem_idx) elem_idx[i] = (int32_t)s.idx;
  }
}

/* ------------------------------------------------------------------------ */
/* Tet walk                                                                 */
/* ------------------------------------------------------------------------ */

struct xo_tetmesh {
  int64_t n_vert, n_tet;
  double* xyz;
  int32_t* conn;
  int32_t* adj;
  int32_t face_table[12];
};

xo_tetmesh* xo_tetmesh_create(int64_t n_vert, const double* xyz, int64_t n_tet,
                              const int32_t* conn, const int32_t* adj,
                              const int32_t face_table[12]) {
  xo_tetmesh* m = (xo_tetmesh*)calloc(1, sizeof(xo_tetmesh));
  m->n_vert = n_vert;
  m->n_tet = n_tet;
  m->xyz = (double*)malloc(sizeof(double) * 3 * (n_vert > 0 ? n_vert : 1));
  m->conn = (int32_t*)malloc(sizeof(int32_t) * 4 * (n_tet > 0 ? n_tet : 1));
  m->adj = (int32_t*)malloc(sizeof(int32_t) * 4 * (n_tet > 0 ? n_tet : 1));
  if (n_vert > 0) memcpy(m->xyz, xyz, sizeof(double) * 3 * n_vert);
  if (n_tet > 0) {
    memcpy(m->conn, conn, sizeof(int32_t) * 4 * n_tet);
    memcpy(m->adj, adj, sizeof(int32_t) * 4 * n_tet);
  }
  memcpy(m->face_table, face_table, sizeof(int32_t) * 12);
  return m;
}

void xo_tetmesh_destroy(xo_tetmesh* m) {
  if (!m) return;
  free(m->xyz); free(m->conn); free(m->adj);
  free(m);
}

static int next_element(const xo_tetmesh* m, int32_t elem, v3 r, v3 u, int32_t* next,
                        double* dist) {
  double dists[4] = {XO_INFTY, XO_INFTY, XO_INFTY, XO_INFTY};
  const int32_t* c = m->conn + 4 * (int64_t)elem;
  for (int i = 0; i < 4; ++i) {
    v3 fv[3];
    for (int j = 0; j < 3; ++j) fv[j] = mk(m->xyz + 3 * (int64_t)c[m->face_table[3 * i + j]]);
    double t;
    int hit = plucker(fv[0], fv[1], fv[2], r, u, XO_INFTY, 0.0, 1, 1, &t);
    /* std::max(0.0, t) == (0.0 < t) ? t : 0.0 */
    dists[i] = hit ? ((0.0 < t) ? t : 0.0) : XO_INFTY;
  }
  int idx = -1;
  double min_dist = XO_INFTY;
  for (int i = 0; i < 4; ++i) {
    if (dists[i] < min_dist) { min_dist = dists[i]; idx = i; }
  }
  *dist = min_dist;
  if (idx < 0) {
    *next = -1;
    return XO_NO_EXIT_FACE;
  }
  *next = m->adj[4 * (int64_t)elem + idx];
  return XO_OK;
}

int xo_next_element(const xo_tetmesh* m, int32_t elem, const double r[3], const double u[3],
                    int32_t* next_out, double* dist_out) {
  return next_element(m, elem, mk(r), mk(u), next_out, dist_out);
}

void xo_walk_elements(const xo_tetmesh* m, int64_t n, const int32_t* start_elem,
                      const double* start, const double* u, const double* distance,
                      int32_t max_segs, int32_t* seg_elem, double* seg_len,
                      int32_t* seg_count, int32_t* status, int n_threads) {
#pragma omp parallel for schedule(dynamic, 64) num_threads(n_threads > 0 ? n_threads : 1)
  for (int64_t i = 0; i < n; ++i) {
    v3 r = mk(start + 3 * i);
    v3 uu = mk(u + 3 * i);
    double dist = distance[i];
    int32_t elem = start_elem[i];
    int32_t k = 0;
    int st = XO_OK;
    int32_t* oe = seg_elem + (int64_t)i * max_segs;
    double* ol = seg_len + (int64_t)i * max_segs;
    while (dist > 0) {
      if (k >= max_segs) { st = XO_WALK_LIMIT; break; }
      int32_t nxt;
      double ex;
      int s = next_element(m, elem, r, uu, &nxt, &ex);
      if (s != XO_OK) st = s;
      /* std::min(exit, distance) == (distance < exit) ? distance : exit */
      ex = (dist < ex) ? dist : ex;
      dist -= ex;
      oe[k] = elem;
      ol[k] = ex;
      ++k;
      r = add(r, scl(ex, uu));
      elem = nxt;
      if (elem == XO_ID_NONE) break;
    }
    seg_count[i] = k;
    status[i] = st;
  }
}

/* ------------------------------------------------------------------------ */
/* Particle loops                                                           */
/* ------------------------------------------------------------------------ */

/* SplitMix64 (Steele, Lea & Flood, OOPSLA 2014): the per-particle stream */
static inline uint64_t splitmix_next(uint64_t* s) {
  *s += 0x9E3779B97F4A7C15ull;
  uint64_t z = *s;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

double xo_uniform(uint64_t* s) { return (double)(splitmix_next(s) >> 11) * 1.1102230246251565e-16; }

/* log x = e ln2 + 2 atanh(s), s = (m-1)/(m+1), m in [sqrt(1/2), sqrt(2)),
 * atanh by its Taylor series to s^23 (x positive and normal) */
double xo_series_log(double x) {
  uint64_t b;
  memcpy(&b, &x, sizeof b);
  int e = (int)((b >> 52) & 0x7ff) - 1023;
  uint64_t mb = (b & 0x000fffffffffffffull) | 0x3ff0000000000000ull;
  double m;
  memcpy(&m, &mb, sizeof m);
  if (m > 1.4142135623730951) {
    m = m * 0.5;
    e += 1;
  }
  const double s = (m - 1.0) / (m + 1.0);
  const double z = s * s;
  double p = 1.0 / 23.0;
  p = p * z + 1.0 / 21.0;
  p = p * z + 1.0 / 19.0;
  p = p * z + 1.0 / 17.0;
  p = p * z + 1.0 / 15.0;
  p = p * z + 1.0 / 13.0;
  p = p * z + 1.0 / 11.0;
  p = p * z + 1.0 / 9.0;
  p = p * z + 1.0 / 7.0;
  p = p * z + 1.0 / 5.0;
  p = p * z + 1.0 / 3.0;
  const double l = (s + s * z * p) * 2.0;
  const double hi = 0.6931471801362932, lo = 4.236521365809284e-10;
  const double de = (double)e;
  return de * hi + (de * lo + l);
}

/* tools/walk_elements.h:79: -std::log(1.0 - drand48()) * mean_free_path */
double xo_sample_collision(uint64_t* s, double mfp) { return -xo_series_log(1.0 - xo_uniform(s)) * mfp; }

/* Marsaglia (1972) in place of rand_dir (vec3da.h:170-176), then normalize */
void xo_sample_direction(uint64_t* s, double out[3]) {
  double x1 = 0.0, x2 = 0.0, q = 0.0;
  int ok = 0;
  for (int k = 0; k < 64 && !ok; ++k) {
    x1 = 2.0 * xo_uniform(s) - 1.0;
    x2 = 2.0 * xo_uniform(s) - 1.0;
    q = x1 * x1 + x2 * x2;
    ok = q < 1.0 && q > 0.0;
  }
  if (!ok) {
    out[0] = 0.0; out[1] = 0.0; out[2] = 1.0;
    return;
  }
  const double w = 2.0 * sqrt(1.0 - q);
  v3 d = {x1 * w, x2 * w, 1.0 - 2.0 * q};
  d = normalize(d);
  out[0] = d.x; out[1] = d.y; out[2] = d.z;
}

/* one event of tools/walk_elements.h:75-87 inside the mesh; returns 0 to go
 * on, else a status (particle stops) */
static int transport_event(const xo_tetmesh* m, int32_t* elem, v3* r, v3* u, uint64_t* rng,
                           double mfp, double* distance, double* tally) {
  int32_t nxt;
  double ex;
  next_element(m, *elem, *r, *u, &nxt, &ex);
  const double c = xo_sample_collision(rng, mfp);
  if (c < ex) {
    *r = add(*r, scl(c, *u));
    *distance += c;
    if (tally) {
#pragma omp atomic
      tally[*elem] += c;
    }
    double d[3];
    xo_sample_direction(rng, d);
    *u = mk(d);
    return 0;
  }
  if (ex >= XO_INFTY) return XO_NO_EXIT_FACE;
  *r = add(*r, scl(ex, *u));
  *distance += ex;
  if (tally) {
#pragma omp atomic
    tally[*elem] += ex;
  }
  *elem = nxt;
  return 0;
}

void xo_transport_elements(const xo_tetmesh* m, int64_t n, int32_t* elem, double* pos,
                           double* dir, uint64_t* rng, double mfp, int32_t max_events,
                           double* distance, int32_t* events, double* tally,
                           int32_t* status, int n_threads) {
#pragma omp parallel for schedule(dynamic, 16) num_threads(n_threads > 0 ? n_threads : 1)
  for (int64_t i = 0; i < n; ++i) {
    v3 r = mk(pos + 3 * i), u = mk(dir + 3 * i);
    int32_t e = elem[i];
    int st = XO_OK;
    while (e >= 0) {
      if (events[i] >= max_events) { st = XO_EVENT_LIMIT; break; }
      st = transport_event(m, &e, &r, &u, &rng[i], mfp, &distance[i], tally);
      if (st) break;
      events[i]++;
    }
    elem[i] = e;
    pos[3 * i] = r.x; pos[3 * i + 1] = r.y; pos[3 * i + 2] = r.z;
    dir[3 * i] = u.x; dir[3 * i + 1] = u.y; dir[3 * i + 2] = u.z;
    if (status) status[i] = st;
  }
}

void xo_walk_particles(const xo_tetmesh* m, const xo_tree* ipc, const xo_tree* etree, int64_t n,
                       int32_t* elem, double* pos, double* dir, uint64_t* rng, double mfp,
                       int32_t max_events, double* distance, int32_t* events, int32_t* status,
                       int n_threads) {
#pragma omp parallel for schedule(dynamic, 16) num_threads(n_threads > 0 ? n_threads : 1)
  for (int64_t i = 0; i < n; ++i) {
    v3 r = mk(pos + 3 * i), u = mk(dir + 3 * i);
    int32_t e = elem[i];
    int st = XO_OK;
    int32_t prims[64];
    int32_t nprim = 0;
    while (e != XO_ID_NONE) {  /* :73 */
      if (events[i] >= max_events) { st = XO_EVENT_LIMIT; break; }
      st = transport_event(m, &e, &r, &u, &rng[i], mfp, &distance[i], NULL);
      if (st) break;
      /* :88-94 re-entry through the implicit complement */
      while (e == XO_ID_NONE) {
        double o[3] = {r.x, r.y, r.z}, d[3] = {u.x, u.y, u.z}, t;
        int32_t off[2] = {0, nprim}, surf, face;
        xo_ray_fire(ipc, 1, o, d, NULL, XO_EXITING, off, prims, &t, &surf, &face, 1);
        if (surf == XO_ID_NONE) break;
        r = add(r, scl(t, u)); /* r += u * ray_hit.first */
        distance[i] += t;
        if (nprim < 64) prims[nprim++] = face; /* ray_fire appends the hit to primitives */
        const v3 q = add(r, scl(1e-10, u)); /* r + u*TINY_BIT */
        double qq[3] = {q.x, q.y, q.z};
        int32_t id, idx;
        xo_find_element(etree, 1, qq, &id, &idx, 1);
        e = idx;
        if (nprim >= 64 && e == XO_ID_NONE) break;
      }
      nprim = 0; /* primitives.clear() */
      events[i]++;
    }
    elem[i] = e;
    pos[3 * i] = r.x; pos[3 * i + 1] = r.y; pos[3 * i + 2] = r.z;
    dir[3 * i] = u.x; dir[3 * i + 1] = u.y; dir[3 * i + 2] = u.z;
    if (status) status[i] = st;
  }
}

/* tools/particle_sim.h:128-141 (Particle::surf_dist / advance / collide /
 * cross_surface) for particles given in a volume's tree, with the engine's
 * per-particle streams.  trees[k] is the tree of tree id k+1; the surface
 * tables are indexed by surface id, face_xyz by face id. */
void xo_transport_surfaces(const xo_tree* const* trees, int32_t n_trees, const int32_t* surf_fwd,
                           const int32_t* surf_rev, const int32_t* surf_bc, int32_t n_surf_ids,
                           const double* face_xyz, int32_t n_face_ids, int64_t n, int32_t* tree,
                           double* pos, double* dir, uint64_t* rng, double mfp,
                           int32_t max_events, int32_t graveyard_tree, double* distance,
                           int32_t* events, double* tally, int32_t* status, int n_threads) {
#pragma omp parallel for schedule(dynamic, 16) num_threads(n_threads > 0 ? n_threads : 1)
  for (int64_t i = 0; i < n; ++i) {
    v3 r = mk(pos + 3 * i), u = mk(dir + 3 * i);
    int32_t t = tree[i];
    int st = XO_OK;
    int32_t cap = 64, nh = 0;
    int32_t* hist = (int32_t*)malloc(sizeof(int32_t) * cap);
    int alive = t > 0;
    if (alive && events[i] >= max_events) { st = XO_EVENT_LIMIT; alive = 0; }
    while (alive) {
      if (t < 1 || t > n_trees) { st = 1; break; }
      /* surf_dist: ray_fire(volume, r, u, INFTY, EXITING, &history) */
      double o[3] = {r.x, r.y, r.z}, d[3] = {u.x, u.y, u.z}, th;
      int32_t off[2] = {0, nh}, surf, face;
      xo_ray_fire(trees[t - 1], 1, o, d, NULL, XO_EXITING, off, hist, &th, &surf, &face, 1);
      if (surf != XO_ID_NONE && th == 0.0) { st = 9; break; }  /* stuck */
      if (surf == XO_ID_NONE) { st = XO_LOST; break; }           /* lost */
      if (nh == cap) { cap *= 2; hist = (int32_t*)realloc(hist, sizeof(int32_t) * cap); }
      hist[nh++] = face;
      const double c = xo_sample_collision(&rng[i], mfp);
      if (c < th) {
        r = add(r, scl(c, u));
        distance[i] += c;
        if (tally) {
#pragma omp atomic
          tally[t] += c;
        }
        events[i]++;
        double nd[3];
        xo_sample_direction(&rng[i], nd);
        u = mk(nd);
        nh = 0;
      } else {
        r = add(r, scl(th, u));
        distance[i] += th;
        if (tally) {
#pragma omp atomic
          tally[t] += th;
        }
        events[i]++;
        const int bc = (surf >= 0 && surf < n_surf_ids) ? surf_bc[surf] : 0;
        if (bc == 2) {
          const double* f = face_xyz + 9 * (int64_t)hist[nh - 1];
          v3 nrm = face_normal(mk(f), mk(f + 3), mk(f + 6));
          const double proj = dot(nrm, u);
          const double mag = length(nrm);
          nrm = scl(2.0 * proj / mag, nrm);
          u = normalize(sub(u, nrm));
          hist[0] = hist[nh - 1];
          nh = 1;
        } else if (bc == 1) {
          alive = 0;
        } else {
          const int32_t fw = surf_fwd[surf], rv = surf_rev[surf];
          if (fw == t) t = rv;
          else if (rv == t) t = fw;
          else { st = 1; alive = 0; }
          if (alive && (t < 1 || t == graveyard_tree)) { t = -1; alive = 0; }
        }
        (void)n_face_ids;
      }
      if (alive && events[i] >= max_events) { st = XO_EVENT_LIMIT; alive = 0; }
    }
    free(hist);
    tree[i] = t;
    pos[3 * i] = r.x; pos[3 * i + 1] = r.y; pos[3 * i + 2] = r.z;
    dir[3 * i] = u.x; dir[3 * i + 1] = u.y; dir[3 * i + 2] = u.z;
    if (status) status[i] = st;
  }
}

int xo_version(void) { return 1; }
