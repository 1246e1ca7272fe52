// queries.cu -- BVH traversal kernels for the XDG ray queries.
//
// One thread owns one query (ray or point) for its whole traversal; a warp
// therefore carries a packet of 32 independent queries.  Each thread walks
// its tree depth-first with a private stack, testing all four children of a
// node at once and descending into the nearest hit child first.
//
// ray_fire / point_in_volume / occluded share one kernel body (MODE); the
// FP64 variant tests FP64 boxes and runs plucker64 on every candidate, the
// mixed variant tests FP32 boxes (rounded outward at build time) and runs the
// FP32 Plucker pre-filter, escalating to plucker64 only when the filter
// cannot certify a miss.  The hit bookkeeping after plucker64 is shared and
// follows triangle_intersect.cpp:52-109 exactly.
//
// Why the FP32 box test never loses a hit: every primitive box is dilated by
// `bump` (>= 1e-3 for surface trees, ray_tracing_interface.cpp:20-24), so the
// exact slab interval of a ray around any hit point has slack bump/|d|_inf on
// both sides, while the FP32 evaluation errs by at most ~5u(|box| + |o|).  A
// ray for which 8u(max|coordinate| + |o|_inf) is not below the bump is traced
// with the FP64 variant instead (checked per ray).
#include "queries.h"

namespace xdgcu {

namespace {

constexpr int kBlock = 128;
constexpr float kU32 = 5.9604645e-08f;  // 2^-24

struct Hit {
  double t;
  int32_t face;
  int32_t surf;
  bool has;
  bool dotpos;
};

struct Counters {
  unsigned long long box, node, prim, esc;
};

__device__ __forceinline__ void flush_counters(unsigned long long* g, const Counters& c,
                                               unsigned long long rays) {
  if (!g) return;
  unsigned long long v[5] = {c.box, c.node, c.prim, c.esc, rays};
  for (int k = 0; k < 5; ++k) {
    unsigned long long x = v[k];
    for (int off = 16; off > 0; off >>= 1) x += __shfl_xor_sync(__activemask(), x, off);
    v[k] = x;
  }
  if ((threadIdx.x & 31) == __ffs(__activemask()) - 1) {
    atomicAdd(&g[CNT_BOX], v[0]);
    atomicAdd(&g[CNT_NODE], v[1]);
    atomicAdd(&g[CNT_PRIM], v[2]);
    atomicAdd(&g[CNT_ESCALATE], v[3]);
    atomicAdd(&g[CNT_RAYS], v[4]);
  }
}

// Sort up to four (key, ref) pairs ascending by key (keys of misses are +inf).
__device__ __forceinline__ void sort4(float* k, int32_t* r) {
#define XDG_CSWAP(a, b)                 \
  if (k[b] < k[a]) {                    \
    float tk = k[a];                    \
    k[a] = k[b];                        \
    k[b] = tk;                          \
    int32_t tr = r[a];                  \
    r[a] = r[b];                        \
    r[b] = tr;                          \
  }
  XDG_CSWAP(0, 1);
  XDG_CSWAP(2, 3);
  XDG_CSWAP(0, 2);
  XDG_CSWAP(1, 3);
  XDG_CSWAP(1, 2);
#undef XDG_CSWAP
}

__device__ __forceinline__ void sort4d(double* k, int32_t* r) {
#define XDG_CSWAP(a, b)                 \
  if (k[b] < k[a]) {                    \
    double tk = k[a];                   \
    k[a] = k[b];                        \
    k[b] = tk;                          \
    int32_t tr = r[a];                  \
    r[a] = r[b];                        \
    r[b] = tr;                          \
  }
  XDG_CSWAP(0, 1);
  XDG_CSWAP(2, 3);
  XDG_CSWAP(0, 2);
  XDG_CSWAP(1, 3);
  XDG_CSWAP(1, 2);
#undef XDG_CSWAP
}

__device__ __forceinline__ float4 ld4(const float4* p) { return __ldg(p); }

// FP32 ray data for the box test
struct BoxRay32 {
  float ix, iy, iz;     // 1 / fl32(d) (tiny components replaced by +-1e-20)
  float ox, oy, oz;     // fl32(o) * inv
  int nx, ny, nz;       // index of the near plane vector (0 = lo, 1 = hi) per axis
};

__device__ __forceinline__ float safe_f(float x) {
  return fabsf(x) < 1e-20f ? copysignf(1e-20f, x) : x;
}
__device__ __forceinline__ double safe_d(double x) {
  return fabs(x) < 1e-200 ? copysign(1e-200, x) : x;
}

__device__ __forceinline__ BoxRay32 make_boxray32(d3 o, d3 d) {
  BoxRay32 r;
  r.ix = 1.0f / safe_f(__double2float_rn(d.x));
  r.iy = 1.0f / safe_f(__double2float_rn(d.y));
  r.iz = 1.0f / safe_f(__double2float_rn(d.z));
  r.ox = __double2float_rn(o.x) * r.ix;
  r.oy = __double2float_rn(o.y) * r.iy;
  r.oz = __double2float_rn(o.z) * r.iz;
  r.nx = signbit(r.ix) ? 1 : 0;
  r.ny = signbit(r.iy) ? 1 : 0;
  r.nz = signbit(r.iz) ? 1 : 0;
  return r;
}

// Slab test of the four children of an FP32 node against [0, tfar].
// Returns the near distances (+inf for misses).
__device__ __forceinline__ void node_test32(const Node32* np, const BoxRay32& r, float tfar,
                                            float tn[4], int32_t ref[4]) {
  const float4* v = reinterpret_cast<const float4*>(np);
  const float4 nx = ld4(v + 0 + r.nx), fx = ld4(v + 1 - r.nx);
  const float4 ny = ld4(v + 2 + r.ny), fy = ld4(v + 3 - r.ny);
  const float4 nz = ld4(v + 4 + r.nz), fz = ld4(v + 5 - r.nz);
  const int4 c = __ldg(reinterpret_cast<const int4*>(v + 6));
  const float nxa[4] = {nx.x, nx.y, nx.z, nx.w}, fxa[4] = {fx.x, fx.y, fx.z, fx.w};
  const float nya[4] = {ny.x, ny.y, ny.z, ny.w}, fya[4] = {fy.x, fy.y, fy.z, fy.w};
  const float nza[4] = {nz.x, nz.y, nz.z, nz.w}, fza[4] = {fz.x, fz.y, fz.z, fz.w};
  const int32_t ca[4] = {c.x, c.y, c.z, c.w};
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const float t0 = fmaxf(fmaxf(__fmaf_rn(nxa[k], r.ix, -r.ox), __fmaf_rn(nya[k], r.iy, -r.oy)),
                           fmaxf(__fmaf_rn(nza[k], r.iz, -r.oz), 0.0f));
    const float t1 = fminf(fminf(__fmaf_rn(fxa[k], r.ix, -r.ox), __fmaf_rn(fya[k], r.iy, -r.oy)),
                           fminf(__fmaf_rn(fza[k], r.iz, -r.oz), tfar));
    const bool hit = t0 <= t1;
    tn[k] = hit ? t0 : INFINITY;
    ref[k] = ca[k];
  }
}

struct BoxRay64 {
  double ix, iy, iz, ox, oy, oz;
  int nx, ny, nz;
};

__device__ __forceinline__ BoxRay64 make_boxray64(d3 o, d3 d) {
  BoxRay64 r;
  r.ix = 1.0 / safe_d(d.x);
  r.iy = 1.0 / safe_d(d.y);
  r.iz = 1.0 / safe_d(d.z);
  r.ox = o.x * r.ix;
  r.oy = o.y * r.iy;
  r.oz = o.z * r.iz;
  r.nx = signbit(r.ix) ? 1 : 0;
  r.ny = signbit(r.iy) ? 1 : 0;
  r.nz = signbit(r.iz) ? 1 : 0;
  return r;
}

__device__ __forceinline__ void node_test64(const Node64* np, const BoxRay64& r, double tfar,
                                            double tn[4], int32_t ref[4]) {
  const double* nx = r.nx ? np->hix : np->lox;
  const double* fx = r.nx ? np->lox : np->hix;
  const double* ny = r.ny ? np->hiy : np->loy;
  const double* fy = r.ny ? np->loy : np->hiy;
  const double* nz = r.nz ? np->hiz : np->loz;
  const double* fz = r.nz ? np->loz : np->hiz;
  const int4 c = __ldg(&np->child);
  const int32_t ca[4] = {c.x, c.y, c.z, c.w};
#pragma unroll
  for (int k = 0; k < 4; k += 2) {
    const double2 nx2 = __ldg(reinterpret_cast<const double2*>(nx + k));
    const double2 fx2 = __ldg(reinterpret_cast<const double2*>(fx + k));
    const double2 ny2 = __ldg(reinterpret_cast<const double2*>(ny + k));
    const double2 fy2 = __ldg(reinterpret_cast<const double2*>(fy + k));
    const double2 nz2 = __ldg(reinterpret_cast<const double2*>(nz + k));
    const double2 fz2 = __ldg(reinterpret_cast<const double2*>(fz + k));
    const double nxa[2] = {nx2.x, nx2.y}, fxa[2] = {fx2.x, fx2.y};
    const double nya[2] = {ny2.x, ny2.y}, fya[2] = {fy2.x, fy2.y};
    const double nza[2] = {nz2.x, nz2.y}, fza[2] = {fz2.x, fz2.y};
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const double t0 = fmax(fmax(fma(nxa[q], r.ix, -r.ox), fma(nya[q], r.iy, -r.oy)),
                             fmax(fma(nza[q], r.iz, -r.oz), 0.0));
      const double t1 = fmin(fmin(fma(fxa[q], r.ix, -r.ox), fma(fya[q], r.iy, -r.oy)),
                             fmin(fma(fza[q], r.iz, -r.oz), tfar));
      const bool hit = t0 <= t1;
      tn[k + q] = hit ? t0 : INFINITY;
      ref[k + q] = ca[k + q];
    }
  }
}

__device__ __forceinline__ void load_tri64(const double* p, d3& v0, d3& v1, d3& v2) {
  const double2 a = __ldg(reinterpret_cast<const double2*>(p));
  const double2 b = __ldg(reinterpret_cast<const double2*>(p + 2));
  const double2 c = __ldg(reinterpret_cast<const double2*>(p + 4));
  const double2 e = __ldg(reinterpret_cast<const double2*>(p + 6));
  const double f = __ldg(p + 8);
  v0 = mk3(a.x, a.y, b.x);
  v1 = mk3(b.y, c.x, c.y);
  v2 = mk3(e.x, e.y, f);
}

// The bookkeeping of TriangleIntersectionFunc (triangle_intersect.cpp:75-108)
// after an FP64 Plucker hit at distance t, plus the fixed tie rule.
template <int MODE>
__device__ __forceinline__ void accept_hit(const SurfArgs& a, const TreeDev& T, int32_t gtri,
                                           d3 v0, d3 v1, d3 v2, d3 d, double t, int32_t tid,
                                           const int32_t* excl, int32_t n_excl, Hit& h) {
  if (t > h.t) return;  // :78
  const int32_t fid = __ldg(&a.tri_face[gtri]);
  if (h.has && t == h.t && fid >= h.face) return;  // tie rule: lowest face id
  d3 nrm = face_normal64(v0, v1, v2);               // :80
  const int32_t sidx = __ldg(&a.tri_surf[gtri]);
  if (__ldg(&a.surf_rev_tree[sidx]) == tid) nrm = neg3(nrm);  // :84-87
  const double dp = dot3(d, nrm);
  if (MODE == MODE_RAY_FIRE) {  // orientation_cull, :12-24
    if (a.orientation == 0 && dp < 0.0) return;   // EXITING
    if (a.orientation == 1 && dp >= 0.0) return;  // ENTERING
  }
  for (int32_t k = 0; k < n_excl; ++k)  // primitive_mask_cull, :26-34
    if (__ldg(&excl[k]) == fid) return;
  h.has = true;
  h.t = t;
  h.face = fid;
  h.surf = __ldg(&a.surf_id[sidx]);
  h.dotpos = dp > 0.0;
}

// One tree traversal.  Returns false when the stack overflowed.
template <int MODE, bool MIXED>
__device__ __forceinline__ bool trace(const SurfArgs& a, const TreeDev& T, int32_t tid, d3 o,
                                      d3 d, const int32_t* excl, int32_t n_excl, Hit& h,
                                      Counters& cnt) {
  const d3 rn = cross3(d, o);  // plucker.h:75
  BoxRay32 br32;
  BoxRay64 br64;
  Ray32 r32;
  if (MIXED) {
    br32 = make_boxray32(o, d);
    r32 = make_ray32(o, d);
  } else {
    br64 = make_boxray64(o, d);
  }
  int32_t stack[kStackSize];
  int sp = 0;
  int32_t ref = T.root;
  if (ref == CHILD_EMPTY) return true;
  while (true) {
    if (!ref_is_leaf(ref)) {
      cnt.node++;
      cnt.box += 4;
      int32_t cr[4];
      int nhit = 0;
      if (MIXED) {
        float tn[4];
        const float tf = (MODE == MODE_OCCLUDED) ? INFINITY : __double2float_ru(h.t);
        node_test32(T.n32 + ref, br32, tf, tn, cr);
        sort4(tn, cr);
        for (int k = 0; k < 4; ++k) nhit += tn[k] < INFINITY ? 1 : 0;
      } else {
        double tn[4];
        const double tf = (MODE == MODE_OCCLUDED) ? INFTY : h.t;
        node_test64(T.n64 + ref, br64, tf, tn, cr);
        sort4d(tn, cr);
        for (int k = 0; k < 4; ++k) nhit += tn[k] < INFINITY ? 1 : 0;
      }
      if (nhit > 0) {
        if (sp + nhit - 1 > kStackSize) return false;
        for (int k = nhit - 1; k >= 1; --k) stack[sp++] = cr[k];
        ref = cr[0];
        continue;
      }
    } else {
      const int32_t first = leaf_first(ref), count = leaf_count(ref);
      for (int32_t p = first; p < first + count; ++p) {
        cnt.prim++;
        if (MIXED) {
          const float4 A = __ldg(&T.prim32[3 * (int64_t)p]);
          const float4 B = __ldg(&T.prim32[3 * (int64_t)p + 1]);
          const float4 C = __ldg(&T.prim32[3 * (int64_t)p + 2]);
          const SignCert c = plucker_filter32(r32, A.x, A.y, A.z, B.x, B.y, B.z, C.x, C.y, C.z,
                                              B.w, A.w);
          if (certified_miss(c)) continue;
          cnt.esc++;
        }
        d3 v0, v1, v2;
        load_tri64(T.prim64 + kPrim64Stride * (int64_t)p, v0, v1, v2);
        double t;
        const double tmax = (MODE == MODE_OCCLUDED) ? INFTY : h.t;
        if (!plucker64(v0, v1, v2, o, d, rn, tmax, 0.0, false, 0, &t)) continue;
        if (MODE == MODE_OCCLUDED) {
          h.has = true;
          return true;
        }
        const int32_t gtri = __ldg(&T.prim_ref[p]);
        accept_hit<MODE>(a, T, gtri, v0, v1, v2, d, t, tid, excl, n_excl, h);
      }
    }
    if (sp == 0) break;
    ref = stack[--sp];
  }
  return true;
}

template <int MODE, bool MIXED>
__global__ void __launch_bounds__(kBlock) k_surface(SurfArgs a) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  Counters cnt = {0, 0, 0, 0};
  if (i < a.n) {
    const int32_t tid = a.ray_trees ? a.ray_trees[i] : a.tree;
    const d3 o = load3(a.org, i);
    d3 d;
    if (MODE == MODE_PIV && a.dir == nullptr)
      d = mk3(1. / sqrt(2.0), 1 / sqrt(2.0), 0.0);  // embree/ray_tracer.cpp:268
    else
      d = load3(a.dir, i);
    double tmax = (MODE == MODE_RAY_FIRE && a.tmax) ? a.tmax[i] : INFTY;
    const int32_t* excl = nullptr;
    int32_t n_excl = 0;
    if (MODE != MODE_OCCLUDED && a.excl_off) {
      const int32_t e0 = a.excl_off[i];
      excl = a.excl_ids + e0;
      n_excl = a.excl_off[i + 1] - e0;
    }
    int32_t st = RAY_OK;
    Hit h;
    h.t = tmax;
    h.face = -1;
    h.surf = -1;
    h.has = false;
    h.dotpos = false;
    if (tid < 1 || tid > a.n_trees || !finite3(o) || !finite3(d) || isnan(tmax)) {
      st = RAY_INVALID;
    } else {
      const TreeDev T = a.trees[tid - 1];
      bool ok;
      bool use32 = MIXED;
      if (MIXED) {
        // FP32 box-test safety (see the file comment)
        const float oa = fmaxf(fabsf((float)o.x), fmaxf(fabsf((float)o.y), fabsf((float)o.z)));
        use32 = 8.0f * kU32 * (T.max_abs + oa) < T.bump;
      }
      if (use32)
        ok = trace<MODE, true>(a, T, tid, o, d, excl, n_excl, h, cnt);
      else
        ok = trace<MODE, false>(a, T, tid, o, d, excl, n_excl, h, cnt);
      if (!ok) st = RAY_STACK_OVERFLOW;
    }
    if (MODE == MODE_RAY_FIRE) {
      a.t_out[i] = h.has ? h.t : INFTY;
      a.surf_out[i] = h.has ? h.surf : -1;
      if (a.face_out) a.face_out[i] = h.has ? h.face : -1;
    } else if (MODE == MODE_PIV) {
      a.flag_out[i] = (h.has && h.dotpos) ? 1 : 0;  // embree/ray_tracer.cpp:282-286
    } else {
      a.flag_out[i] = h.has ? 1 : 0;
      if (a.dist_out) a.dist_out[i] = h.has ? -INFTY : INFTY;  // embree/ray_tracer.cpp:368-369
    }
    if (a.status) a.status[i] = st;
  }
  if (a.counters) flush_counters(a.counters, cnt, i < a.n ? 1ull : 0ull);
}

// ---------------------------------------------------------------------------
// closest (point query, embree/ray_tracer.cpp:328-345)
// ---------------------------------------------------------------------------

template <bool MIXED>
__global__ void __launch_bounds__(kBlock) k_closest(PointArgs a) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  Counters cnt = {0, 0, 0, 0};
  if (i < a.n) {
    const int32_t tid = a.ray_trees ? a.ray_trees[i] : a.tree;
    const d3 p = load3(a.pts, i);
    double best = INFTY;
    int32_t best_face = -1;
    int32_t st = RAY_OK;
    if (tid < 1 || tid > a.n_trees || !finite3(p)) {
      st = RAY_INVALID;
    } else {
      const TreeDev T = a.trees[tid - 1];
      const float px = __double2float_rn(p.x), py = __double2float_rn(p.y),
                  pz = __double2float_rn(p.z);
      const float pabs = fmaxf(fabsf(px), fmaxf(fabsf(py), fabsf(pz)));
      int32_t stack[kStackSize];
      int sp = 0;
      int32_t ref = T.root;
      bool run = ref != CHILD_EMPTY;
      while (run) {
        if (!ref_is_leaf(ref)) {
          cnt.node++;
          cnt.box += 4;
          int32_t cr[4];
          int nhit = 0;
          if (MIXED) {
            const Node32* np = T.n32 + ref;
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
              float s = 0.0f;
              bool empty = false;
#pragma unroll
              for (int ax = 0; ax < 3; ++ax) {
                empty |= !(la[ax][k] <= ha[ax][k]);
                const float e = fmaxf(fmaxf(la[ax][k] - pa[ax], pa[ax] - ha[ax][k]), 0.0f);
                s += e * e;
              }
              const float dist = sqrtf(s);
              const float lb = dist * (1.0f - 8.0f * kU32) - 4.0f * kU32 * pabs;
              key[k] = (!empty && lb <= bestf) ? dist : INFINITY;
              cr[k] = ca[k];
            }
            sort4(key, cr);
            for (int k = 0; k < 4; ++k) nhit += key[k] < INFINITY ? 1 : 0;
          } else {
            const Node64* np = T.n64 + ref;
            const int4 c = __ldg(&np->child);
            const int32_t ca[4] = {c.x, c.y, c.z, c.w};
            double key[4];
            const double pa[3] = {p.x, p.y, p.z};
            const double* lo[3] = {np->lox, np->loy, np->loz};
            const double* hi[3] = {np->hix, np->hiy, np->hiz};
#pragma unroll
            for (int k = 0; k < 4; ++k) {
              double s = 0.0;
              bool empty = false;
#pragma unroll
              for (int ax = 0; ax < 3; ++ax) {
                const double l = __ldg(lo[ax] + k), u = __ldg(hi[ax] + k);
                empty |= !(l <= u);
                const double e = fmax(fmax(l - pa[ax], pa[ax] - u), 0.0);
                s += e * e;
              }
              const double dist = sqrt(s);
              key[k] = (!empty && dist * (1.0 - 1e-12) <= best) ? dist : INFINITY;
              cr[k] = ca[k];
            }
            sort4d(key, cr);
            for (int k = 0; k < 4; ++k) nhit += key[k] < INFINITY ? 1 : 0;
          }
          if (nhit > 0) {
            if (sp + nhit - 1 > kStackSize) {
              st = RAY_STACK_OVERFLOW;
              break;
            }
            for (int k = nhit - 1; k >= 1; --k) stack[sp++] = cr[k];
            ref = cr[0];
            continue;
          }
        } else {
          const int32_t first = leaf_first(ref), count = leaf_count(ref);
          for (int32_t q = first; q < first + count; ++q) {
            cnt.prim++;
            d3 v0, v1, v2;
            load_tri64(T.prim64 + kPrim64Stride * (int64_t)q, v0, v1, v2);
            const d3 r = closest64(v0, v1, v2, p);
            const double dd = dist64(r, p);
            const int32_t fid = __ldg(&a.tri_face[__ldg(&T.prim_ref[q])]);
            // triangle_intersect.cpp:126-133 (strict <) plus the tie rule
            if (dd < best || (dd == best && best_face >= 0 && fid < best_face)) {
              best = dd;
              best_face = fid;
            }
          }
        }
        if (sp == 0) break;
        ref = stack[--sp];
      }
    }
    a.dist_out[i] = best_face >= 0 ? best : INFTY;
    if (a.id_out) a.id_out[i] = best_face;
    if (a.status) a.status[i] = st;
  }
  if (a.counters) flush_counters(a.counters, cnt, i < a.n ? 1ull : 0ull);
}

// ---------------------------------------------------------------------------
// find_element (embree/ray_tracer.cpp:226-257 + tetrahedron_contain.cpp:94-114)
// ---------------------------------------------------------------------------

template <bool MIXED>
__global__ void __launch_bounds__(kBlock) k_find_element(PointArgs a) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
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
      int32_t stack[kStackSize];
      int sp = 0;
      int32_t ref = T.root;
      bool run = ref != CHILD_EMPTY;
      while (run) {
        if (!ref_is_leaf(ref)) {
          cnt.node++;
          cnt.box += 4;
          int32_t cr[4];
          int nhit = 0;
          if (MIXED) {
            const Node32* np = T.n32 + ref;
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
            const Node64* np = T.n64 + ref;
            const int4 c = __ldg(&np->child);
            const int32_t ca[4] = {c.x, c.y, c.z, c.w};
            for (int k = 0; k < 4; ++k) {
              const bool in = p.x >= __ldg(np->lox + k) && p.x <= __ldg(np->hix + k) &&
                              p.y >= __ldg(np->loy + k) && p.y <= __ldg(np->hiy + k) &&
                              p.z >= __ldg(np->loz + k) && p.z <= __ldg(np->hiz + k);
              if (in) cr[nhit++] = ca[k];
            }
          }
          if (nhit > 0) {
            if (sp + nhit - 1 > kStackSize) {
              st = RAY_STACK_OVERFLOW;
              break;
            }
            for (int k = nhit - 1; k >= 1; --k) stack[sp++] = cr[k];
            ref = cr[0];
            continue;
          }
        } else {
          const int32_t first = leaf_first(ref), count = leaf_count(ref);
          for (int32_t q = first; q < first + count; ++q) {
            cnt.prim++;
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

inline unsigned grid_for(int64_t n) { return (unsigned)((n + kBlock - 1) / kBlock); }

}  // namespace

cudaError_t launch_surface_query(int mode, bool mixed, const SurfArgs& a, cudaStream_t st) {
  if (a.n <= 0) return cudaSuccess;
  const unsigned g = grid_for(a.n);
  switch (mode * 2 + (mixed ? 1 : 0)) {
    case 0: k_surface<MODE_RAY_FIRE, false><<<g, kBlock, 0, st>>>(a); break;
    case 1: k_surface<MODE_RAY_FIRE, true><<<g, kBlock, 0, st>>>(a); break;
    case 2: k_surface<MODE_PIV, false><<<g, kBlock, 0, st>>>(a); break;
    case 3: k_surface<MODE_PIV, true><<<g, kBlock, 0, st>>>(a); break;
    case 4: k_surface<MODE_OCCLUDED, false><<<g, kBlock, 0, st>>>(a); break;
    case 5: k_surface<MODE_OCCLUDED, true><<<g, kBlock, 0, st>>>(a); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_closest(bool mixed, const PointArgs& a, cudaStream_t st) {
  if (a.n <= 0) return cudaSuccess;
  if (mixed)
    k_closest<true><<<grid_for(a.n), kBlock, 0, st>>>(a);
  else
    k_closest<false><<<grid_for(a.n), kBlock, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_find_element(bool mixed, const PointArgs& a, cudaStream_t st) {
  if (a.n <= 0) return cudaSuccess;
  if (mixed)
    k_find_element<true><<<grid_for(a.n), kBlock, 0, st>>>(a);
  else
    k_find_element<false><<<grid_for(a.n), kBlock, 0, st>>>(a);
  return cudaGetLastError();
}

}  // namespace xdgcu
