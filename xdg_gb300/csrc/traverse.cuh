// traverse.cuh -- device helpers shared by the BVH traversal kernels:
// per-ray FP32/FP64 slab-test setup, the 4-child node tests, small sorting
// networks and the FP64 triangle fetch.
#pragma once

#include "queries.h"

namespace xdgcu {

constexpr float kU32 = 5.9604645e-08f;  // 2^-24

struct Hit {
  double t;
  int32_t face;
  int32_t surf;
  bool has;
  bool dotpos;
};

// per-thread work counts (32-bit: a thread's share of one launch stays far
// below 2^32; the launch totals are 64-bit)
struct Counters {
  uint32_t box, node, prim, esc;
};

__device__ __forceinline__ void flush_counters(unsigned long long* g, const Counters& c,
                                               unsigned long long rays) {
  if (!g) return;
  unsigned long long v[5] = {(unsigned long long)c.box, (unsigned long long)c.node,
                            (unsigned long long)c.prim, (unsigned long long)c.esc, rays};
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

// Merges two ascending (key, ref) lists k[0..3] and k[4..7] into one
// ascending list of eight (bitonic merge: reverse the second half, then
// compare-exchange at distances 4, 2, 1).
__device__ __forceinline__ void merge8(float* k, int32_t* r) {
#define XDG_CSWAP(a, b)                 \
  if (k[b] < k[a]) {                    \
    float tk = k[a];                    \
    k[a] = k[b];                        \
    k[b] = tk;                          \
    int32_t tr = r[a];                  \
    r[a] = r[b];                        \
    r[b] = tr;                          \
  }
#define XDG_SWAP(a, b)                  \
  {                                     \
    float tk = k[a];                    \
    k[a] = k[b];                        \
    k[b] = tk;                          \
    int32_t tr = r[a];                  \
    r[a] = r[b];                        \
    r[b] = tr;                          \
  }
  XDG_SWAP(4, 7);
  XDG_SWAP(5, 6);
  XDG_CSWAP(0, 4);
  XDG_CSWAP(1, 5);
  XDG_CSWAP(2, 6);
  XDG_CSWAP(3, 7);
  XDG_CSWAP(0, 2);
  XDG_CSWAP(1, 3);
  XDG_CSWAP(4, 6);
  XDG_CSWAP(5, 7);
  XDG_CSWAP(0, 1);
  XDG_CSWAP(2, 3);
  XDG_CSWAP(4, 5);
  XDG_CSWAP(6, 7);
#undef XDG_SWAP
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
  float ix, iy, iz;     // 1 / f32(d) (tiny components replaced by +-1e-20)
  float ox, oy, oz;     // f32(o) * inv
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
  r.ix = 1.0f / safe_f(f32_trunc(d.x));
  r.iy = 1.0f / safe_f(f32_trunc(d.y));
  r.iz = 1.0f / safe_f(f32_trunc(d.z));
  r.ox = f32_trunc(o.x) * r.ix;
  r.oy = f32_trunc(o.y) * r.iy;
  r.oz = f32_trunc(o.z) * r.iz;
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


}  // namespace xdgcu
