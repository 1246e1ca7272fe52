// cbound.h -- the four FP32 planes per triangle behind closest's FP32 lower
// bound of the point-triangle distance (k_closest in queries.cu).  Plain C++
// shared by the device build (k_tri_cbound) and a host build in the tests.
//
// Planes, as (x, y, z, offset): the face plane (n, d), then for each edge k
// (V[k] -> V[k+1]) an in-plane plane (m_k, c_k) facing away from the
// triangle.  They are certified against the triangle's own vertices, in FP64
// with the standard dot-product error bound (3 terms: |error| <= 3 eps sum|a b|,
// eps = 2^-53; 8 eps is used), so that for every point x of the triangle
//   |n . x - d| <= 7 u max|V|  and  m_k . x <= c_k     (u = 2^-24),
// whatever the accuracy of the computed normal (a needle's FP64 normal can be
// far off its true direction: the checks, not the construction, carry the
// proof), and the rows n, m_k are near-orthonormal: |n|, |m_k| <= 1 + 4u and
// |n . m_k| <= 4u.  A triangle that fails a check (degenerate, ill-conditioned,
// or with coordinates beyond 1e30) gets a NaN face offset, and the bound never
// skips it.
#pragma once

#include <math.h>

#ifdef __CUDACC__
#define XDG_CB_HD __host__ __device__
#else
#define XDG_CB_HD
#endif

namespace xdgcu {

// the smallest float >= x (x finite)
XDG_CB_HD inline float cb_f32_up(double x) {
  float f = (float)x;
  if ((double)f < x) f = nextafterf(f, INFINITY);
  return f;
}

// v: 9 doubles (three vertices); out: 16 floats (four planes)
XDG_CB_HD inline void tri_cbound(const double* v, float* out) {
  const double eps = 1.1102230246251565e-16;  // 2^-53
  const double u = 5.9604644775390625e-08;    // 2^-24
  double V[3][3];
  double vmax = 0.0;
  for (int k = 0; k < 3; ++k)
    for (int i = 0; i < 3; ++i) {
      V[k][i] = v[3 * k + i];
      vmax = fmax(vmax, fabs(V[k][i]));
    }
  bool ok = vmax < 1e30;  // (a NaN coordinate fails on the normal's length below)
  double e1[3], e2[3];
  for (int i = 0; i < 3; ++i) {
    e1[i] = V[1][i] - V[0][i];
    e2[i] = V[2][i] - V[0][i];
  }
  const double n[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2],
                       e1[0] * e2[1] - e1[1] * e2[0]};
  const double ln = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
  ok = ok && ln > 0.0 && ln < INFINITY;
  float nf[3];
  for (int i = 0; i < 3; ++i) nf[i] = ok ? (float)(n[i] / ln) : 0.0f;
  // face offset: the middle of the vertices' heights over nf
  double hmin = INFINITY, hmax = -INFINITY, g = 0.0;
  for (int k = 0; k < 3; ++k) {
    const double h = (double)nf[0] * V[k][0] + (double)nf[1] * V[k][1] + (double)nf[2] * V[k][2];
    hmin = fmin(hmin, h);
    hmax = fmax(hmax, h);
    g = fmax(g, fabs((double)nf[0] * V[k][0]) + fabs((double)nf[1] * V[k][1]) +
                    fabs((double)nf[2] * V[k][2]));
  }
  const float d = ok ? (float)(0.5 * (hmin + hmax)) : 0.0f;
  double slack = 0.0;
  for (int k = 0; k < 3; ++k) {
    const double h = (double)nf[0] * V[k][0] + (double)nf[1] * V[k][1] + (double)nf[2] * V[k][2];
    slack = fmax(slack, fabs(h - (double)d));
  }
  slack += 8.0 * eps * (g + fabs((double)d));
  ok = ok && slack <= 7.0 * u * vmax;
  const double nn = (double)nf[0] * nf[0] + (double)nf[1] * nf[1] + (double)nf[2] * nf[2];
  ok = ok && nn <= (1.0 + 4.0 * u) * (1.0 + 4.0 * u);
  out[0] = nf[0];
  out[1] = nf[1];
  out[2] = nf[2];
  out[3] = d;
  for (int k = 0; k < 3; ++k) {
    const double* a = V[k];
    const double* b = V[(k + 1) % 3];
    const double e[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
    const double m[3] = {e[1] * n[2] - e[2] * n[1], e[2] * n[0] - e[0] * n[2],
                         e[0] * n[1] - e[1] * n[0]};
    const double lm = sqrt(m[0] * m[0] + m[1] * m[1] + m[2] * m[2]);
    ok = ok && lm > 0.0 && lm < INFINITY;
    float mf[3];
    for (int i = 0; i < 3; ++i) mf[i] = ok ? (float)(m[i] / lm) : 0.0f;
    // offset: the largest vertex height over mf, rounded up past the error
    double c = -INFINITY;
    for (int q = 0; q < 3; ++q) {
      const double s = (double)mf[0] * V[q][0] + (double)mf[1] * V[q][1] + (double)mf[2] * V[q][2];
      const double ga = fabs((double)mf[0] * V[q][0]) + fabs((double)mf[1] * V[q][1]) +
                        fabs((double)mf[2] * V[q][2]);
      c = fmax(c, s + 8.0 * eps * ga);
    }
    const double mm = (double)mf[0] * mf[0] + (double)mf[1] * mf[1] + (double)mf[2] * mf[2];
    const double nm = (double)nf[0] * mf[0] + (double)nf[1] * mf[1] + (double)nf[2] * mf[2];
    ok = ok && mm <= (1.0 + 4.0 * u) * (1.0 + 4.0 * u) && fabs(nm) <= 4.0 * u;
    out[4 * (k + 1) + 0] = mf[0];
    out[4 * (k + 1) + 1] = mf[1];
    out[4 * (k + 1) + 2] = mf[2];
    out[4 * (k + 1) + 3] = ok ? cb_f32_up(c) : 0.0f;
  }
  if (!ok) out[3] = NAN;
}

}  // namespace xdgcu
