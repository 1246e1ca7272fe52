// sample.cuh -- random sampling for the device particle loops.
//
// The reference tools draw from one global drand48() stream
// (tools/walk_elements.h:75-86, tools/particle_sim.h:47-64) and sample
// directions with acos/sin/cos (rand_dir, include/xdg/vec3da.h:170-176), so no
// run of them can be reproduced particle by particle once particles run in
// parallel.  The engine gives every particle its own stream instead, and
// uses only operations that round identically on the GPU and on the host
// (integer arithmetic, IEEE +, -, *, / and sqrt, no contraction), so a CPU
// restatement reproduces every particle history bit for bit:
//
//   * stream: SplitMix64 (Steele, Lea & Flood, "Fast splittable pseudorandom
//     number generators", OOPSLA 2014) on a 64-bit state per particle;
//     uniform = top 53 bits x 2^-53, in [0, 1);
//   * collision distance -log(1 - U) * mfp with a logarithm evaluated here
//     from its series: x = m 2^e with m in [sqrt(1/2), sqrt(2)),
//     log x = e ln2 + 2 atanh(s), s = (m - 1) / (m + 1), atanh by its Taylor
//     series to s^23 (|s| <= 0.1716, truncation below 1e-20 relative);
//   * isotropic direction by Marsaglia's method ("Choosing a point from the
//     surface of a sphere", Ann. Math. Stat. 43, 1972): (x1, x2) uniform in
//     the unit disc, d = (2 x1 sqrt(1-s), 2 x2 sqrt(1-s), 1 - 2s), then
//     Vec3da::normalize as rand_dir does.  The distribution is the same as
//     rand_dir's (uniform on the sphere); the draws are not.
#pragma once

#include "geom.cuh"

namespace xdgcu {

constexpr unsigned long long kGolden = 0x9E3779B97F4A7C15ull;

__device__ __forceinline__ unsigned long long splitmix_next(unsigned long long& s) {
  s += kGolden;
  unsigned long long z = s;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// uniform in [0, 1) with 53 random bits
__device__ __forceinline__ double uniform53(unsigned long long& s) {
  return (double)(splitmix_next(s) >> 11) * 1.1102230246251565e-16;  // 2^-53
}

// natural logarithm of a positive normal double (see the file comment)
__device__ __forceinline__ double series_log(double x) {
  const long long b = __double_as_longlong(x);
  int e = (int)((b >> 52) & 0x7ff) - 1023;
  double m = __longlong_as_double((b & 0x000fffffffffffffll) | 0x3ff0000000000000ll);
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
  // ln 2 split so that e * kLn2Hi is exact for |e| < 2^22
  const double kLn2Hi = 0.6931471801362932;
  const double kLn2Lo = 4.236521365809284e-10;
  const double de = (double)e;
  return de * kLn2Hi + (de * kLn2Lo + l);
}

// collision distance, tools/walk_elements.h:79 and tools/particle_sim.h:47-49
__device__ __forceinline__ double sample_collision(unsigned long long& s, double mfp) {
  return -series_log(1.0 - uniform53(s)) * mfp;
}

// isotropic unit direction (see the file comment); gives up after 64
// rejections (probability below 1e-42) with +z
__device__ __forceinline__ d3 sample_direction(unsigned long long& s) {
  double x1 = 0.0, x2 = 0.0, q = 0.0;
  bool ok = false;
  for (int k = 0; k < 64 && !ok; ++k) {
    x1 = 2.0 * uniform53(s) - 1.0;
    x2 = 2.0 * uniform53(s) - 1.0;
    q = x1 * x1 + x2 * x2;
    ok = q < 1.0 && q > 0.0;
  }
  if (!ok) return mk3(0.0, 0.0, 1.0);
  const double w = 2.0 * sqrt(1.0 - q);
  return normalize64(mk3(x1 * w, x2 * w, 1.0 - 2.0 * q));
}

}  // namespace xdgcu
