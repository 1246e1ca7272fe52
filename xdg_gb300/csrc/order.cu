// order.cu -- coherent ray order for the traversal kernels.
//
// Rays of one warp that start close together, run in the same tree and point
// into the same octant visit mostly the same upper BVH nodes, so their node
// fetches hit L1 and their loops diverge less.  ray_order() computes one
// 32-bit key per ray,
//
//   [tree id | direction octant (3 bits) | Morton code of the origin]
//
// (tree bits only when rays carry their own tree ids), sorts the ray indices
// by it with a device radix sort, and returns the permutation.  The traversal
// kernel reads ray order[k] at position k and writes its results at the
// original index, so results do not depend on the order.
#include <cub/cub.cuh>

#include "queries.h"

namespace xdgcu {

namespace {

// spreads the low 10 bits of v so that bit i moves to bit 3i
__device__ __forceinline__ uint32_t spread3(uint32_t v) {
  v &= 0x3ffu;
  v = (v | (v << 16)) & 0x030000ffu;
  v = (v | (v << 8)) & 0x0300f00fu;
  v = (v | (v << 4)) & 0x030c30c3u;
  v = (v | (v << 2)) & 0x09249249u;
  return v;
}

__device__ __forceinline__ uint32_t quant(double x, double lo, double scale, uint32_t top) {
  const double q = (x - lo) * scale;
  if (!(q > 0.0)) return 0u;  // also NaN
  if (q >= (double)top) return top;
  return (uint32_t)q;
}

__global__ void k_ray_keys(const double* org, const double* dir, const int32_t* ray_trees,
                           int64_t n, double extent, int tree_bits, int axis_bits,
                           uint32_t* keys, int32_t* idx) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t top = (1u << axis_bits) - 1u;
  const double scale = (double)(1u << axis_bits) / (2.0 * extent);
  const uint32_t qx = quant(org[3 * i], -extent, scale, top);
  const uint32_t qy = quant(org[3 * i + 1], -extent, scale, top);
  const uint32_t qz = quant(org[3 * i + 2], -extent, scale, top);
  const uint32_t morton = spread3(qx) | (spread3(qy) << 1) | (spread3(qz) << 2);
  uint32_t oct = 0u;
  if (dir) {
    oct = (signbit(dir[3 * i]) ? 1u : 0u) | (signbit(dir[3 * i + 1]) ? 2u : 0u) |
          (signbit(dir[3 * i + 2]) ? 4u : 0u);
  }
  uint32_t key = (oct << (3 * axis_bits)) | morton;
  if (tree_bits > 0) {
    const uint32_t t = (uint32_t)ray_trees[i] & ((1u << tree_bits) - 1u);
    key |= t << (3 * axis_bits + 3);
  }
  keys[i] = key;
  idx[i] = (int32_t)i;
}

size_t al256(size_t b) { return (b + 255) & ~(size_t)255; }

int bits_for(int32_t v) {
  int b = 0;
  while (b < 31 && (1 << b) <= v) ++b;
  return b;
}

}  // namespace

size_t ray_order_scratch_bytes(int64_t n) {
  size_t tmp = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, tmp, (const uint32_t*)nullptr, (uint32_t*)nullptr,
                                  (const int32_t*)nullptr, (int32_t*)nullptr, (int)n);
  return al256(tmp) + 2 * al256(sizeof(uint32_t) * n) + al256(sizeof(int32_t) * n);
}

cudaError_t ray_order(const double* org, const double* dir, const int32_t* ray_trees,
                      int32_t n_trees, int64_t n, double extent, int32_t* order, void* scratch,
                      size_t scratch_bytes, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  if (n >= ((int64_t)1 << 31) || !(extent > 0.0)) return cudaErrorInvalidValue;
  // tree bits (per-ray trees only), 3 octant bits, the rest for the origin
  const int tree_bits = ray_trees ? std::min(bits_for(n_trees), 11) : 0;
  const int axis_bits = std::min(10, (32 - 3 - tree_bits) / 3);
  const int end_bit = 3 * axis_bits + 3 + tree_bits;
  size_t tmp = 0;
  cudaError_t e = cub::DeviceRadixSort::SortPairs(
      nullptr, tmp, (const uint32_t*)nullptr, (uint32_t*)nullptr, (const int32_t*)nullptr,
      (int32_t*)nullptr, (int)n, 0, end_bit, st);
  if (e != cudaSuccess) return e;
  char* p = (char*)scratch;
  const size_t kb = al256(sizeof(uint32_t) * n);
  if (al256(tmp) + 2 * kb + al256(sizeof(int32_t) * n) > scratch_bytes) return cudaErrorInvalidValue;
  uint32_t* keys_in = (uint32_t*)(p + al256(tmp));
  uint32_t* keys_out = (uint32_t*)(p + al256(tmp) + kb);
  int32_t* idx = (int32_t*)(p + al256(tmp) + 2 * kb);
  k_ray_keys<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(org, dir, ray_trees, n, extent,
                                                          tree_bits, axis_bits, keys_in, idx);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return cub::DeviceRadixSort::SortPairs(p, tmp, keys_in, keys_out, idx, order, (int)n, 0,
                                         end_bit, st);
}

}  // namespace xdgcu
