// internal.cuh -- data layout of the ray-query engine in device memory.
//
// Trees are 4- or 8-wide BVHs (an 8-wide node is two consecutive 4-wide
// records) stored twice: once with FP32 boxes rounded outward
// (the mixed-precision path) and once with FP64 boxes (the all-FP64 path).
// A node holds its four children's boxes as six float4 (or 6x4 double)
// vectors -- lo.x of children 0..3, hi.x, lo.y, hi.y, lo.z, hi.z -- followed
// by the four child references, so one thread fetches a node with seven
// (FP32) or thirteen (FP64) 16-byte loads and tests all four children with
// vector-wide arithmetic.
//
// Child references: >= 0 is an inner node index; < 0 is a leaf holding
// `count` (1..16) consecutive primitives of the tree's leaf-ordered primitive
// arrays starting at `first`; CHILD_EMPTY marks an unused slot (its box is
// empty, so no ray ever enters it).
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>

#include "geom.cuh"

namespace xdgcu {

constexpr int kWidth = 4;
constexpr int32_t CHILD_EMPTY = 0x7fffffff;
constexpr int kStackSize = 96;

__host__ __device__ __forceinline__ bool ref_is_leaf(int32_t c) { return c < 0; }
__host__ __device__ __forceinline__ int32_t leaf_first(int32_t c) {
  return (int32_t)(((uint32_t)c & 0x7fffffffu) >> 4);
}
__host__ __device__ __forceinline__ int32_t leaf_count(int32_t c) {
  return (int32_t)((uint32_t)c & 15u) + 1;
}
__host__ __device__ __forceinline__ int32_t make_leaf(int32_t first, int32_t count) {
  return (int32_t)(0x80000000u | ((uint32_t)first << 4) | (uint32_t)(count - 1));
}

struct __align__(16) Node32 {
  float4 lox, hix, loy, hiy, loz, hiz;
  int4 child;
};
static_assert(sizeof(Node32) == 112, "Node32 layout");

struct __align__(16) Node64 {
  double lox[4], hix[4], loy[4], hiy[4], loz[4], hiz[4];
  int4 child;
};
static_assert(sizeof(Node64) == 208, "Node64 layout");

enum TreeKind : int32_t { TREE_SURFACE = 0, TREE_ELEMENT = 1 };

// Everything a kernel needs to traverse one tree.  Primitive arrays are in
// leaf order (the BVH's sorted order):
//   surface trees: prim32 = 3 float4 per triangle
//                     (v0.xyz, |v0|_inf), (v1-v0, max edge |.|_inf),
//                     (v2-v0, 1 if well shaped at v0 for closest's upper bound, else 0)
//                  prim64 = 10 doubles per triangle (v0, v1, v2, pad)
//                  prim_ref = global triangle index
//   element trees: prim64 = 12 doubles per tet (v0..v3), prim_ref = tet index
struct TreeDev {
  const Node32* n32;
  const Node64* n64;
  const float4* prim32;
  const double* prim64;
  const int32_t* prim_ref;
  int32_t root;      // a child reference (inner node 0, or a leaf, or CHILD_EMPTY)
  int32_t n_prims;
  int32_t depth;
  int32_t tree_id;
  float bump;        // box dilation used for this tree (FP32, rounded down)
  float max_abs;     // max |coordinate| over the tree's (bumped) bounds
  int32_t kind;
  int32_t width;     // 4 or 8 children per node; node k = records k*width/4 ..
};

constexpr int kPrim64Stride = 10;  // doubles per triangle in prim64

// Devices a process can use with per-device launch caches (more are
// served, with the caches bypassed).
constexpr int kMaxDevices = 64;

// The current device, or -1.
inline int current_device() {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return -1;
  }
  return dev;
}

// Number of SMs of the current device, read once per device (any host
// thread) for the persistent launches' grid sizes.
inline int device_sm_count() {
  static std::atomic<int> cache[kMaxDevices];
  const int dev = current_device();
  if (dev >= 0 && dev < kMaxDevices) {
    const int c = cache[dev].load(std::memory_order_acquire);
    if (c > 0) return c;
  }
  int v = 0;
  if (dev < 0 || cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    cudaGetLastError();
    v = 0;
  }
  v = v > 0 ? v : 1;
  if (dev >= 0 && dev < kMaxDevices) cache[dev].store(v, std::memory_order_release);
  return v;
}

// Resident blocks per SM of `kern` on the current device (`block` threads,
// `smem` bytes of dynamic shared memory), looked up once per device in the
// caller's `cache` (one per kernel variant and launch shape).
template <typename K>
cudaError_t occupancy_cached(std::atomic<int>* cache, K kern, int block, size_t smem,
                             int& per_sm) {
  const int dev = current_device();
  const bool use = dev >= 0 && dev < kMaxDevices;
  per_sm = use ? cache[dev].load(std::memory_order_acquire) : 0;
  if (per_sm > 0) return cudaSuccess;
  const cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, block, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  if (use) cache[dev].store(per_sm, std::memory_order_release);
  return cudaSuccess;
}

// Makes `device` current for the scope of an entry point and makes the
// caller's current device current again on the way out, so that a host
// thread driving several GPUs keeps the device it selected.
class DeviceGuard {
 public:
  explicit DeviceGuard(int device) : prev_(current_device()) {
    ok_ = prev_ == device || cudaSetDevice(device) == cudaSuccess;
    if (!ok_) cudaGetLastError();
  }
  ~DeviceGuard() {
    if (prev_ >= 0 && current_device() != prev_) cudaSetDevice(prev_);
  }
  DeviceGuard(const DeviceGuard&) = delete;
  DeviceGuard& operator=(const DeviceGuard&) = delete;
  bool ok() const { return ok_; }

 private:
  int prev_;
  bool ok_ = false;
};
// doubles per global triangle in the mixed path's table of ray-independent
// FP64 terms (k_tri_prime in api.cu)
constexpr int kTriPrimeStride = 32;

// status codes (mirrors xdgcu.h)
enum : int32_t {
  RAY_OK = 0,
  RAY_INVALID = 1,
  RAY_STACK_OVERFLOW = 2,
  RAY_WALK_LIMIT = 4,
  RAY_NO_EXIT_FACE = 5,
  RAY_OUTPUT_FULL = 6,
  RAY_EVENT_LIMIT = 7,
  RAY_LOST = 8,
  RAY_STUCK = 9,
};

// work counters (xdgcu_get_counters)
enum : int {
  CNT_BOX = 0,
  CNT_NODE = 1,
  CNT_PRIM = 2,
  CNT_ESCALATE = 3,
  CNT_RAYS = 4,
  CNT_STEPS = 5,
  CNT_N = 8,
};

// inputs the engine accepts: finite, |x| < 2^300 (see geom.cuh)
__device__ __forceinline__ bool finite3(d3 a) {
  return sane_bits(a.x) && sane_bits(a.y) && sane_bits(a.z);
}

__device__ __forceinline__ d3 load3(const double* p, int64_t i) {
  return mk3(p[3 * i], p[3 * i + 1], p[3 * i + 2]);
}

}  // namespace xdgcu
