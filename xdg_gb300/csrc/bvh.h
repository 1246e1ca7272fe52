// bvh.h -- device BVH builder interface and a small device-memory holder.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>

#include "internal.cuh"

namespace xdgcu {

// RAII device allocation (build-time temporaries and context-owned arrays).
template <typename T>
struct DevMem {
  T* p = nullptr;
  int64_t n = 0;
  DevMem() = default;
  explicit DevMem(int64_t count) : n(count) {}
  DevMem(const DevMem&) = delete;
  DevMem& operator=(const DevMem&) = delete;
  DevMem(DevMem&& o) noexcept : p(o.p), n(o.n) {
    o.p = nullptr;
    o.n = 0;
  }
  DevMem& operator=(DevMem&& o) noexcept {
    if (this != &o) {
      reset();
      p = o.p;
      n = o.n;
      o.p = nullptr;
      o.n = 0;
    }
    return *this;
  }
  ~DevMem() { reset(); }
  cudaError_t alloc() {
    if (p) return cudaSuccess;
    if (n <= 0) return cudaSuccess;
    return cudaMalloc(&p, sizeof(T) * (size_t)n);
  }
  cudaError_t alloc(int64_t count) {
    reset();
    n = count;
    return alloc();
  }
  void reset() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  size_t bytes() const { return sizeof(T) * (size_t)n; }
};

// Result of build_wide_bvh.  n32/n64/order are cudaMalloc'ed and owned by the
// caller afterwards.  order[j] = input primitive index at leaf position j.
struct BuiltTree {
  Node32* n32;
  Node64* n64;
  int32_t* order;
  int32_t n_nodes;
  int32_t depth;
  int32_t root;
  int32_t width;     // children per node: 4 (one record) or 8 (two records)
  double bounds[6];  // union of the primitive boxes
};

// Cost weights of the SAH collapse: a wide node visited (node) and a
// primitive tested (prim), per unit of surface area.
struct BvhCost {
  double node;
  double prim;
};

// d_boxes: 6 doubles per primitive (lo.xyz, hi.xyz), already dilated.
// sah_cost: collapse by the SAH (bvh.cu, step 6a), or nullptr for the greedy
// largest-area collapse (6b).
cudaError_t build_wide_bvh(const double* d_boxes, int32_t n, int32_t leaf_max, int32_t width,
                           const BvhCost* sah_cost, cudaStream_t st, BuiltTree* out);

}  // namespace xdgcu
