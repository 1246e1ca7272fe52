// tune.cu -- autotuner for the launch parameters of the traversal and walk
// kernels (no counterpart in the reference, whose Embree backend has none).
//
// The tuner runs the caller's sample batch (device arrays) through the public
// entry points under different settings of the context's tuning keys and
// keeps the fastest.  It searches one key at a time (coordinate descent, at
// most three passes, stopping when a pass changes nothing), timing each
// setting as the median of `reps` launches after one untimed launch, with
// CUDA events on a private stream.
//
// With tune_tree the search runs once per tree shape -- node width 4 or 8,
// leaf size 2, 3 or 4 -- the surface trees rebuilt for each, and the fastest
// shape is kept.
//
// Every setting must give the same results: the tuner compares each run's
// outputs byte for byte with the first run's and fails with XDGCU_ERR_STATE
// if they differ.  The one accepted difference is a smaller stack that makes
// rays overflow (XDGCU_RAY_STACK_OVERFLOW): such a setting is skipped.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

#include "xdgcu.h"
#include "internal.cuh"

namespace xdgcu {
int set_last_error(int code, const char* msg);
int ctx_device(const xdgcu_ctx* c);
}

namespace {

using xdgcu::set_last_error;

struct Buf {
  void* p = nullptr;
  size_t bytes = 0;
  ~Buf() {
    if (p) cudaFree(p);
  }
  cudaError_t alloc(size_t b) {
    bytes = b;
    return cudaMalloc(&p, std::max<size_t>(b, 16));
  }
};

struct Stream {
  cudaStream_t s = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  ~Stream() {
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (s) cudaStreamDestroy(s);
  }
  bool init() {
    return cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) == cudaSuccess &&
           cudaEventCreate(&e0) == cudaSuccess && cudaEventCreate(&e1) == cudaSuccess;
  }
};

bool all_device(std::initializer_list<const void*> ptrs) {
  for (const void* p : ptrs) {
    if (!p) continue;
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    if (at.type != cudaMemoryTypeDevice && at.type != cudaMemoryTypeManaged) return false;
  }
  return true;
}

struct Knob {
  const char* key;
  std::vector<int64_t> values;
};

// Times `run` (which enqueues one batch on st.s and returns an xdgcu status)
// as the median of reps launches after one untimed launch.
template <typename Run>
int time_median(Stream& st, int reps, Run run, double* ms) {
  int rc = run();
  if (rc) return rc;
  std::vector<float> t;
  for (int r = 0; r < reps; ++r) {
    if (cudaEventRecord(st.e0, st.s) != cudaSuccess) return set_last_error(XDGCU_ERR_CUDA, "event");
    rc = run();
    if (rc) return rc;
    if (cudaEventRecord(st.e1, st.s) != cudaSuccess) return set_last_error(XDGCU_ERR_CUDA, "event");
    if (cudaEventSynchronize(st.e1) != cudaSuccess)
      return set_last_error(XDGCU_ERR_CUDA, "autotune: launch failed");
    float x = 0.f;
    cudaEventElapsedTime(&x, st.e0, st.e1);
    t.push_back(x);
  }
  std::sort(t.begin(), t.end());
  *ms = t[t.size() / 2];
  return XDGCU_OK;
}

// Coordinate descent over `knobs`.  `measure` runs the sample under the
// context's current settings and returns its time, or a negative time when
// the setting is not admissible (stack overflow).
template <typename Measure>
int descend(xdgcu_ctx* c, const std::vector<Knob>& knobs, Measure measure, double* best_ms) {
  std::vector<int64_t> best(knobs.size());
  for (size_t k = 0; k < knobs.size(); ++k) {
    int rc = xdgcu_get_tuning(c, knobs[k].key, &best[k]);
    if (rc) return rc;
  }
  double cur = 0.0;
  int rc = measure(&cur);
  if (rc) return rc;
  if (cur < 0.0) return set_last_error(XDGCU_ERR_STATE, "autotune: the starting settings overflow");
  for (int pass = 0; pass < 3; ++pass) {
    bool changed = false;
    for (size_t k = 0; k < knobs.size(); ++k) {
      for (int64_t v : knobs[k].values) {
        if (v == best[k]) continue;
        rc = xdgcu_set_tuning(c, knobs[k].key, v);
        if (rc) return rc;
        double ms = 0.0;
        rc = measure(&ms);
        if (rc) {
          xdgcu_set_tuning(c, knobs[k].key, best[k]);
          return rc;
        }
        // a new setting must win by 1% to replace the current one
        if (ms >= 0.0 && ms < 0.99 * cur) {
          cur = ms;
          best[k] = v;
          changed = true;
        }
      }
      rc = xdgcu_set_tuning(c, knobs[k].key, best[k]);
      if (rc) return rc;
    }
    if (!changed) break;
  }
  if (best_ms) *best_ms = cur;
  return XDGCU_OK;
}

// compares the outputs of a run with the reference copy; returns 1 when equal,
// 0 when they differ only on rays that overflowed the stack, -1 otherwise
int compare(const std::vector<std::vector<char>>& ref, const std::vector<Buf*>& bufs,
            const Buf& status, const std::vector<int32_t>& ref_status, size_t n) {
  std::vector<int32_t> st(n);
  cudaMemcpy(st.data(), status.p, sizeof(int32_t) * n, cudaMemcpyDeviceToHost);
  bool overflow = false;
  for (size_t i = 0; i < n; ++i)
    if (st[i] != ref_status[i]) {
      if (st[i] == XDGCU_RAY_STACK_OVERFLOW) overflow = true;
      else return -1;
    }
  if (overflow) return 0;
  std::vector<char> h;
  for (size_t k = 0; k < bufs.size(); ++k) {
    h.resize(bufs[k]->bytes);
    cudaMemcpy(h.data(), bufs[k]->p, bufs[k]->bytes, cudaMemcpyDeviceToHost);
    if (std::memcmp(h.data(), ref[k].data(), h.size()) != 0) return -1;
  }
  return 1;
}

}  // namespace

extern "C" {

int xdgcu_autotune_trace(xdgcu_ctx* c, int32_t query, int32_t tree, const int32_t* ray_trees,
                         int64_t n, const double* origins, const double* directions,
                         int32_t precision, int32_t reps, int32_t tune_tree, double* best_ms) {
  if (!c) return set_last_error(XDGCU_ERR_INVALID_ARG, "null context");
  xdgcu::DeviceGuard guard(xdgcu::ctx_device(c));
  if (!guard.ok()) return set_last_error(XDGCU_ERR_CUDA, "cudaSetDevice failed");
  if (query < XDGCU_QUERY_RAY_FIRE || query > XDGCU_QUERY_FIND_VOLUME)
    return set_last_error(XDGCU_ERR_INVALID_ARG, "autotune: unknown query");
  if (n <= 0 || !origins || (!directions && query != XDGCU_QUERY_POINT_IN_VOLUME &&
                             query != XDGCU_QUERY_FIND_VOLUME))
    return set_last_error(XDGCU_ERR_INVALID_ARG, "autotune: empty sample or null inputs");
  if (precision != XDGCU_FP64 && precision != XDGCU_MIXED)
    return set_last_error(XDGCU_ERR_INVALID_ARG, "precision must be XDGCU_FP64 or XDGCU_MIXED");
  if (!all_device({ray_trees, origins, directions}))
    return set_last_error(XDGCU_ERR_INVALID_ARG, "autotune: the sample must be in device memory");
  reps = std::max(1, std::min(reps, 50));
  Stream st;
  if (!st.init()) return set_last_error(XDGCU_ERR_CUDA, "autotune: stream creation failed");
  Buf t, s, f, flag, stat;
  const size_t un = (size_t)n;
  if (t.alloc(8 * un) || s.alloc(4 * un) || f.alloc(4 * un) || flag.alloc(4 * un) ||
      stat.alloc(4 * un))
    return set_last_error(XDGCU_ERR_OUT_OF_MEMORY, "autotune: output buffers");
  std::vector<Buf*> outs;
  if (query == XDGCU_QUERY_RAY_FIRE) outs = {&t, &s, &f};
  else if (query == XDGCU_QUERY_OCCLUDED) outs = {&flag, &t};
  else outs = {&flag};
  auto run = [&]() -> int {
    switch (query) {
      case XDGCU_QUERY_RAY_FIRE:
        return xdgcu_ray_fire(c, tree, ray_trees, n, origins, directions, nullptr, XDGCU_EXITING,
                              nullptr, nullptr, (double*)t.p, (int32_t*)s.p, (int32_t*)f.p,
                              (int32_t*)stat.p, precision, st.s);
      case XDGCU_QUERY_POINT_IN_VOLUME:
        return xdgcu_point_in_volume(c, tree, ray_trees, n, origins, directions, nullptr, nullptr,
                                     (int32_t*)flag.p, (int32_t*)stat.p, precision, st.s);
      case XDGCU_QUERY_OCCLUDED:
        return xdgcu_occluded(c, tree, ray_trees, n, origins, directions, (int32_t*)flag.p,
                              (double*)t.p, (int32_t*)stat.p, precision, st.s);
      default:
        return xdgcu_find_volume(c, n, origins, directions, (int32_t*)flag.p, (int32_t*)stat.p,
                                 precision, st.s);
    }
  };
  std::vector<std::vector<char>> ref;
  std::vector<int32_t> ref_status;
  auto measure = [&](double* ms) -> int {
    int rc = time_median(st, reps, run, ms);
    if (rc) return rc;
    if (ref.empty()) {
      for (Buf* b : outs) {
        ref.emplace_back(b->bytes);
        cudaMemcpy(ref.back().data(), b->p, b->bytes, cudaMemcpyDeviceToHost);
      }
      ref_status.resize(un);
      cudaMemcpy(ref_status.data(), stat.p, 4 * un, cudaMemcpyDeviceToHost);
      return XDGCU_OK;
    }
    const int eq = compare(ref, outs, stat, ref_status, un);
    if (eq < 0)
      return set_last_error(XDGCU_ERR_STATE,
                            "autotune: results differ between launch settings");
    if (eq == 0) *ms = -1.0;
    return XDGCU_OK;
  };
  const bool mixed = precision == XDGCU_MIXED;
  std::vector<Knob> knobs = {
      {"trace_occupancy", {2, 3, 4}},
      {"trace_stack", {32, 40, 48, 64}},
      {mixed ? "trace_node_iters" : "trace_node_iters_fp64", {1, 2, 4, 8, 16}},
      {"trace_flush_wait", {4, 8, 16, 32}},
      {"trace_grab", {0, 64, 256, 1024, 4096}},
  };
  if (n >= 65536) knobs.push_back({"trace_sort_min", {0, n}});
  // tree shapes: the current one first, then (tune_tree) every node width
  // and leaf size; each shape rebuilds the surface trees
  int64_t w0 = 4, l0 = 4;
  int rc = xdgcu_get_tuning(c, "node_width", &w0);
  if (!rc) rc = xdgcu_get_tuning(c, "leaf_max", &l0);
  if (rc) return rc;
  std::vector<std::pair<int64_t, int64_t>> shapes = {{w0, l0}};
  if (tune_tree)
    for (int64_t w : {4, 8})
      for (int64_t l : {2, 3, 4})
        if (!(w == w0 && l == l0)) shapes.push_back({w, l});
  double best = -1.0;
  std::pair<int64_t, int64_t> best_shape = shapes[0], cur_shape = shapes[0];
  std::vector<int64_t> best_vals(knobs.size());
  for (const auto& sh : shapes) {
    if (sh != cur_shape) {
      rc = xdgcu_set_tuning(c, "node_width", sh.first);
      if (!rc) rc = xdgcu_set_tuning(c, "leaf_max", sh.second);
      if (!rc) rc = xdgcu_rebuild_trees(c, 1);
      if (rc) return rc;
      cur_shape = sh;
    }
    double ms = 0.0;
    rc = descend(c, knobs, measure, &ms);
    if (rc) return rc;
    if (best < 0.0 || ms < 0.99 * best) {
      best = ms;
      best_shape = sh;
      for (size_t k = 0; k < knobs.size(); ++k) xdgcu_get_tuning(c, knobs[k].key, &best_vals[k]);
    }
  }
  if (best_shape != cur_shape) {
    rc = xdgcu_set_tuning(c, "node_width", best_shape.first);
    if (!rc) rc = xdgcu_set_tuning(c, "leaf_max", best_shape.second);
    if (!rc) rc = xdgcu_rebuild_trees(c, 1);
    if (rc) return rc;
  }
  for (size_t k = 0; k < knobs.size(); ++k) xdgcu_set_tuning(c, knobs[k].key, best_vals[k]);
  if (best_ms) *best_ms = best;
  // a coherent order that paid off on this sample is kept for batches of at
  // least a quarter of its size (and never below 65,536 rays)
  int64_t sm = 0;
  xdgcu_get_tuning(c, "trace_sort_min", &sm);
  if (sm > 0) xdgcu_set_tuning(c, "trace_sort_min", std::max<int64_t>(65536, n / 4));
  return XDGCU_OK;
}

int xdgcu_autotune_walk(xdgcu_ctx* c, int64_t n, const int32_t* start_index, const double* start,
                        const double* u, const double* distance, int32_t max_segs,
                        int32_t precision, int32_t reps, double* best_ms) {
  if (!c) return set_last_error(XDGCU_ERR_INVALID_ARG, "null context");
  xdgcu::DeviceGuard guard(xdgcu::ctx_device(c));
  if (!guard.ok()) return set_last_error(XDGCU_ERR_CUDA, "cudaSetDevice failed");
  if (n <= 0 || !start_index || !start || !u || !distance || max_segs <= 0)
    return set_last_error(XDGCU_ERR_INVALID_ARG, "autotune: empty sample or bad arguments");
  if (precision != XDGCU_FP64 && precision != XDGCU_MIXED)
    return set_last_error(XDGCU_ERR_INVALID_ARG, "precision must be XDGCU_FP64 or XDGCU_MIXED");
  if (!all_device({start_index, start, u, distance}))
    return set_last_error(XDGCU_ERR_INVALID_ARG, "autotune: the sample must be in device memory");
  reps = std::max(1, std::min(reps, 50));
  Stream st;
  if (!st.init()) return set_last_error(XDGCU_ERR_CUDA, "autotune: stream creation failed");
  Buf e, l, cnt, stat;
  const size_t un = (size_t)n, cap = un * (size_t)max_segs;
  if (e.alloc(4 * cap) || l.alloc(8 * cap) || cnt.alloc(4 * un) || stat.alloc(4 * un))
    return set_last_error(XDGCU_ERR_OUT_OF_MEMORY, "autotune: output buffers");
  // entries past a track's count are never written: start from zeros
  cudaMemset(e.p, 0, e.bytes);
  cudaMemset(l.p, 0, l.bytes);
  auto run = [&]() -> int {
    return xdgcu_walk_elements(c, n, start_index, start, u, distance, max_segs, (int32_t*)e.p,
                               (double*)l.p, (int32_t*)cnt.p, (int32_t*)stat.p, precision, st.s);
  };
  std::vector<Buf*> outs = {&e, &l, &cnt};
  std::vector<std::vector<char>> ref;
  std::vector<int32_t> ref_status;
  auto measure = [&](double* ms) -> int {
    int rc = time_median(st, reps, run, ms);
    if (rc) return rc;
    if (ref.empty()) {
      for (Buf* b : outs) {
        ref.emplace_back(b->bytes);
        cudaMemcpy(ref.back().data(), b->p, b->bytes, cudaMemcpyDeviceToHost);
      }
      ref_status.resize(un);
      cudaMemcpy(ref_status.data(), stat.p, 4 * un, cudaMemcpyDeviceToHost);
      return XDGCU_OK;
    }
    if (compare(ref, outs, stat, ref_status, un) != 1)
      return set_last_error(XDGCU_ERR_STATE, "autotune: results differ between launch settings");
    return XDGCU_OK;
  };
  std::vector<Knob> knobs;
  if (precision == XDGCU_MIXED) knobs.push_back({"walk_queue", {0, 1}});
  knobs.push_back({"walk_flush_wait", {4, 8, 16, 32}});
  if (n >= 16384) knobs.push_back({"walk_sort_min", {0, n}});
  int rc = descend(c, knobs, measure, best_ms);
  if (rc) return rc;
  int64_t sm = 0;
  xdgcu_get_tuning(c, "walk_sort_min", &sm);
  if (sm > 0) xdgcu_set_tuning(c, "walk_sort_min", std::max<int64_t>(16384, n / 4));
  return XDGCU_OK;
}

}  // extern "C"
