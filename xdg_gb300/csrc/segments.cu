// segments.cu -- kernels of the global track loop (segments.h).  The FP64
// operations follow xdg.cpp:142-198 with Vec3da's arithmetic (vec3da.h):
// component-wise sums, differences, products and quotients, each rounded once
// (-fmad=false).
#include <cuda_runtime.h>

#include <algorithm>

#include "internal.cuh"
#include "segments.h"

namespace xdgcu {

namespace {

constexpr int kSegBlock = 256;
constexpr double kTinyBit = 1e-10;  // TINY_BIT, constants.h:32

inline unsigned seg_grid(int64_t n) { return (unsigned)((n + kSegBlock - 1) / kSegBlock); }

__device__ __forceinline__ void store3(double* p, int64_t i, d3 v) {
  p[3 * i] = v.x;
  p[3 * i + 1] = v.y;
  p[3 * i + 2] = v.z;
}

// r + u * s, component by component (Vec3da operator+ and operator*)
__device__ __forceinline__ d3 advance3(d3 r, d3 u, double s) {
  return mk3(r.x + u.x * s, r.y + u.y * s, r.z + u.z * s);
}

__global__ void __launch_bounds__(kSegBlock) k_seg_init(SegState s, const double* __restrict__ starts,
                                                         const double* __restrict__ ends,
                                                         int32_t* __restrict__ act,
                                                         int32_t* __restrict__ n_act) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= s.n) return;
  const d3 a = load3(starts, t), b = load3(ends, t);
  s.written[t] = 0;
  s.last[t] = -1;
  s.status[t] = RAY_OK;
  s.stopped[t] = 0;
  s.paused[t] = 0;
  store3(s.r, t, a);
  if (!finite3(a) || !finite3(b)) {
    s.status[t] = RAY_INVALID;
    s.stopped[t] = 1;
    s.dist[t] = 0.0;
    store3(s.u, t, mk3(0.0, 0.0, 0.0));
    return;
  }
  // Direction u = end - start; double distance = u.length(); u /= distance;
  const d3 w = mk3(b.x - a.x, b.y - a.y, b.z - a.z);
  const double len = sqrt(w.x * w.x + w.y * w.y + w.z * w.z);
  s.dist[t] = len;
  if (!gt0(len)) {  // while (distance > 0) never runs
    s.stopped[t] = 1;
    store3(s.u, t, mk3(0.0, 0.0, 0.0));
    return;
  }
  store3(s.u, t, mk3(w.x / len, w.y / len, w.z / len));
  act[atomicAdd(n_act, 1)] = (int32_t)t;
}

// walk_elements of every track in rounds (the packed walk): each track starts
// as a walk paused at its start element, position and distance.
__global__ void __launch_bounds__(kSegBlock) k_seg_walk_init(SegState s, const int32_t* __restrict__ start,
                                                              const double* __restrict__ org,
                                                              const double* __restrict__ dir,
                                                              const double* __restrict__ dist,
                                                              int32_t* __restrict__ act) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= s.n) return;
  s.written[t] = 0;
  s.last[t] = -1;
  s.status[t] = RAY_OK;
  s.stopped[t] = 0;
  s.paused[t] = 1;
  s.welem[t] = start[t];
  store3(s.wr, t, load3(org, t));
  store3(s.u, t, load3(dir, t));
  s.wd[t] = dist[t];
  s.wsum[t] = 0.0;
  s.wcount[t] = 0;
  act[t] = (int32_t)t;
}

// A new walk of track t from its current r and distance (xdg.cpp:187).
__device__ __forceinline__ void start_walk(const SegState& s, int32_t t) {
  store3(s.wr, t, load3(s.r, t));
  s.wd[t] = s.dist[t];
  s.wsum[t] = 0.0;
  s.wcount[t] = 0;
}

__global__ void __launch_bounds__(kSegBlock) k_seg_split(SegState s, const int32_t* __restrict__ act,
                                                          int64_t m, int32_t* __restrict__ walk_t,
                                                          int32_t* __restrict__ walk_start,
                                                          int32_t* __restrict__ n_walk,
                                                          int32_t* __restrict__ loc,
                                                          int32_t* __restrict__ n_loc) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= m) return;
  const int32_t t = act[k];
  if (s.paused[t]) {
    const int32_t w = atomicAdd(n_walk, 1);
    walk_t[w] = t;
    walk_start[w] = s.welem[t];
  } else {
    loc[atomicAdd(n_loc, 1)] = t;
  }
}

__global__ void __launch_bounds__(kSegBlock) k_seg_gather_points(SegState s,
                                                                  const int32_t* __restrict__ act,
                                                                  int64_t m, double* __restrict__ pts) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= m) return;
  store3(pts, k, load3(s.r, act[k]));
}

__global__ void __launch_bounds__(kSegBlock) k_seg_decide(
    SegState s, const int32_t* __restrict__ act, int64_t m, const int32_t* __restrict__ eid,
    const int32_t* __restrict__ eidx, int32_t* __restrict__ walk_t, int32_t* __restrict__ walk_start,
    int32_t* __restrict__ n_walk, int32_t* __restrict__ out_t, double* __restrict__ ray_org,
    double* __restrict__ ray_dir, int32_t* __restrict__ n_out) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= m) return;
  const int32_t t = act[k];
  int32_t cur = eidx[k];
  // on the face of the element just walked: not inside it (xdg.cpp:161-162)
  if (s.written[t] > 0 && eid[k] == s.last[t]) cur = -1;
  if (cur >= 0) {
    start_walk(s, t);
    const int32_t w = atomicAdd(n_walk, 1);
    walk_t[w] = t;
    walk_start[w] = cur;
    return;
  }
  // ray_fire(ipc, r + u * TINY_BIT, u, INFTY, EXITING, &hit_primitives)
  const d3 r = load3(s.r, t), u = load3(s.u, t);
  const int32_t o = atomicAdd(n_out, 1);
  out_t[o] = t;
  store3(ray_org, o, advance3(r, u, kTinyBit));
  store3(ray_dir, o, u);
}

// get_boundary_face_element(face): binary search of the ascending face ids
__device__ __forceinline__ int32_t boundary_element(const int32_t* __restrict__ faces,
                                                    const int32_t* __restrict__ elems, int64_t n,
                                                    int32_t face) {
  int64_t lo = 0, hi = n;
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (faces[mid] < face) lo = mid + 1;
    else hi = mid;
  }
  return (lo < n && faces[lo] == face) ? elems[lo] : -1;
}

__global__ void __launch_bounds__(kSegBlock) k_seg_reenter(
    SegState s, const int32_t* __restrict__ out_t, int64_t m, const double* __restrict__ t_hit,
    const int32_t* __restrict__ surf, const int32_t* __restrict__ face,
    const int32_t* __restrict__ bfe_face, const int32_t* __restrict__ bfe_elem, int64_t n_bfe,
    int32_t n_tets, int32_t* __restrict__ walk_t, int32_t* __restrict__ walk_start,
    int32_t* __restrict__ n_walk) {
  const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (j >= m) return;
  const int32_t t = out_t[j];
  const double dist = s.dist[t];
  // if (hit.second == ID_NONE || hit.first > distance) return segments;
  if (surf[j] < 0 || dlt(dist, t_hit[j])) {
    s.stopped[t] = 1;
    return;
  }
  // double hit_dist = hit.first + TINY_BIT; r += u * hit_dist; distance -= hit_dist;
  const double hd = t_hit[j] + kTinyBit;
  store3(s.r, t, advance3(load3(s.r, t), load3(s.u, t), hd));
  s.dist[t] = dist - hd;
  const int32_t e = n_bfe > 0 ? boundary_element(bfe_face, bfe_elem, n_bfe, face[j]) : -1;
  if (e < 0 || e >= n_tets) {  // no element behind the hit face: return segments
    s.stopped[t] = 1;
    return;
  }
  start_walk(s, t);
  const int32_t w = atomicAdd(n_walk, 1);
  walk_t[w] = t;
  walk_start[w] = e;
}

__global__ void __launch_bounds__(kSegBlock) k_seg_walk_inputs(SegState s,
                                                                const int32_t* __restrict__ walk_t,
                                                                int64_t m, double* __restrict__ wr,
                                                                double* __restrict__ wu,
                                                                double* __restrict__ wd,
                                                                double* __restrict__ wsum) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= m) return;
  const int32_t t = walk_t[k];
  store3(wr, k, load3(s.wr, t));
  store3(wu, k, load3(s.u, t));
  wd[k] = s.wd[t];
  wsum[k] = s.wsum[t];
}

__global__ void __launch_bounds__(kSegBlock) k_seg_round_counts(SegState s,
                                                                 const int32_t* __restrict__ walk_t,
                                                                 int64_t m,
                                                                 const int32_t* __restrict__ cnt,
                                                                 int32_t max_segs,
                                                                 int64_t* __restrict__ off) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= m) return;
  const int32_t left = max(0, max_segs - s.wcount[walk_t[k]]);
  off[k] = min(cnt[k], left);
}

// Warp-per-row copy: row k's kept entries, read from the K-strided buffer and
// written contiguously, 32 at a time.
__global__ void __launch_bounds__(kSegBlock) k_seg_pack(int64_t m, int32_t K,
                                                         const int32_t* __restrict__ seg_elem,
                                                         const double* __restrict__ seg_len,
                                                         const int64_t* __restrict__ off,
                                                         int32_t* __restrict__ out_elem,
                                                         double* __restrict__ out_len) {
  const int lane = threadIdx.x & 31;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t k = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; k < m; k += nw) {
    const int64_t o = off[k], kept = off[k + 1] - o;
    const int32_t* se = seg_elem + k * (int64_t)K;
    const double* sl = seg_len + k * (int64_t)K;
    for (int64_t q = lane; q < kept; q += 32) {
      out_elem[o + q] = se[q];
      out_len[o + q] = sl[q];
    }
  }
}

__global__ void __launch_bounds__(kSegBlock) k_seg_advance(
    SegState s, const int32_t* __restrict__ walk_t, int64_t m, int32_t K,
    const int32_t* __restrict__ seg_elem, const int32_t* __restrict__ cnt,
    const int32_t* __restrict__ wst, const int32_t* __restrict__ wstop,
    const double* __restrict__ wend_r, const double* __restrict__ wend_d,
    const double* __restrict__ wsum, int32_t max_segs, const int64_t* __restrict__ off,
    int64_t* __restrict__ dst_rel, int32_t* __restrict__ act_next, int32_t* __restrict__ n_act,
    int walk_only) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= m) return;
  const int32_t t = walk_t[k];
  const int64_t kept = off[k + 1] - off[k];
  // std::accumulate(vol_segments, 0.0, ...) continued across pauses: the walk
  // kernel added this round's lengths, in order, to the sum it was given
  const double sum = wsum[k];
  dst_rel[k] = s.written[t];
  s.written[t] += kept;
  if (kept > 0) s.last[t] = seg_elem[k * (int64_t)K + kept - 1];
  const int32_t wc = s.wcount[t] + (int32_t)kept;
  s.wcount[t] = wc;
  const int32_t st = wst[k];
  if (kept < cnt[k] || (st == RAY_WALK_LIMIT && wc >= max_segs)) {
    // the walk passes max_segs segments: the track stops there
    if (s.status[t] == RAY_OK) s.status[t] = RAY_WALK_LIMIT;
    s.stopped[t] = 1;
    s.paused[t] = 0;
    return;
  }
  if (st == RAY_WALK_LIMIT) {  // paused at K segments: resumes next round
    // where the walk's own steps left it (distance -= len, r += len * u)
    store3(s.wr, t, load3(wend_r, k));
    s.wd[t] = wend_d[k];
    s.wsum[t] = sum;
    s.welem[t] = wstop[k];
    s.paused[t] = 1;
    act_next[atomicAdd(n_act, 1)] = t;
    return;
  }
  s.paused[t] = 0;
  if (walk_only) {  // the packed walk: the track's walk_elements is done
    if (st != RAY_OK && s.status[t] == RAY_OK) s.status[t] = st;
    s.stopped[t] = 1;
    return;
  }
  // the walk has ended: r += u * segment_sum; distance -= segment_sum;
  const d3 u = load3(s.u, t);
  store3(s.r, t, advance3(load3(s.r, t), u, sum));
  const double dist = s.dist[t] - sum;
  s.dist[t] = dist;
  if (st != RAY_OK) {
    if (s.status[t] == RAY_OK) s.status[t] = st;
    // a walk that found no exit face ended as the reference's does; invalid
    // data does not go on
    if (st != RAY_NO_EXIT_FACE) {
      s.stopped[t] = 1;
      return;
    }
  }
  if (gt0(dist)) act_next[atomicAdd(n_act, 1)] = t;  // while (distance > 0)
}

__global__ void __launch_bounds__(kSegBlock) k_seg_stop_active(SegState s,
                                                                const int32_t* __restrict__ act,
                                                                int64_t m, int32_t code) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= m) return;
  const int32_t t = act[k];
  s.stopped[t] = 1;
  if (s.status[t] == RAY_OK) s.status[t] = code;
}

__global__ void __launch_bounds__(kSegBlock) k_seg_counts(SegState s, int64_t* __restrict__ offsets) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= s.n) return;
  offsets[t] = s.written[t];
}

__global__ void __launch_bounds__(kSegBlock) k_seg_mark_full(SegState s,
                                                              const int64_t* __restrict__ offsets,
                                                              int64_t capacity) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= s.n) return;
  if (offsets[t + 1] > capacity && offsets[t + 1] > offsets[t] && s.status[t] == RAY_OK)
    s.status[t] = RAY_OUTPUT_FULL;
}

__global__ void __launch_bounds__(kSegBlock) k_seg_scatter(
    const int32_t* __restrict__ walk_t, int64_t m, const int64_t* __restrict__ off,
    const int64_t* __restrict__ dst_rel, const int32_t* __restrict__ seg_elem,
    const double* __restrict__ seg_len, const int64_t* __restrict__ offsets, int64_t capacity,
    int32_t* __restrict__ out_elem, double* __restrict__ out_len) {
  const int lane = threadIdx.x & 31;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t k = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; k < m; k += nw) {
    const int32_t t = walk_t[k];
    if (offsets[t + 1] > capacity) continue;  // the track does not fit: nothing is written
    const int64_t o0 = off[k], o1 = off[k + 1];
    const int64_t d = offsets[t] + dst_rel[k] - o0;
    for (int64_t q = o0 + lane; q < o1; q += 32) {
      out_elem[d + q] = seg_elem[q];
      out_len[d + q] = seg_len[q];
    }
  }
}

// grid of the warp-per-row kernels: a few blocks per SM, rows strided
inline unsigned seg_warp_grid(int64_t rows) {
  const int64_t need = (rows + kSegBlock / 32 - 1) / (kSegBlock / 32);
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(need, (int64_t)device_sm_count() * 8));
}

}  // namespace

cudaError_t seg_init(const SegState& s, const double* starts, const double* ends, int32_t* act,
                     int32_t* n_act, cudaStream_t st) {
  if (s.n <= 0) return cudaSuccess;
  k_seg_init<<<seg_grid(s.n), kSegBlock, 0, st>>>(s, starts, ends, act, n_act);
  return cudaGetLastError();
}

cudaError_t seg_walk_init(const SegState& s, const int32_t* start, const double* org,
                          const double* dir, const double* dist, int32_t* act, cudaStream_t st) {
  if (s.n <= 0) return cudaSuccess;
  k_seg_walk_init<<<seg_grid(s.n), kSegBlock, 0, st>>>(s, start, org, dir, dist, act);
  return cudaGetLastError();
}

cudaError_t seg_split(const SegState& s, const int32_t* act, int64_t m, int32_t* walk_t,
                      int32_t* walk_start, int32_t* n_walk, int32_t* loc, int32_t* n_loc,
                      cudaStream_t st) {
  if (m <= 0) return cudaSuccess;
  k_seg_split<<<seg_grid(m), kSegBlock, 0, st>>>(s, act, m, walk_t, walk_start, n_walk, loc, n_loc);
  return cudaGetLastError();
}

cudaError_t seg_round_counts(const SegState& s, const int32_t* walk_t, int64_t m,
                             const int32_t* cnt, int32_t max_segs, int64_t* off, cudaStream_t st) {
  if (m <= 0) return cudaSuccess;
  k_seg_round_counts<<<seg_grid(m), kSegBlock, 0, st>>>(s, walk_t, m, cnt, max_segs, off);
  return cudaGetLastError();
}

cudaError_t seg_gather_points(const SegState& s, const int32_t* act, int64_t m, double* pts,
                              cudaStream_t st) {
  if (m <= 0) return cudaSuccess;
  k_seg_gather_points<<<seg_grid(m), kSegBlock, 0, st>>>(s, act, m, pts);
  return cudaGetLastError();
}

cudaError_t seg_decide(const SegState& s, const int32_t* act, int64_t m, const int32_t* eid,
                       const int32_t* eidx, int32_t* walk_t, int32_t* walk_start,
                       int32_t* n_walk, int32_t* out_t, double* ray_org, double* ray_dir,
                       int32_t* n_out, cudaStream_t st) {
  if (m <= 0) return cudaSuccess;
  k_seg_decide<<<seg_grid(m), kSegBlock, 0, st>>>(s, act, m, eid, eidx, walk_t, walk_start, n_walk,
                                                   out_t, ray_org, ray_dir, n_out);
  return cudaGetLastError();
}

cudaError_t seg_reenter(const SegState& s, const int32_t* out_t, int64_t m, const double* t_hit,
                        const int32_t* surf, const int32_t* face, const int32_t* bfe_face,
                        const int32_t* bfe_elem, int64_t n_bfe, int32_t n_tets, int32_t* walk_t,
                        int32_t* walk_start, int32_t* n_walk, cudaStream_t st) {
  if (m <= 0) return cudaSuccess;
  k_seg_reenter<<<seg_grid(m), kSegBlock, 0, st>>>(s, out_t, m, t_hit, surf, face, bfe_face,
                                                    bfe_elem, n_bfe, n_tets, walk_t, walk_start,
                                                    n_walk);
  return cudaGetLastError();
}

cudaError_t seg_walk_inputs(const SegState& s, const int32_t* walk_t, int64_t m, double* wr,
                            double* wu, double* wd, double* wsum, cudaStream_t st) {
  if (m <= 0) return cudaSuccess;
  k_seg_walk_inputs<<<seg_grid(m), kSegBlock, 0, st>>>(s, walk_t, m, wr, wu, wd, wsum);
  return cudaGetLastError();
}

cudaError_t seg_pack(int64_t m, int32_t K, const int32_t* seg_elem, const double* seg_len,
                     const int64_t* off, int32_t* out_elem, double* out_len, cudaStream_t st) {
  if (m <= 0) return cudaSuccess;
  k_seg_pack<<<seg_warp_grid(m), kSegBlock, 0, st>>>(m, K, seg_elem, seg_len, off, out_elem,
                                                      out_len);
  return cudaGetLastError();
}

cudaError_t seg_advance(const SegState& s, const int32_t* walk_t, int64_t m, int32_t K,
                        const int32_t* seg_elem, const int32_t* cnt, const int32_t* wst,
                        const int32_t* wstop, const double* wend_r, const double* wend_d,
                        const double* wsum, int32_t max_segs, const int64_t* off,
                        int64_t* dst_rel, int32_t* act_next, int32_t* n_act, cudaStream_t st,
                        bool walk_only) {
  if (m <= 0) return cudaSuccess;
  k_seg_advance<<<seg_grid(m), kSegBlock, 0, st>>>(s, walk_t, m, K, seg_elem, cnt, wst, wstop,
                                                    wend_r, wend_d, wsum, max_segs, off, dst_rel,
                                                    act_next, n_act, walk_only ? 1 : 0);
  return cudaGetLastError();
}

cudaError_t seg_stop_active(const SegState& s, const int32_t* act, int64_t m, int32_t code,
                            cudaStream_t st) {
  if (m <= 0) return cudaSuccess;
  k_seg_stop_active<<<seg_grid(m), kSegBlock, 0, st>>>(s, act, m, code);
  return cudaGetLastError();
}

cudaError_t seg_counts(const SegState& s, int64_t* offsets, cudaStream_t st) {
  if (s.n <= 0) return cudaSuccess;
  k_seg_counts<<<seg_grid(s.n), kSegBlock, 0, st>>>(s, offsets);
  return cudaGetLastError();
}

cudaError_t seg_mark_full(const SegState& s, const int64_t* offsets, int64_t capacity,
                          cudaStream_t st) {
  if (s.n <= 0) return cudaSuccess;
  k_seg_mark_full<<<seg_grid(s.n), kSegBlock, 0, st>>>(s, offsets, capacity);
  return cudaGetLastError();
}

cudaError_t seg_scatter(const SegState& s, const int32_t* walk_t, int64_t m, const int64_t* off,
                        const int64_t* dst_rel, const int32_t* seg_elem, const double* seg_len,
                        const int64_t* offsets, int64_t capacity, int32_t* out_elem,
                        double* out_len, cudaStream_t st) {
  (void)s;
  if (m <= 0) return cudaSuccess;
  k_seg_scatter<<<seg_warp_grid(m), kSegBlock, 0, st>>>(walk_t, m, off, dst_rel, seg_elem, seg_len,
                                                    offsets, capacity, out_elem, out_len);
  return cudaGetLastError();
}

}  // namespace xdgcu
