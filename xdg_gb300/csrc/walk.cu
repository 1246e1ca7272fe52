// walk.cu -- face-adjacency tet walk (MeshManager::next_element /
// walk_elements, mesh_manager_interface.cpp:106-200) on the GPU.
//
// One thread walks one track.  Each step tests the four faces of the current
// tet for an exiting Plucker hit (orientation +1, plucker.h:64-161), takes
// the nearest (strict <, lowest face index on ties, :186-196), emits
// (element id, min(exit, remaining)) -- zero-length segments included -- and
// moves r += len * u in FP64, exactly like :117-133.
//
// The FP64 variant evaluates all four faces with plucker64.  The mixed
// variant first evaluates the six edge coordinates of the tet once in FP32
// (each face uses three of them, with a sign flip when it runs an edge
// backwards -- the exact coordinates of opposite directions are exact
// negatives) and skips a face only when some coordinate is certainly
// positive, which makes the FP64 test exit early (plucker.h:83-113).  The
// remaining faces -- normally just the exit face -- are evaluated with
// plucker64, so lengths and element sequences are bit-identical.
//
// FP32 bound for a tet (u = 2^-24, D = |u|_inf, W = max |v_k - r|_inf,
// Av = max |v_k|_inf, A = Av + |r|_inf; vertices and r rounded to FP32
// individually, edges e = v_b - v_a so |e| <= 2W):
//    |pip32 - pip| <= u D W (97 W + 13 Av + 13 A)
// (gamma_5 rounding of the triple product plus the input perturbations; the
// FP64 evaluation error and the 20*DBL_EPSILON snap are added as in geom.cuh).
#include "walk.h"

#include <atomic>

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include "internal.cuh"
#include "sample.cuh"

namespace xdgcu {

namespace {

constexpr int kBlock = 128;
constexpr float kU32 = 5.9604645e-08f;

// MOAB canonical face order (moab/direct_access.h:181-183)
__device__ __forceinline__ constexpr int moab_face(int f, int j) {
  return (f == 0) ? (j == 0 ? 0 : (j == 1 ? 1 : 3))
         : (f == 1) ? (j == 0 ? 1 : (j == 1 ? 2 : 3))
         : (f == 2) ? (j == 0 ? 2 : (j == 1 ? 0 : 3))
                    : (j == 0 ? 0 : (j == 1 ? 2 : 1));
}

template <int FO>
__device__ __forceinline__ int face_local(const WalkArgs& a, int f, int j) {
  if (FO == 0) return moab_face(f, j);
  return a.face[3 * f + j];
}

template <typename T>
__device__ __forceinline__ T sel4(const T* v, int k) {
  return k == 0 ? v[0] : (k == 1 ? v[1] : (k == 2 ? v[2] : v[3]));
}

__device__ __forceinline__ float sel6(const float* v, int k) {
  return k == 0 ? v[0]
                : (k == 1 ? v[1] : (k == 2 ? v[2] : (k == 3 ? v[3] : (k == 4 ? v[4] : v[5]))));
}

__device__ __forceinline__ float triple32(float dx, float dy, float dz, float ex, float ey,
                                          float ez, float wx, float wy, float wz) {
  const float cx = ey * wz - ez * wy;
  const float cy = ez * wx - ex * wz;
  const float cz = ex * wy - ey * wx;
  return dx * cx + dy * cy + dz * cz;
}

// index of the unordered vertex pair (i, j), i != j, in
// (0,1),(0,2),(0,3),(1,2),(1,3),(2,3)
__device__ __forceinline__ int pair_index(int i, int j) {
  const int a = i < j ? i : j, b = i < j ? j : i;
  return a == 0 ? b - 1 : (a == 1 ? b + 1 : 5);
}

struct StepCnt {
  unsigned long long steps, esc;
};

// plucker64 for the face (l0, l1, l2) of tet `tet` (vertex indices ci), its
// three edge coordinates taken from the mesh's edge table: the same values
// plucker_edge64 computes from the vertices, for a third of the FP64
// operations.  Only component plucker_axis(u) of the vertices is read.
__device__ __forceinline__ bool plucker64_face_pre(const WalkArgs& a, int32_t tet,
                                                   const int32_t ci[4], int l0, int l1, int l2,
                                                   d3 r, d3 u, d3 rn, double* t) {
  const int32_t* te = a.tet_edge + 6 * (int64_t)tet;
  auto coord = [&](int la, int lb) {
    const int32_t ref = __ldg(&te[pair_index(la, lb)]);
    // the test runs la -> lb; the reference keeps the sign when la's vertex
    // is the edge's lo (first(va, vb), plucker.h:48)
    const bool second_is_lo = ref < 0;
    const bool la_is_lo = second_is_lo == (la > lb);
    return plucker_edge_pre(a.edge + 6 * (int64_t)(ref & 0x7fffffff), !la_is_lo, u, rn);
  };
  const double c0 = coord(l0, l1), c1 = coord(l1, l2), c2 = coord(l2, l0);
  const int idx = plucker_axis(u);
  const double v0i = __ldg(&a.xyz[3 * (int64_t)sel4(ci, l0) + idx]);
  const double v1i = __ldg(&a.xyz[3 * (int64_t)sel4(ci, l1) + idx]);
  const double v2i = __ldg(&a.xyz[3 * (int64_t)sel4(ci, l2) + idx]);
  return plucker64_coords(c0, c1, c2, v0i, v1i, v2i, comp3(r, idx), comp3(u, idx), INFTY, 0.0,
                          true, 1, t);
}

// MeshManager::next_element for tet `elem` at r along u.  Returns the face
// index (or -1) and writes the exit distance.
template <int FO, bool MIXED>
__device__ __forceinline__ int next_face(const WalkArgs& a, int32_t elem, d3 r, d3 u,
                                         double* exit_dist, StepCnt& cnt) {
  const int4 c = __ldg(&a.conn[elem]);
  const int32_t ci[4] = {c.x, c.y, c.z, c.w};
  const d3 rn = cross3(u, r);  // plucker.h:75
  double dists[4];
  if (!MIXED) {
    d3 V[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) V[k] = load3(a.xyz, ci[k]);
#pragma unroll
    for (int f = 0; f < 4; ++f) {
      const d3 f0 = sel4(V, face_local<FO>(a, f, 0));
      const d3 f1 = sel4(V, face_local<FO>(a, f, 1));
      const d3 f2 = sel4(V, face_local<FO>(a, f, 2));
      double t;
      const bool hit = plucker64(f0, f1, f2, r, u, rn, INFTY, 0.0, true, 1, &t);
      dists[f] = hit ? (gt0(t) ? t : 0.0) : INFTY;  // std::max(0.0, t)
    }
    cnt.esc += 4;
  } else {
    float4 P[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) P[k] = __ldg(&a.xyz32[ci[k]]);
    const float rx = __double2float_rn(r.x), ry = __double2float_rn(r.y),
                rz = __double2float_rn(r.z);
    const float ux = __double2float_rn(u.x), uy = __double2float_rn(u.y),
                uz = __double2float_rn(u.z);
    float wx[4], wy[4], wz[4];
    float W = 0.0f, Av = 0.0f;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      wx[k] = P[k].x - rx;
      wy[k] = P[k].y - ry;
      wz[k] = P[k].z - rz;
      W = fmaxf(W, fmaxf(fabsf(wx[k]), fmaxf(fabsf(wy[k]), fabsf(wz[k]))));
      Av = fmaxf(Av, P[k].w);
    }
    const float D = fmaxf(fabsf(ux), fmaxf(fabsf(uy), fabsf(uz)));
    const float A = Av + fmaxf(fabsf(rx), fmaxf(fabsf(ry), fabsf(rz)));
    const float thr =
        kU32 * 1.000001f * D * W * (97.0f * W + 13.0f * Av + 13.0f * A) * 1.0001f + 4.5e-15f;
    // pip(i -> j) = u . ((v_j - v_i) x (v_i - r)) for the six pairs i < j
    float pe[6];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = i + 1; j < 4; ++j)
        pe[pair_index(i, j)] = triple32(ux, uy, uz, P[j].x - P[i].x, P[j].y - P[i].y,
                                        P[j].z - P[i].z, wx[i], wy[i], wz[i]);
    // faces whose FP32 coordinates do not certify an early exit
    unsigned escm = 0u;
#pragma unroll
    for (int f = 0; f < 4; ++f) {
      const int l0 = face_local<FO>(a, f, 0), l1 = face_local<FO>(a, f, 1),
                l2 = face_local<FO>(a, f, 2);
      const int e0 = pair_index(l0, l1), e1 = pair_index(l1, l2), e2 = pair_index(l2, l0);
      const float p0 = l0 < l1 ? sel6(pe, e0) : -sel6(pe, e0);
      const float p1 = l1 < l2 ? sel6(pe, e1) : -sel6(pe, e1);
      const float p2 = l2 < l0 ? sel6(pe, e2) : -sel6(pe, e2);
      if (!(p0 > thr || p1 > thr || p2 > thr)) escm |= 1u << f;
    }
    // FP64 for the remaining faces, in increasing face order (the strict-<
    // argmin below is then the reference's, :191-196).  Every lane runs its
    // first escalated face in the same iteration, so the FP64 work of a warp
    // is issued once for all lanes.
    int idx = -1;
    double best = INFTY;
    while (escm) {
      const int f = __ffs(escm) - 1;
      escm &= escm - 1u;
      cnt.esc++;
      const int l0 = face_local<FO>(a, f, 0), l1 = face_local<FO>(a, f, 1),
                l2 = face_local<FO>(a, f, 2);
      double t;
      bool hit;
      if (a.edge) {
        hit = plucker64_face_pre(a, elem, ci, l0, l1, l2, r, u, rn, &t);
      } else {
        const d3 f0 = load3(a.xyz, sel4(ci, l0));
        const d3 f1 = load3(a.xyz, sel4(ci, l1));
        const d3 f2 = load3(a.xyz, sel4(ci, l2));
        hit = plucker64(f0, f1, f2, r, u, rn, INFTY, 0.0, true, 1, &t);
      }
      const double df = hit ? (gt0(t) ? t : 0.0) : INFTY;  // std::max(0.0, t)
      if (dlt(df, best)) {
        best = df;
        idx = f;
      }
    }
    *exit_dist = best;
    return idx;
  }
  int idx = -1;
  double best = INFTY;
#pragma unroll
  for (int f = 0; f < 4; ++f) {
    if (dlt(dists[f], best)) {
      best = dists[f];
      idx = f;
    }
  }
  *exit_dist = best;
  return idx;
}

__device__ __forceinline__ void flush(unsigned long long* g, const StepCnt& c, unsigned long long rays) {
  unsigned long long v[3] = {c.steps, c.esc, rays};
  for (int k = 0; k < 3; ++k) {
    unsigned long long x = v[k];
    for (int off = 16; off > 0; off >>= 1) x += __shfl_xor_sync(__activemask(), x, off);
    v[k] = x;
  }
  if ((threadIdx.x & 31) == __ffs(__activemask()) - 1) {
    atomicAdd(&g[CNT_STEPS], v[0]);
    atomicAdd(&g[CNT_ESCALATE], v[1]);
    atomicAdd(&g[CNT_RAYS], v[2]);
  }
}

// The optional end state of track i's walk (WalkArgs::sum_out, end_r,
// end_dist): the running length sum, the position and the distance left.
__device__ __forceinline__ void walk_end_state(const WalkArgs& a, int64_t i, d3 r, double dist,
                                               double sum) {
  if (a.sum_out) a.sum_out[i] = sum;
  if (a.end_r) {
    a.end_r[3 * i] = r.x;
    a.end_r[3 * i + 1] = r.y;
    a.end_r[3 * i + 2] = r.z;
  }
  if (a.end_dist) a.end_dist[i] = dist;
}

// Persistent walk: each warp owns a contiguous chunk of tracks; a lane whose
// track has ended takes the next track of the chunk, so a warp keeps all 32
// lanes stepping until its chunk is exhausted (track lengths are
// exponentially distributed, so one-track-per-lane would leave most lanes
// idle behind the longest track of the warp).
template <int FO, bool MIXED>
__global__ void __launch_bounds__(kBlock) k_walk(WalkArgs a, int64_t chunk) {
  const int lane = threadIdx.x & 31;
  const int64_t gwarp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  // the warp's tracks: positions first + k * stride, k < count (a contiguous
  // chunk, or with a length order every W-th track of it, longest first)
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int64_t first = a.order ? gwarp : gwarp * chunk;
  const int64_t stride = a.order ? nwarps : 1;
  const int64_t count = a.order ? (gwarp < a.n ? (a.n - gwarp + nwarps - 1) / nwarps : 0)
                                : max((int64_t)0, min(a.n, first + chunk) - first);
  int64_t cursor = 0;
  const int64_t end = count;
  StepCnt cnt = {0, 0};
  unsigned long long tracks = 0;
  bool has = false;
  int64_t i = 0;
  d3 r = mk3(0, 0, 0), u = mk3(0, 0, 0);
  double dist = 0.0, sum = 0.0;
  int32_t elem = -1, k = 0, st = RAY_OK;
  int32_t* oe = nullptr;
  double* ol = nullptr;
  while (true) {
    const unsigned need = __ballot_sync(0xffffffffu, !has);
    if (need != 0u && cursor < end) {
      if (!has) {
        unsigned lt;
        asm("mov.u32 %0, %%lanemask_lt;" : "=r"(lt));
        const int64_t kk = cursor + __popc(need & lt);
        const int64_t pos = first + kk * stride;
        const int64_t cand = kk < end ? (a.order ? (int64_t)__ldg(&a.order[pos]) : pos) : -1;
        if (cand >= 0 && cand < a.n) {  // (an order entry out of range names no track)
          i = cand;
          has = true;
          r = load3(a.org, i);
          u = load3(a.dir, i);
          dist = a.dist[i];
          sum = a.sum_in ? a.sum_in[i] : 0.0;
          elem = a.start[i];
          k = 0;
          st = RAY_OK;
          if (a.out_mode == WALK_STRIDED) {
            oe = a.seg_elem + i * (int64_t)a.max_segs;
            ol = a.seg_len + i * (int64_t)a.max_segs;
          } else if (a.out_mode == WALK_PACKED) {
            const int64_t off = a.offsets[i];
            const int64_t cnt_i = a.offsets[i + 1] - off;
            if (off + cnt_i <= a.capacity) {
              oe = a.seg_elem + off;
              ol = a.seg_len + off;
            } else {
              oe = nullptr;  // does not fit: the track is walked, nothing is written
              ol = nullptr;
            }
          } else {
            oe = nullptr;
            ol = nullptr;
          }
          if (elem < 0 || elem >= a.n_tets || !finite3(r) || !finite3(u) || nan_bits(dist)) {
            st = RAY_INVALID;
            dist = 0.0;  // finishes below without a step
          }
        }
      }
      cursor += __popc(need);
    }
    if (__ballot_sync(0xffffffffu, has) == 0u) break;
    if (has) {
      bool done = !gt0(dist);  // while (distance > 0), mesh_manager_interface.cpp:117
      if (!done && k >= a.max_segs) {
        st = RAY_WALK_LIMIT;
        done = true;
      }
      if (!done) {
        cnt.steps++;
        double ex;
        const int f = next_face<FO, MIXED>(a, elem, r, u, &ex, cnt);
        int32_t nxt = -1;
        if (f < 0) {
          st = RAY_NO_EXIT_FACE;  // the reference would index adjacency with -1
        } else {
          const int4 ad = __ldg(&a.adj[elem]);
          nxt = f == 0 ? ad.x : (f == 1 ? ad.y : (f == 2 ? ad.z : ad.w));
        }
        ex = dlt(dist, ex) ? dist : ex;  // std::min(exit, distance)
        dist -= ex;
        if (a.sum_out) sum = sum + ex;
        if (oe) {
          oe[k] = __ldg(&a.elem_ids[elem]);
          ol[k] = ex;
        }
        ++k;
        r = add3(r, scl3(ex, u));  // r += exit.second * u
        if (nxt < -1 || nxt >= a.n_tets) {
          st = RAY_INVALID;  // corrupt adjacency: stop instead of reading out of range
          done = true;
        } else {
          elem = nxt;
          if (elem == -1) done = true;
        }
      }
      if (done) {
        if (a.out_mode == WALK_COUNT) {
          a.offsets[i] = k;
        } else {
          if (a.seg_count) a.seg_count[i] = k;
          if (a.out_mode == WALK_PACKED && !oe && k > 0 && st == RAY_OK) st = RAY_OUTPUT_FULL;
        }
        if (a.status) a.status[i] = st;
        if (a.stop_elem) a.stop_elem[i] = elem;  // where a capped walk resumes
        walk_end_state(a, i, r, dist, sum);
        has = false;
        tracks++;
      }
    }
  }
  if (a.counters) flush(a.counters, cnt, tracks);
}

template <int FO, bool MIXED>
__global__ void __launch_bounds__(kBlock) k_next(WalkArgs a) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  StepCnt cnt = {0, 0};
  if (i < a.n) {
    const d3 r = load3(a.org, i);
    const d3 u = load3(a.dir, i);
    const int32_t elem = a.start[i];
    int32_t st = RAY_OK, nxt = -1;
    double ex = INFTY;
    if (elem < 0 || elem >= a.n_tets || !finite3(r) || !finite3(u)) {
      st = RAY_INVALID;
    } else {
      cnt.steps++;
      const int f = next_face<FO, MIXED>(a, elem, r, u, &ex, cnt);
      if (f < 0) {
        st = RAY_NO_EXIT_FACE;
      } else {
        const int4 ad = __ldg(&a.adj[elem]);
        nxt = f == 0 ? ad.x : (f == 1 ? ad.y : (f == 2 ? ad.z : ad.w));
      }
    }
    a.next_out[i] = nxt;
    a.dist_out[i] = ex;
    if (a.status) a.status[i] = st;
  }
  if (a.counters) flush(a.counters, cnt, i < a.n ? 1ull : 0ull);
}

// ---------------------------------------------------------------------------
// Mixed-precision walk with a per-warp FP64 queue.
//
// Each step of a track runs the FP32 edge filter for its tet (six edge
// coordinates, truncated FP32 inputs, bound below) and queues every face the
// filter cannot reject as a (lane, face) task.  When 32 tasks are queued, or
// lanes wait on the queue, the whole warp runs 32 tasks at once -- each lane
// evaluates one face of some lane's tet with the FP64 Plucker test -- and each
// owner keeps the smallest (distance, face index) of its results, which is
// the reference's strict-< scan over faces 0..3 (:186-196) in any order.  A
// lane whose tasks are all done completes its step (segment, r += len * u)
// and starts the next one, so FP64 instructions run with (nearly) all 32
// lanes busy however many faces each step escalates.
//
// FP32 bound with truncated inputs (u = 2^-24; r and the direction truncated,
// relative error 2u; stored vertices rounded, u; W = max |v_k - r|_inf over
// the FP32 differences; Wb = W (1 + 2^-20) + 1.01 u (Av + 2 R) bounds the
// exact |v_k - r|_inf; edges |e| <= 2 Wb; D = |u|_inf, Av = max |v_k|_inf,
// R = |r|_inf):
//   rounding of the triple product (gamma_5, six terms)   <= 60 u D Wb^2
//   input perturbation (direction 2u, edges, differences) <= u D Wb (48 Wb + 24 Av + 24 R)
// so |pip32 - pip| <= u D Wb (108 Wb + 24 Av + 24 R); the threshold uses
// 110 / 26 / 26 and a factor 1.01 for second-order terms, the FP64
// evaluation error and the rounding of the threshold itself, plus the
// 20*DBL_EPSILON snap.
// ---------------------------------------------------------------------------

constexpr int kWQ = 256;  // ring entries per warp: < 32 left over + 4 per lane

struct WalkQueue {
  uint32_t ent[kWQ];  // (owner lane << 2) | face
  double rd[32];
  int32_t rf[32];
  uint32_t head, tail;
};

template <int FO>
__device__ __forceinline__ unsigned walk_filter32(const WalkArgs& a, const int32_t ci[4], float rx,
                                                  float ry, float rz, float ux, float uy, float uz,
                                                  float D, float R) {
  float4 P[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) P[k] = __ldg(&a.xyz32[ci[k]]);
  float wx[4], wy[4], wz[4];
  float W = 0.0f, Av = 0.0f;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    wx[k] = P[k].x - rx;
    wy[k] = P[k].y - ry;
    wz[k] = P[k].z - rz;
    W = fmaxf(W, fmaxf(fabsf(wx[k]), fmaxf(fabsf(wy[k]), fabsf(wz[k]))));
    Av = fmaxf(Av, P[k].w);
  }
  const float Wb = W * 1.000001f + kU32 * 1.01f * (Av + 2.0f * R);
  const float thr = kU32 * D * Wb * (110.0f * Wb + 26.0f * Av + 26.0f * R) * 1.01f + 4.5e-15f;
  float pe[6];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = i + 1; j < 4; ++j)
      pe[pair_index(i, j)] = triple32(ux, uy, uz, P[j].x - P[i].x, P[j].y - P[i].y,
                                      P[j].z - P[i].z, wx[i], wy[i], wz[i]);
  unsigned escm = 0u;
#pragma unroll
  for (int f = 0; f < 4; ++f) {
    const int l0 = face_local<FO>(a, f, 0), l1 = face_local<FO>(a, f, 1),
              l2 = face_local<FO>(a, f, 2);
    const int e0 = pair_index(l0, l1), e1 = pair_index(l1, l2), e2 = pair_index(l2, l0);
    const float p0 = l0 < l1 ? sel6(pe, e0) : -sel6(pe, e0);
    const float p1 = l1 < l2 ? sel6(pe, e1) : -sel6(pe, e1);
    const float p2 = l2 < l0 ? sel6(pe, e2) : -sel6(pe, e2);
    if (!(p0 > thr || p1 > thr || p2 > thr)) escm |= 1u << f;
  }
  return escm;
}

template <int FO>
__global__ void __launch_bounds__(kBlock) k_walk_q(WalkArgs a, int64_t chunk) {
  __shared__ WalkQueue qs[kBlock / 32];
  WalkQueue& Q = qs[threadIdx.x >> 5];
  const int lane = threadIdx.x & 31;
  const int64_t gwarp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  // the warp's tracks: positions first + k * stride, k < count (a contiguous
  // chunk, or with a length order every W-th track of it, longest first)
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int64_t first = a.order ? gwarp : gwarp * chunk;
  const int64_t stride = a.order ? nwarps : 1;
  const int64_t count = a.order ? (gwarp < a.n ? (a.n - gwarp + nwarps - 1) / nwarps : 0)
                                : max((int64_t)0, min(a.n, first + chunk) - first);
  int64_t cursor = 0;
  const int64_t end = count;
  if (lane == 0) {
    Q.head = 0u;
    Q.tail = 0u;
  }
  __syncwarp();
  StepCnt cnt = {0, 0};
  unsigned long long tracks = 0;
  // track state
  bool has = false;
  int64_t i = 0;
  d3 r = mk3(0, 0, 0), u = mk3(0, 0, 0);
  double dist = 0.0, sum = 0.0;
  int32_t elem = -1, k = 0, st = RAY_OK;
  int32_t* oe = nullptr;
  double* ol = nullptr;
  float ux = 0.f, uy = 0.f, uz = 0.f, D = 0.f;
  // step state
  bool in_step = false;
  int npend = 0;
  double bd = INFTY;
  int32_t bf = -1;
  d3 rn = mk3(0, 0, 0);
  int32_t ci[4] = {0, 0, 0, 0};

  while (true) {
    // ---- refill lanes without a track from the warp's chunk ----
    const unsigned need = __ballot_sync(0xffffffffu, !has);
    if (need != 0u && cursor < end) {
      if (!has) {
        unsigned lt;
        asm("mov.u32 %0, %%lanemask_lt;" : "=r"(lt));
        const int64_t kk = cursor + __popc(need & lt);
        const int64_t pos = first + kk * stride;
        const int64_t cand = kk < end ? (a.order ? (int64_t)__ldg(&a.order[pos]) : pos) : -1;
        if (cand >= 0 && cand < a.n) {  // (an order entry out of range names no track)
          i = cand;
          has = true;
          in_step = false;
          r = load3(a.org, i);
          u = load3(a.dir, i);
          dist = a.dist[i];
          sum = a.sum_in ? a.sum_in[i] : 0.0;
          elem = a.start[i];
          k = 0;
          st = RAY_OK;
          ux = f32_trunc(u.x);
          uy = f32_trunc(u.y);
          uz = f32_trunc(u.z);
          D = fmaxf(fabsf(ux), fmaxf(fabsf(uy), fabsf(uz))) * 1.0000002f;
          if (a.out_mode == WALK_STRIDED) {
            oe = a.seg_elem + i * (int64_t)a.max_segs;
            ol = a.seg_len + i * (int64_t)a.max_segs;
          } else if (a.out_mode == WALK_PACKED) {
            const int64_t off = a.offsets[i];
            const int64_t cnt_i = a.offsets[i + 1] - off;
            if (off + cnt_i <= a.capacity) {
              oe = a.seg_elem + off;
              ol = a.seg_len + off;
            } else {
              oe = nullptr;  // does not fit: the track is walked, nothing is written
              ol = nullptr;
            }
          } else {
            oe = nullptr;
            ol = nullptr;
          }
          if (elem < 0 || elem >= a.n_tets || !finite3(r) || !finite3(u) || nan_bits(dist)) {
            st = RAY_INVALID;
            dist = 0.0;  // finishes below without a step
          }
        }
      }
      cursor += __popc(need);
    }
    if (__ballot_sync(0xffffffffu, has) == 0u) break;

    // ---- start a step: FP32 filter, queue the faces it cannot reject ----
    unsigned escm = 0u;
    if (has && !in_step) {
      bool done = !gt0(dist);  // while (distance > 0), mesh_manager_interface.cpp:117
      if (!done && k >= a.max_segs) {
        st = RAY_WALK_LIMIT;
        done = true;
      }
      if (done) {
        if (a.out_mode == WALK_COUNT) {
          a.offsets[i] = k;
        } else {
          if (a.seg_count) a.seg_count[i] = k;
          if (a.out_mode == WALK_PACKED && !oe && k > 0 && st == RAY_OK) st = RAY_OUTPUT_FULL;
        }
        if (a.status) a.status[i] = st;
        if (a.stop_elem) a.stop_elem[i] = elem;  // where a capped walk resumes
        walk_end_state(a, i, r, dist, sum);
        has = false;
        tracks++;
      } else {
        cnt.steps++;
        in_step = true;
        const int4 c = __ldg(&a.conn[elem]);
        ci[0] = c.x;
        ci[1] = c.y;
        ci[2] = c.z;
        ci[3] = c.w;
        const float rx = f32_trunc(r.x), ry = f32_trunc(r.y), rz = f32_trunc(r.z);
        const float R = fmaxf(fabsf(rx), fmaxf(fabsf(ry), fabsf(rz))) * 1.0000002f;
        escm = walk_filter32<FO>(a, ci, rx, ry, rz, ux, uy, uz, D, R);
        rn = cross3(u, r);  // plucker.h:75
        bd = INFTY;
        bf = -1;
        npend = __popc(escm);
        cnt.esc += npend;
      }
    }
    {
      const int c = __popc(escm);
      int incl = c;
#pragma unroll
      for (int off = 1; off < 32; off <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, off);
        if (lane >= off) incl += y;
      }
      const int total = __shfl_sync(0xffffffffu, incl, 31);
      if (total > 0) {
        const uint32_t tail = Q.tail;
        __syncwarp();
        uint32_t pos = tail + (uint32_t)(incl - c);
        unsigned m = escm;
        while (m) {
          const int f = __ffs(m) - 1;
          m &= m - 1u;
          Q.ent[pos & (kWQ - 1)] = ((uint32_t)lane << 2) | (uint32_t)f;
          ++pos;
        }
        __syncwarp();
        if (lane == 0) Q.tail = tail + (uint32_t)total;
      }
      __syncwarp();
    }

    // ---- run queued FP64 face tests with the whole warp ----
    while (true) {
      const uint32_t head = Q.head;
      const int qn = (int)(Q.tail - head);
      const unsigned waiting = __ballot_sync(0xffffffffu, in_step && npend > 0);
      const unsigned progress = __ballot_sync(0xffffffffu, has && !(in_step && npend > 0));
      if (!(qn >= 32 || (qn > 0 && (progress == 0u || __popc(waiting) >= a.flush_wait)))) break;
      const int nq = min(qn, 32);
      const bool mine = lane < nq;
      const uint32_t ent = mine ? Q.ent[(head + lane) & (kWQ - 1)] : ((uint32_t)lane << 2);
      const int owner = (int)(ent >> 2);
      const int f = (int)(ent & 3u);
      d3 orr, ou, orn;
      orr.x = __shfl_sync(0xffffffffu, r.x, owner);
      orr.y = __shfl_sync(0xffffffffu, r.y, owner);
      orr.z = __shfl_sync(0xffffffffu, r.z, owner);
      ou.x = __shfl_sync(0xffffffffu, u.x, owner);
      ou.y = __shfl_sync(0xffffffffu, u.y, owner);
      ou.z = __shfl_sync(0xffffffffu, u.z, owner);
      orn.x = __shfl_sync(0xffffffffu, rn.x, owner);
      orn.y = __shfl_sync(0xffffffffu, rn.y, owner);
      orn.z = __shfl_sync(0xffffffffu, rn.z, owner);
      int32_t oc[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) oc[q] = __shfl_sync(0xffffffffu, ci[q], owner);
      const int32_t oel = __shfl_sync(0xffffffffu, elem, owner);
      double df = INFTY;
      if (mine) {
        const int l0 = face_local<FO>(a, f, 0), l1 = face_local<FO>(a, f, 1),
                  l2 = face_local<FO>(a, f, 2);
        double t;
        bool hit;
        if (a.edge) {
          hit = plucker64_face_pre(a, oel, oc, l0, l1, l2, orr, ou, orn, &t);
        } else {
          const d3 f0 = load3(a.xyz, sel4(oc, l0));
          const d3 f1 = load3(a.xyz, sel4(oc, l1));
          const d3 f2 = load3(a.xyz, sel4(oc, l2));
          hit = plucker64(f0, f1, f2, orr, ou, orn, INFTY, 0.0, true, 1, &t);
        }
        df = hit ? (gt0(t) ? t : 0.0) : INFTY;  // std::max(0.0, t)
      }
      Q.rd[lane] = df;
      Q.rf[lane] = f;
      __syncwarp();
      for (int j = 0; j < nq; ++j) {
        if (__shfl_sync(0xffffffffu, owner, j) != lane) continue;
        npend--;
        const double dj = Q.rd[j];
        const int32_t fj = Q.rf[j];
        // first minimum over faces 0..3 with strict < (:186-196)
        if (dlt(dj, bd) || (bf >= 0 && okey(dj) == okey(bd) && fj < bf)) {
          bd = dj;
          bf = fj;
        }
      }
      __syncwarp();
      if (lane == 0) Q.head = head + (uint32_t)nq;
      __syncwarp();
    }

    // ---- complete the steps whose faces are all evaluated ----
    if (has && in_step && npend == 0) {
      in_step = false;
      int32_t nxt = -1;
      double ex = bd;
      if (bf < 0) {
        st = RAY_NO_EXIT_FACE;  // the reference would index adjacency with -1
      } else {
        const int4 ad = __ldg(&a.adj[elem]);
        nxt = bf == 0 ? ad.x : (bf == 1 ? ad.y : (bf == 2 ? ad.z : ad.w));
      }
      ex = dlt(dist, ex) ? dist : ex;  // std::min(exit, distance)
      dist -= ex;
      if (a.sum_out) sum = sum + ex;
      if (oe) {
        oe[k] = __ldg(&a.elem_ids[elem]);
        ol[k] = ex;
      }
      ++k;
      r = add3(r, scl3(ex, u));  // r += exit.second * u
      bool done = false;
      if (nxt < -1 || nxt >= a.n_tets) {
        st = RAY_INVALID;  // corrupt adjacency: stop instead of reading out of range
        done = true;
      } else {
        elem = nxt;
        if (elem == -1) done = true;
      }
      if (done) {
        if (a.out_mode == WALK_COUNT) {
          a.offsets[i] = k;
        } else {
          if (a.seg_count) a.seg_count[i] = k;
          if (a.out_mode == WALK_PACKED && !oe && k > 0 && st == RAY_OK) st = RAY_OUTPUT_FULL;
        }
        if (a.status) a.status[i] = st;
        if (a.stop_elem) a.stop_elem[i] = elem;  // where a capped walk resumes
        walk_end_state(a, i, r, dist, sum);
        has = false;
        tracks++;
      }
    }
  }
  if (a.counters) flush(a.counters, cnt, tracks);
}

constexpr int kScanBlock = 1024;

// sum of each block of kScanBlock counts
__global__ void __launch_bounds__(kScanBlock) k_block_sums(const int64_t* __restrict__ v, int64_t n,
                                                           int64_t* __restrict__ sums) {
  __shared__ int64_t ws[kScanBlock / 32];
  const int64_t i = blockIdx.x * (int64_t)kScanBlock + threadIdx.x;
  int64_t x = i < n ? v[i] : 0;
  for (int off = 16; off > 0; off >>= 1) x += __shfl_xor_sync(0xffffffffu, x, off);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = x;
  __syncthreads();
  if (threadIdx.x < 32) {
    int64_t y = ws[threadIdx.x];
    for (int off = 16; off > 0; off >>= 1) y += __shfl_xor_sync(0xffffffffu, y, off);
    if (threadIdx.x == 0) sums[blockIdx.x] = y;
  }
}

// exclusive scan of the block sums by one block; sums[nb] = total
__global__ void __launch_bounds__(kScanBlock) k_scan_sums(int64_t* __restrict__ sums, int64_t nb) {
  __shared__ int64_t ws[kScanBlock / 32];
  __shared__ int64_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int64_t base = 0; base < nb; base += kScanBlock) {
    const int64_t i = base + threadIdx.x;
    const int64_t x = i < nb ? sums[i] : 0;
    int64_t incl = x;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int off = 1; off < 32; off <<= 1) {
      const int64_t y = __shfl_up_sync(0xffffffffu, incl, off);
      if (lane >= off) incl += y;
    }
    if (lane == 31) ws[w] = incl;
    __syncthreads();
    if (w == 0) {
      int64_t s = ws[lane];
      for (int off = 1; off < 32; off <<= 1) {
        const int64_t y = __shfl_up_sync(0xffffffffu, s, off);
        if (lane >= off) s += y;
      }
      ws[lane] = s;
    }
    __syncthreads();
    const int64_t before = carry + (w > 0 ? ws[w - 1] : 0) + incl - x;
    if (i < nb) sums[i] = before;
    __syncthreads();
    if (threadIdx.x == kScanBlock - 1) carry = before + x;
    __syncthreads();
  }
  if (threadIdx.x == 0) sums[nb] = carry;
}

// in-place exclusive scan of each block plus its block offset
__global__ void __launch_bounds__(kScanBlock) k_scan_apply(int64_t* __restrict__ v, int64_t n,
                                                           const int64_t* __restrict__ sums,
                                                           int64_t nb) {
  __shared__ int64_t ws[kScanBlock / 32];
  const int64_t i = blockIdx.x * (int64_t)kScanBlock + threadIdx.x;
  const int64_t x = i < n ? v[i] : 0;
  int64_t incl = x;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int off = 1; off < 32; off <<= 1) {
    const int64_t y = __shfl_up_sync(0xffffffffu, incl, off);
    if (lane >= off) incl += y;
  }
  if (lane == 31) ws[w] = incl;
  __syncthreads();
  if (w == 0) {
    int64_t s = ws[lane];
    for (int off = 1; off < 32; off <<= 1) {
      const int64_t y = __shfl_up_sync(0xffffffffu, s, off);
      if (lane >= off) s += y;
    }
    ws[lane] = s;
  }
  __syncthreads();
  const int64_t excl = sums[blockIdx.x] + (w > 0 ? ws[w - 1] : 0) + incl - x;
  if (i < n) v[i] = excl;
  if (blockIdx.x == 0 && threadIdx.x == 0) v[n] = sums[nb];
}

template <int FO, bool MIXED, bool QUEUE>
cudaError_t launch_walk_t(const WalkArgs& a, cudaStream_t st) {
  static std::atomic<int> cached[kMaxDevices];  // resident blocks per SM, per device
  auto kern = QUEUE ? k_walk_q<FO> : k_walk<FO, MIXED>;
  int per_sm = 0;
  const cudaError_t e = occupancy_cached(cached, kern, kBlock, 0, per_sm);
  if (e != cudaSuccess) return e;
  int64_t blocks = (int64_t)device_sm_count() * per_sm;
  const int64_t max_blocks = (a.n + kBlock - 1) / kBlock;
  if (blocks > max_blocks) blocks = max_blocks;
  if (blocks < 1) blocks = 1;
  const int64_t warps = blocks * (kBlock / 32);
  const int64_t chunk = (a.n + warps - 1) / warps;
  kern<<<(unsigned)blocks, kBlock, 0, st>>>(a, chunk);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_walk(bool mixed, int face_order, const WalkArgs& a, cudaStream_t st) {
  if (a.n <= 0) return cudaSuccess;
  const int sel = (face_order == 0 ? 0 : 2) + (mixed ? 1 : 0);
  const bool q = mixed && a.walk_queue;
  switch (sel) {
    case 0: return launch_walk_t<0, false, false>(a, st);
    case 1: return q ? launch_walk_t<0, true, true>(a, st) : launch_walk_t<0, true, false>(a, st);
    case 2: return launch_walk_t<1, false, false>(a, st);
    default: return q ? launch_walk_t<1, true, true>(a, st) : launch_walk_t<1, true, false>(a, st);
  }
}

namespace {

// ---------------------------------------------------------------------------
// Device particle loop over the tet mesh: the body of the walk_elements tool
// (tools/walk_elements.h:73-95) for particles inside the mesh.  Per event:
//   (next, exit) = next_element(elem, r, u)             (next_face above)
//   c = -log(1 - U) * mfp                                (sample.cuh)
//   c < exit: r += u c, distance += c, u = new isotropic direction
//   else:     r += u exit, distance += exit, elem = next
//   events++
// until the particle leaves the mesh (elem = -1, status OK: the caller
// decides on re-entry, which the tool does by ray_fire in the implicit
// complement and find_element, :88-94) or reaches max_events
// (RAY_EVENT_LIMIT).  With `tally`, each event adds its path length to the
// tet it was made in (atomicAdd, so the sums' rounding depends on the order).
// Warps own contiguous chunks of particles and refill lanes as particles
// finish, as in k_walk.  The collision sample's FP64 logarithm and the new
// direction are only computed where needed (see the FP32 test below) and for
// many lanes at once.
// ---------------------------------------------------------------------------

template <int FO, bool MIXED>
__global__ void __launch_bounds__(kBlock) k_transport(TransportArgs t, int64_t chunk) {
  const WalkArgs& a = t.mesh;
  const int64_t gwarp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  int64_t cursor = gwarp * chunk;
  const int64_t end = min(t.n, cursor + chunk);
  StepCnt cnt = {0, 0};
  unsigned long long parts = 0;
  bool has = false;
  int64_t i = 0;
  d3 r = mk3(0, 0, 0), u = mk3(0, 0, 0);
  double dist = 0.0;
  int32_t elem = -1, ev = 0, st = RAY_OK;
  unsigned long long rs = 0;
  // an event whose FP64 part waits for the warp's batch: its uniform draw,
  // exit distance and exit face
  bool pend = false;
  double pu = 0.0, pex = 0.0;
  int pf = -1;
  const float mfp32 = (float)t.mfp;
  const bool quick = t.mfp < 1e30;

  // moves the particle to the exit face and into the neighbour (:86-90);
  // returns true when it stops
  auto exit_step = [&](double ex, int f) -> bool {
    if (f < 0) {
      st = RAY_NO_EXIT_FACE;  // exit = INFTY and c >= INFTY: no finite step exists
      return true;
    }
    const int4 ad = __ldg(&a.adj[elem]);
    const int32_t nxt = f == 0 ? ad.x : (f == 1 ? ad.y : (f == 2 ? ad.z : ad.w));
    r = add3(r, scl3(ex, u));
    dist += ex;
    if (t.tally) atomicAdd(&t.tally[elem], ex);
    if (nxt < -1 || nxt >= a.n_tets) {
      st = RAY_INVALID;  // corrupt adjacency
      return true;
    }
    elem = nxt;
    ++ev;
    return elem < 0;
  };

  while (true) {
    const unsigned need = __ballot_sync(0xffffffffu, !has);
    if (need != 0u && cursor < end) {
      if (!has) {
        unsigned lt;
        asm("mov.u32 %0, %%lanemask_lt;" : "=r"(lt));
        const int64_t kk = cursor + __popc(need & lt);
        if (kk < end) {
          i = kk;
          has = true;
          pend = false;
          elem = t.elem[i];
          r = load3(t.pos, i);
          u = load3(t.dir, i);
          rs = t.rng[i];
          dist = t.distance[i];
          ev = t.events[i];
          st = RAY_OK;
          if (elem >= a.n_tets || !finite3(r) || !finite3(u) || nan_bits(dist)) st = RAY_INVALID;
        }
      }
      cursor += __popc(need);
    }
    if (__ballot_sync(0xffffffffu, has) == 0u) break;
    bool done = false;
    if (has && !pend) {
      done = st != RAY_OK || elem < 0;  // nothing to do outside the mesh
      if (!done && ev >= t.max_events) {
        st = RAY_EVENT_LIMIT;
        done = true;
      }
      if (!done) {
        cnt.steps++;
        double ex;
        const int f = next_face<FO, MIXED>(a, elem, r, u, &ex, cnt);
        const double U = uniform53(rs);
        // Most events leave the tet: an FP32 logarithm with a certified
        // margin decides c >= exit without the FP64 series.  |c32 - c| <=
        // 6.1e-8 mfp + 3.7e-7 c (rounding 1 - U to FP32, logf within 2 ulp,
        // two FP32 products); the margin below is 1.1e-6 (c32 + mfp).
        bool leaves = false;
        if (quick) {
          const float c32 = -logf(__double2float_rn(1.0 - U)) * mfp32;
          const float lo = c32 - 1.1e-6f * (c32 + mfp32);
          leaves = dlt(ex, (double)lo);  // c >= lo > exit
        }
        if (leaves) {
          done = exit_step(ex, f);
        } else {
          pend = true;  // the exact sample and the event run with the warp's batch
          pu = U;
          pex = ex;
          pf = f;
        }
      }
    }
    // Events that need the FP64 sample (collisions, and exits the FP32 test
    // could not certify) run together once event_wait lanes wait or no lane
    // can step: FP64 instructions cost the same issue time for 1 or 32 lanes.
    const unsigned pm = __ballot_sync(0xffffffffu, has && pend);
    if (pm != 0u) {
      const unsigned run = __ballot_sync(0xffffffffu, has && !pend && !done);
      if (__popc(pm) >= t.event_wait || run == 0u) {
        if (has && pend) {
          pend = false;
          const double c = -series_log(1.0 - pu) * t.mfp;  // sample_collision's value
          if (dlt(c, pex)) {
            // collision inside the tet (:81-85)
            r = add3(r, scl3(c, u));
            dist += c;
            if (t.tally) atomicAdd(&t.tally[elem], c);
            u = sample_direction(rs);
            ++ev;
          } else {
            done = exit_step(pex, pf);
          }
        }
      }
    }
    if (has && done) {
      t.elem[i] = elem;
      t.pos[3 * i] = r.x;
      t.pos[3 * i + 1] = r.y;
      t.pos[3 * i + 2] = r.z;
      t.dir[3 * i] = u.x;
      t.dir[3 * i + 1] = u.y;
      t.dir[3 * i + 2] = u.z;
      t.rng[i] = rs;
      t.distance[i] = dist;
      t.events[i] = ev;
      if (t.status) t.status[i] = st;
      has = false;
      parts++;
    }
  }
  if (t.counters) flush(t.counters, cnt, parts);
}

template <int FO, bool MIXED>
cudaError_t launch_transport_t(const TransportArgs& a, cudaStream_t st) {
  static std::atomic<int> cached[kMaxDevices];  // resident blocks per SM, per device
  auto kern = k_transport<FO, MIXED>;
  int per_sm = 0;
  const cudaError_t e = occupancy_cached(cached, kern, kBlock, 0, per_sm);
  if (e != cudaSuccess) return e;
  int64_t blocks = (int64_t)device_sm_count() * per_sm;
  const int64_t max_blocks = (a.n + kBlock - 1) / kBlock;
  if (blocks > max_blocks) blocks = max_blocks;
  if (blocks < 1) blocks = 1;
  const int64_t warps = blocks * (kBlock / 32);
  const int64_t chunk = (a.n + warps - 1) / warps;
  kern<<<(unsigned)blocks, kBlock, 0, st>>>(a, chunk);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_transport(bool mixed, int face_order, const TransportArgs& a, cudaStream_t st) {
  if (a.n <= 0) return cudaSuccess;
  switch ((face_order == 0 ? 0 : 2) + (mixed ? 1 : 0)) {
    case 0: return launch_transport_t<0, false>(a, st);
    case 1: return launch_transport_t<0, true>(a, st);
    case 2: return launch_transport_t<1, false>(a, st);
    default: return launch_transport_t<1, true>(a, st);
  }
}

int64_t scan_scratch_entries(int64_t n) { return (n + kScanBlock - 1) / kScanBlock + 1; }

namespace {
__global__ void k_iota(int32_t* v, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) v[i] = (int32_t)i;
}
}  // namespace

namespace {

// local vertex pairs of a tet in pair_index order
__device__ __forceinline__ void pair_of(int p, int& i, int& j) {
  i = p < 3 ? 0 : (p < 5 ? 1 : 2);
  j = p < 3 ? p + 1 : (p < 5 ? p - 1 : 3);
}

__device__ __forceinline__ int32_t conn_at(int4 c, int k) {
  return k == 0 ? c.x : (k == 1 ? c.y : (k == 2 ? c.z : c.w));
}

__global__ void k_edge_keys(const int4* __restrict__ conn, int64_t n_tets,
                            unsigned long long* __restrict__ keys, int32_t* __restrict__ slots) {
  const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= 6 * n_tets) return;
  const int4 c = conn[s / 6];
  int i, j;
  pair_of((int)(s % 6), i, j);
  const unsigned a = (unsigned)conn_at(c, i), b = (unsigned)conn_at(c, j);
  const unsigned lo = a < b ? a : b, hi = a < b ? b : a;
  keys[s] = ((unsigned long long)lo << 32) | hi;
  slots[s] = (int32_t)s;
}

__global__ void k_edge_heads(const unsigned long long* __restrict__ keys, int64_t n,
                             int32_t* __restrict__ head) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= n) return;
  head[k] = (k == 0 || keys[k] != keys[k - 1]) ? 1 : 0;
}

// e = hi - lo and en = e x lo of each unique edge (plucker.h:45-62 with
// first() ordering the two vertices); lo_vertex = the vertex index of lo
__global__ void k_edge_data(const unsigned long long* __restrict__ keys,
                            const int32_t* __restrict__ head, const int32_t* __restrict__ id,
                            int64_t n, const double* __restrict__ xyz, double* __restrict__ edge,
                            int32_t* __restrict__ lo_vertex) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= n || !head[k]) return;
  const int64_t e = id[k] - 1;
  const int32_t ga = (int32_t)(keys[k] >> 32), gb = (int32_t)(keys[k] & 0xffffffffull);
  const d3 va = load3(xyz, ga), vb = load3(xyz, gb);
  const bool f = first_lower(va, vb);
  const d3 lo = f ? va : vb;
  const d3 hi = f ? vb : va;
  const d3 ev = sub3(hi, lo);
  const d3 en = cross3(ev, lo);
  double* E = edge + 6 * e;
  E[0] = ev.x;
  E[1] = ev.y;
  E[2] = ev.z;
  E[3] = en.x;
  E[4] = en.y;
  E[5] = en.z;
  lo_vertex[e] = f ? ga : gb;
}

__global__ void k_edge_scatter(const int32_t* __restrict__ slots, const int32_t* __restrict__ id,
                               int64_t n, const int4* __restrict__ conn,
                               const int32_t* __restrict__ lo_vertex,
                               int32_t* __restrict__ tet_edge) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int32_t s = slots[k];
  const int32_t e = id[k] - 1;
  int i, j;
  pair_of(s % 6, i, j);
  const bool second_is_lo = conn_at(conn[s / 6], j) == lo_vertex[e];
  tet_edge[s] = e | (second_is_lo ? (int32_t)0x80000000u : 0);
}

}  // namespace

cudaError_t build_edge_table(const double* xyz, const int4* conn, int64_t n_tets, double** edge,
                             int32_t** tet_edge, int64_t* n_edges, cudaStream_t st) {
  *edge = nullptr;
  *tet_edge = nullptr;
  *n_edges = 0;
  const int64_t n = 6 * n_tets;
  if (n_tets <= 0 || n >= (1ll << 31)) return cudaErrorInvalidValue;
  const unsigned g = (unsigned)((n + 255) / 256);
  unsigned long long *keys = nullptr, *keys2 = nullptr;
  int32_t *slots = nullptr, *slots2 = nullptr, *head = nullptr, *id = nullptr, *lo = nullptr;
  void* tmp = nullptr;
  size_t tb_sort = 0, tb_scan = 0;
  cudaError_t e = cub::DeviceRadixSort::SortPairs(nullptr, tb_sort, keys, keys2, slots, slots2,
                                                  (int)n, 0, 64, st);
  if (e == cudaSuccess) e = cub::DeviceScan::InclusiveSum(nullptr, tb_scan, head, id, (int)n, st);
  const size_t tb = tb_sort > tb_scan ? tb_sort : tb_scan;
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&keys, sizeof(*keys) * n, st);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&keys2, sizeof(*keys2) * n, st);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&slots, sizeof(*slots) * n, st);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&slots2, sizeof(*slots2) * n, st);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&head, sizeof(*head) * n, st);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&id, sizeof(*id) * n, st);
  if (e == cudaSuccess) e = cudaMallocAsync(&tmp, tb, st);
  if (e == cudaSuccess) {
    k_edge_keys<<<g, 256, 0, st>>>(conn, n_tets, keys, slots);
    e = cudaGetLastError();
  }
  size_t t1 = tb;
  if (e == cudaSuccess)
    e = cub::DeviceRadixSort::SortPairs(tmp, t1, keys, keys2, slots, slots2, (int)n, 0, 64, st);
  if (e == cudaSuccess) {
    k_edge_heads<<<g, 256, 0, st>>>(keys2, n, head);
    e = cudaGetLastError();
  }
  size_t t2 = tb;
  if (e == cudaSuccess) e = cub::DeviceScan::InclusiveSum(tmp, t2, head, id, (int)n, st);
  int32_t ne = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&ne, id + (n - 1), sizeof(ne), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e == cudaSuccess) e = cudaMalloc((void**)edge, sizeof(double) * 6 * (size_t)ne);
  if (e == cudaSuccess) e = cudaMalloc((void**)tet_edge, sizeof(int32_t) * (size_t)n);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&lo, sizeof(int32_t) * (size_t)ne, st);
  if (e == cudaSuccess) {
    k_edge_data<<<g, 256, 0, st>>>(keys2, head, id, n, xyz, *edge, lo);
    k_edge_scatter<<<g, 256, 0, st>>>(slots2, id, n, conn, lo, *tet_edge);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  for (void* p : {(void*)keys, (void*)keys2, (void*)slots, (void*)slots2, (void*)head, (void*)id,
                  tmp, (void*)lo})
    if (p) cudaFreeAsync(p, st);
  cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    if (*edge) cudaFree(*edge);
    if (*tet_edge) cudaFree(*tet_edge);
    *edge = nullptr;
    *tet_edge = nullptr;
    return e;
  }
  *n_edges = ne;
  return cudaSuccess;
}

size_t walk_order_scratch_bytes(int64_t n) {
  size_t tmp = 0;
  cub::DeviceRadixSort::SortPairsDescending(nullptr, tmp, (const double*)nullptr, (double*)nullptr,
                                            (const int32_t*)nullptr, (int32_t*)nullptr, (int)n);
  return ((tmp + 255) & ~(size_t)255) + ((sizeof(double) * n + 255) & ~(size_t)255) +
         ((sizeof(int32_t) * n + 255) & ~(size_t)255);
}

cudaError_t walk_order(const double* dist, int64_t n, int32_t* order, void* scratch,
                       size_t scratch_bytes, cudaStream_t st) {
  size_t tmp = 0;
  cudaError_t e = cub::DeviceRadixSort::SortPairsDescending(
      nullptr, tmp, (const double*)nullptr, (double*)nullptr, (const int32_t*)nullptr,
      (int32_t*)nullptr, (int)n, 0, 64, st);
  if (e != cudaSuccess) return e;
  char* p = (char*)scratch;
  const size_t tmp_al = (tmp + 255) & ~(size_t)255;
  double* keys_out = (double*)(p + tmp_al);
  int32_t* idx = (int32_t*)(p + tmp_al + ((sizeof(double) * n + 255) & ~(size_t)255));
  if (tmp_al + ((sizeof(double) * n + 255) & ~(size_t)255) + sizeof(int32_t) * n > scratch_bytes)
    return cudaErrorInvalidValue;
  k_iota<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(idx, n);
  return cub::DeviceRadixSort::SortPairsDescending(p, tmp, dist, keys_out, idx, order, (int)n, 0,
                                                   64, st);
}

cudaError_t scan_offsets(int64_t* offsets, int64_t n, int64_t* block_sums, cudaStream_t st) {
  if (n <= 0) return cudaMemsetAsync(offsets, 0, sizeof(int64_t), st);
  const int64_t nb = (n + kScanBlock - 1) / kScanBlock;
  k_block_sums<<<(unsigned)nb, kScanBlock, 0, st>>>(offsets, n, block_sums);
  k_scan_sums<<<1, kScanBlock, 0, st>>>(block_sums, nb);
  k_scan_apply<<<(unsigned)nb, kScanBlock, 0, st>>>(offsets, n, block_sums, nb);
  return cudaGetLastError();
}

cudaError_t launch_next_element(bool mixed, int face_order, const WalkArgs& a, cudaStream_t st) {
  if (a.n <= 0) return cudaSuccess;
  const unsigned g = (unsigned)((a.n + kBlock - 1) / kBlock);
  const int sel = (face_order == 0 ? 0 : 2) + (mixed ? 1 : 0);
  switch (sel) {
    case 0: k_next<0, false><<<g, kBlock, 0, st>>>(a); break;
    case 1: k_next<0, true><<<g, kBlock, 0, st>>>(a); break;
    case 2: k_next<1, false><<<g, kBlock, 0, st>>>(a); break;
    default: k_next<1, true><<<g, kBlock, 0, st>>>(a); break;
  }
  return cudaGetLastError();
}

}  // namespace xdgcu
