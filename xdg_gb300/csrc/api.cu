// api.cu -- the C ABI declared in include/xdgcu.h.
//
// A context owns every device copy of the geometry: the registered surface
// triangles (FP64, mesh vertex order), the tet mesh (FP64 + FP32 vertices,
// connectivity, adjacency), and one 4-wide BVH per tree with its primitives
// re-laid out in leaf order.  Callers keep ownership of their own arrays; they
// are only read during the call.
//
// Query calls accept device pointers (enqueued on the caller's stream, no
// synchronisation) or host pointers (staged through a per-thread device
// workspace and stream, synchronised before returning), so the scalar,
// one-ray-per-call use of the reference API can run concurrently from many
// host threads.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <chrono>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/xdgcu.h"
#include "bvh.h"
#include "cbound.h"
#include "queries.h"
#include "segments.h"
#include "walk.h"

using namespace xdgcu;

namespace {

thread_local std::string g_last_error;

struct SurfaceRec {
  int32_t id;
  int64_t first;
  int64_t count;
  int32_t fwd_tree = -1;
  int32_t rev_tree = -1;
  int32_t bc = 0;  // boundary condition for the particle loop (xdgcu_set_surface_boundary)
  double bump = 0.0;
};

struct TreeHost {
  int32_t id = -1;
  int32_t kind = TREE_SURFACE;
  Node32* n32 = nullptr;
  Node64* n64 = nullptr;
  DevMem<float4> prim32;
  DevMem<double> prim64;
  DevMem<int32_t> prim_ref;
  int32_t n_nodes = 0;
  int32_t depth = 0;
  TreeDev dev{};
  std::vector<int32_t> members;  // surfaces (surface tree) or tet indices (element tree)
  double bump_arg = 0.0;         // surface trees: the bump the tree was created with
  ~TreeHost() {
    if (n32) cudaFree(n32);
    if (n64) cudaFree(n64);
  }
};

// Per-host-thread staging state for calls with host arrays: a device
// workspace, the compute stream, two copy streams and chunk events, so that
// host->device copies, kernels and device->host copies of consecutive chunks
// overlap.
struct Slot {
  cudaStream_t stream = nullptr;    // compute
  cudaStream_t stream2 = nullptr;   // compute, odd chunks of a staged call
  cudaStream_t copy_in = nullptr;
  cudaStream_t copy_out = nullptr;
  std::vector<cudaEvent_t> ev;
  DevMem<char> buf;
  ~Slot() {
    for (cudaEvent_t e : ev) cudaEventDestroy(e);
    if (stream) cudaStreamDestroy(stream);
    if (stream2) cudaStreamDestroy(stream2);
    if (copy_in) cudaStreamDestroy(copy_in);
    if (copy_out) cudaStreamDestroy(copy_out);
  }
  bool events(size_t k) {
    while (ev.size() < k) {
      cudaEvent_t e;
      if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return false;
      ev.push_back(e);
    }
    return true;
  }
};

int set_err(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

int cuda_err(cudaError_t e, const char* what) {
  return set_err(XDGCU_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define API_CUDA(x, what)                         \
  do {                                            \
    cudaError_t e_ = (x);                         \
    if (e_ != cudaSuccess) return cuda_err(e_, what); \
  } while (0)

const int32_t kMoabFaces[12] = {0, 1, 3, 1, 2, 3, 2, 0, 3, 0, 2, 1};

// ---------------------------------------------------------------------------
// build-time kernels
// ---------------------------------------------------------------------------

__global__ void k_tri_boxes(const double* __restrict__ tri_xyz, const int32_t* __restrict__ tris,
                            const double* __restrict__ bump, int32_t n, double* __restrict__ box) {
  int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double* v = tri_xyz + 9 * (int64_t)tris[i];
  for (int c = 0; c < 3; ++c) {
    // bbox.h:104-111 + triangle_intersect.cpp:36-50
    const double lo = fmin(fmin(v[c], v[3 + c]), v[6 + c]);
    const double hi = fmax(fmax(v[c], v[3 + c]), v[6 + c]);
    box[6 * (int64_t)i + c] = lo - bump[i];
    box[6 * (int64_t)i + 3 + c] = hi + bump[i];
  }
}

__global__ void k_tri_gather(const double* __restrict__ tri_xyz, const int32_t* __restrict__ tris,
                             const int32_t* __restrict__ order, int32_t n,
                             float4* __restrict__ prim32, double* __restrict__ prim64,
                             int32_t* __restrict__ prim_ref) {
  int32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const int32_t g = tris[order[j]];
  const double* v = tri_xyz + 9 * (int64_t)g;
  double* o = prim64 + kPrim64Stride * (int64_t)j;
  for (int k = 0; k < 9; ++k) o[k] = v[k];
  o[9] = 0.0;
  prim_ref[j] = g;
  const double e1[3] = {v[3] - v[0], v[4] - v[1], v[5] - v[2]};
  const double e2[3] = {v[6] - v[0], v[7] - v[1], v[8] - v[2]};
  double emax = 0.0;
  for (int c = 0; c < 3; ++c) {
    emax = fmax(emax, fabs(e1[c]));
    emax = fmax(emax, fabs(e2[c]));
    emax = fmax(emax, fabs(e2[c] - e1[c]));
  }
  const float v0x = __double2float_rn(v[0]), v0y = __double2float_rn(v[1]),
              v0z = __double2float_rn(v[2]);
  const float v0abs = fmaxf(fabsf(v0x), fmaxf(fabsf(v0y), fabsf(v0z)));
  // the edge bound must cover the exact edges and the FP32 difference of the
  // stored edges, hence the 1 + 2^-20 margin on the upward rounding
  const float emaxf = __double2float_ru(emax * (1.0 + 9.5367431640625e-07));
  prim32[3 * (int64_t)j] = make_float4(v0x, v0y, v0z, v0abs);
  prim32[3 * (int64_t)j + 1] = make_float4(__double2float_rn(e1[0]), __double2float_rn(e1[1]),
                                           __double2float_rn(e1[2]), emaxf);
  // fourth slot: 1 when the triangle is well shaped at v0 for closest's
  // upper bound, |e1 x e2|^2 >= 1e-6 |e1|^2 |e2|^2 (the determinant of
  // closest.cpp:60-65 against its two squared lengths)
  const double ss = e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2];
  const double tt = e2[0] * e2[0] + e2[1] * e2[1] + e2[2] * e2[2];
  const double st = e1[0] * e2[0] + e1[1] * e2[1] + e1[2] * e2[2];
  const double det = ss * tt - st * st;
  const bool shaped = ss * tt > 0.0 && ss * tt < 1e300 && det >= 1e-6 * (ss * tt);
  prim32[3 * (int64_t)j + 2] = make_float4(__double2float_rn(e2[0]), __double2float_rn(e2[1]),
                                           __double2float_rn(e2[2]), shaped ? 1.0f : 0.0f);
}

// Per global triangle (kTriPrimeStride doubles), the ray-independent terms
// of the FP64 test, with the operations of plucker_edge64 and
// normal_dot_sign: for the test edges (v0,v1), (v1,v2), (v2,v0) e = hi - lo
// and e x lo (lo, hi in first() order), both negated when the test runs the
// edge from hi to lo (offsets 0, 6, 12); the normal (v1-v0) x (v2-v0)
// (offset 18); the 9 vertex coordinates (offset 22).  A mixed FP64 test
// reads this one 256-byte record.
__global__ void k_tri_prime(const double* __restrict__ tri_xyz, int64_t n,
                            double* __restrict__ out) {
  const int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (g >= n) return;
  const double* v = tri_xyz + 9 * g;
  const d3 V[3] = {mk3(v[0], v[1], v[2]), mk3(v[3], v[4], v[5]), mk3(v[6], v[7], v[8])};
  double* pe = out + kTriPrimeStride * g;
  for (int k = 0; k < 3; ++k) {
    const d3 va = V[k], vb = V[(k + 1) % 3];
    const bool f = first_lower(va, vb);
    const d3 lo = f ? va : vb;
    const d3 hi = f ? vb : va;
    d3 e = sub3(hi, lo);
    d3 en = cross3(e, lo);
    if (!f) {
      e = mk3(-e.x, -e.y, -e.z);
      en = mk3(-en.x, -en.y, -en.z);
    }
    pe[6 * k] = e.x;
    pe[6 * k + 1] = e.y;
    pe[6 * k + 2] = e.z;
    pe[6 * k + 3] = en.x;
    pe[6 * k + 4] = en.y;
    pe[6 * k + 5] = en.z;
  }
  const d3 c = cross3(sub3(V[1], V[0]), sub3(V[2], V[0]));
  pe[18] = c.x;
  pe[19] = c.y;
  pe[20] = c.z;
  pe[21] = 0.0;
  for (int k = 0; k < 9; ++k) pe[22 + k] = v[k];
  pe[31] = 0.0;
}

// closest's bound planes (PointArgs::tri_cb), certified against each
// triangle's vertices (tri_cbound)
__global__ void k_tri_cbound(const double* __restrict__ tri_xyz, int64_t n,
                             float4* __restrict__ out) {
  const int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (g >= n) return;
  float r[16];
  tri_cbound(tri_xyz + 9 * g, r);
  for (int k = 0; k < 4; ++k) out[4 * g + k] = make_float4(r[4 * k], r[4 * k + 1], r[4 * k + 2], r[4 * k + 3]);
}

__global__ void k_tet_boxes(const double* __restrict__ xyz, const int4* __restrict__ conn,
                            const int32_t* __restrict__ tets, int32_t n, double* __restrict__ box) {
  int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int4 c = conn[tets[i]];
  const int32_t ci[4] = {c.x, c.y, c.z, c.w};
  double lo[3], hi[3];
  for (int a = 0; a < 3; ++a) {
    lo[a] = INFINITY;
    hi[a] = -INFINITY;
  }
  for (int k = 0; k < 4; ++k)
    for (int a = 0; a < 3; ++a) {
      const double x = xyz[3 * (int64_t)ci[k] + a];
      lo[a] = fmin(lo[a], x);
      hi[a] = fmax(hi[a], x);
    }
  // bbox.h:85-102: dilation = |width| * FP_BOX_TOL (tetrahedron_contain.cpp:47-63)
  const double wx = hi[0] - lo[0], wy = hi[1] - lo[1], wz = hi[2] - lo[2];
  const double bump = sqrt(wx * wx + wy * wy + wz * wz) * 1e-6;
  for (int a = 0; a < 3; ++a) {
    box[6 * (int64_t)i + a] = lo[a] - bump;
    box[6 * (int64_t)i + 3 + a] = hi[a] + bump;
  }
}

// Leaf-ordered tet data.  prim64: the 4 vertices (12 doubles).  prim32: the
// data of the FP32 containment pre-filter (geom.cuh, tet_filter32):
//   float4 (v0.xyz, m)  (M row 0, |v0|_inf)  (M row 1, e64)  (M row 2, 0)
// with M = T^{-1} (T's columns v1-v0, v2-v0, v3-v0) rounded to FP32,
// m >= max row |.|_1 of M, and e64 a bound on the error of the reference's
// FP64 barycentric coordinates for any point in the tet's box (+inf for
// degenerate or badly conditioned tets, which then always take the FP64 test).
__global__ void k_tet_gather(const double* __restrict__ xyz, const int4* __restrict__ conn,
                             const int32_t* __restrict__ tets, const int32_t* __restrict__ order,
                             int32_t n, double* __restrict__ prim64, float4* __restrict__ prim32,
                             int32_t* __restrict__ prim_ref) {
  int32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const int32_t t = tets[order[j]];
  const int4 c = conn[t];
  const int32_t ci[4] = {c.x, c.y, c.z, c.w};
  double v[4][3];
  double* o = prim64 + 12 * (int64_t)j;
  for (int k = 0; k < 4; ++k)
    for (int a = 0; a < 3; ++a) {
      v[k][a] = xyz[3 * (int64_t)ci[k] + a];
      o[3 * k + a] = v[k][a];
    }
  prim_ref[j] = t;
  // T[r][col]: column col = v_{col+1} - v0
  double T[3][3], Tmax = 0.0, lo[3], hi[3];
  for (int r = 0; r < 3; ++r) {
    lo[r] = fmin(fmin(v[0][r], v[1][r]), fmin(v[2][r], v[3][r]));
    hi[r] = fmax(fmax(v[0][r], v[1][r]), fmax(v[2][r], v[3][r]));
    for (int col = 0; col < 3; ++col) {
      T[r][col] = v[col + 1][r] - v[0][r];
      Tmax = fmax(Tmax, fabs(T[r][col]));
    }
  }
  const double det = T[0][0] * (T[1][1] * T[2][2] - T[1][2] * T[2][1]) -
                     T[0][1] * (T[1][0] * T[2][2] - T[1][2] * T[2][0]) +
                     T[0][2] * (T[1][0] * T[2][1] - T[1][1] * T[2][0]);
  double M[3][3];
  M[0][0] = (T[1][1] * T[2][2] - T[1][2] * T[2][1]) / det;
  M[0][1] = (T[0][2] * T[2][1] - T[0][1] * T[2][2]) / det;
  M[0][2] = (T[0][1] * T[1][2] - T[0][2] * T[1][1]) / det;
  M[1][0] = (T[1][2] * T[2][0] - T[1][0] * T[2][2]) / det;
  M[1][1] = (T[0][0] * T[2][2] - T[0][2] * T[2][0]) / det;
  M[1][2] = (T[0][2] * T[1][0] - T[0][0] * T[1][2]) / det;
  M[2][0] = (T[1][0] * T[2][1] - T[1][1] * T[2][0]) / det;
  M[2][1] = (T[0][1] * T[2][0] - T[0][0] * T[2][1]) / det;
  M[2][2] = (T[0][0] * T[1][1] - T[0][1] * T[1][0]) / det;
  double m = 0.0;
  for (int r = 0; r < 3; ++r) m = fmax(m, fabs(M[r][0]) + fabs(M[r][1]) + fabs(M[r][2]));
  // largest |p - v0|_inf for p in the (dilated) box
  double rmax = 0.0;
  for (int r = 0; r < 3; ++r) rmax = fmax(rmax, fmax(fabs(hi[r] - v[0][r]), fabs(v[0][r] - lo[r])));
  const double w = sqrt((hi[0] - lo[0]) * (hi[0] - lo[0]) + (hi[1] - lo[1]) * (hi[1] - lo[1]) +
                        (hi[2] - lo[2]) * (hi[2] - lo[2]));
  rmax += 2.0 * w * 1e-6 + 1e-300;
  const double krel = Tmax * Tmax * Tmax / fabs(det);
  const double eps = DBL_EPSILON;
  // error of adjugate/determinant barycentrics, see tet_filter32
  double e64 = 3.0 * eps * rmax * (18.0 * krel / Tmax + 47.0 * krel * m) +
               3.0 * eps * (1.0 + 3.0 * m * rmax);
  e64 *= 2.0;
  const bool ok = det > 0.0 && isfinite(det) && m < 1e20 && krel < 1e6 && isfinite(e64);
  const float mf = ok ? __double2float_ru(m * (1.0 + 1e-6)) : INFINITY;
  const float ef = ok ? __double2float_ru(e64) : INFINITY;
  const float v0x = __double2float_rn(v[0][0]), v0y = __double2float_rn(v[0][1]),
              v0z = __double2float_rn(v[0][2]);
  const float v0abs = fmaxf(fabsf(v0x), fmaxf(fabsf(v0y), fabsf(v0z)));
  float4* q = prim32 + 4 * (int64_t)j;
  q[0] = make_float4(v0x, v0y, v0z, mf);
  q[1] = make_float4(__double2float_rn(M[0][0]), __double2float_rn(M[0][1]),
                     __double2float_rn(M[0][2]), v0abs);
  q[2] = make_float4(__double2float_rn(M[1][0]), __double2float_rn(M[1][1]),
                     __double2float_rn(M[1][2]), ef);
  q[3] = make_float4(__double2float_rn(M[2][0]), __double2float_rn(M[2][1]),
                     __double2float_rn(M[2][2]), 0.0f);
}

__global__ void k_vert32(const double* __restrict__ xyz, int64_t n, float4* __restrict__ out) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float x = __double2float_rn(xyz[3 * i]), y = __double2float_rn(xyz[3 * i + 1]),
              z = __double2float_rn(xyz[3 * i + 2]);
  out[i] = make_float4(x, y, z, fmaxf(fabsf(x), fmaxf(fabsf(y), fabsf(z))));
}

inline unsigned grid(int64_t n, int b = 256) { return (unsigned)((n + b - 1) / b); }

bool is_device_ptr(const void* p) {
  if (!p) return false;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

}  // namespace

struct xdgcu_ctx {
  int device = 0;
  std::mutex mu;
  // surfaces
  std::vector<SurfaceRec> surfs;
  std::unordered_map<int32_t, int32_t> surf_index;
  std::vector<double> h_tri_xyz;
  std::vector<int32_t> h_tri_face, h_tri_surf;
  DevMem<double> d_tri_xyz;
  DevMem<int32_t> d_tri_face, d_tri_surf, d_surf_id, d_surf_rev, d_surf_fwd, d_surf_bc;
  DevMem<double> d_tri_prime;  // kTriPrimeStride doubles per triangle (k_tri_prime)
  DevMem<float4> d_tri_cb;     // 4 per triangle: closest's FP32 bound planes (k_tri_cbound)
  bool tri_dirty = true, surf_dirty = true;
  // tet mesh
  bool has_tets = false;
  int64_t n_vert = 0, n_tet = 0;
  DevMem<double> d_xyz;
  DevMem<float4> d_xyz32;
  DevMem<int4> d_conn, d_adj;
  // edge table for the mixed walk's FP64 face tests (build_edge_table)
  DevMem<double> d_edge;
  DevMem<int32_t> d_tet_edge;
  int64_t n_edges = 0;
  DevMem<int32_t> d_elem_ids;
  int32_t face[12] = {0};
  int face_order = 0;
  // MeshManager::get_boundary_face_element for the global track loop:
  // ascending face ids and the tet index behind each
  DevMem<int32_t> d_bfe_face, d_bfe_elem;
  int64_t n_bfe = 0;
  // trees
  std::vector<std::unique_ptr<TreeHost>> surf_trees, elem_trees;
  DevMem<TreeDev> d_surf_trees, d_elem_trees;
  bool surf_trees_dirty = true, elem_trees_dirty = true;
  // volume -> surface tree map for find_volume (xdgcu_set_volume_map)
  DevMem<int32_t> d_vol_ids, d_vol_trees;
  int32_t n_vols = 0;
  int32_t ipc_volume = -1;
  bool has_volume_map = false;
  // tuning (xdgcu_set_tuning)
  int32_t trace_occupancy = 4;
  int32_t trace_node_iters = 4;       // mixed precision
  int32_t trace_node_iters_fp64 = 1;  // all-FP64 path
  int32_t trace_node_iters_direct = 6;  // mixed launches reading their rays in place from host memory
  int32_t trace_flush_wait = 4;
  int32_t trace_stack = 40;      // shared-memory stack entries per lane
  int32_t trace_grab = 0;        // 0: one contiguous chunk per warp; > 0: device work queue
  int64_t trace_sort_min = 0;    // batches of at least this many rays run in coherent order (0 = never)
  int32_t surf_stack_bound = 0;       // largest (width - 1) * depth of the surface trees
  int32_t particle_event_wait = 16;  // particle_sim loop: lanes gathered before their events run
  int32_t transport_event_wait = 4;  // walk_elements tool loop (mixed): the same
  int32_t leaf_max = 2;
  int32_t node_width = 4;        // children per BVH node (4 or 8) of trees built afterwards
  int32_t bvh_sah = 1;           // trees built afterwards: SAH collapse (1) or greedy (0)
  int32_t bvh_prim_cost = 300;   // SAH: primitive test / wide-node visit, in thousandths
  int32_t walk_queue = 0;
  int32_t walk_flush_wait = 8;
  // host arrays the kernels address directly instead of staging them:
  // 0 none, 1 page-locked memory, 2 also pageable memory when the device
  // reads it through the host's page tables (pageable_direct), 3 / 4 stage
  // all / the outputs of large calls' page-locked arrays, 5 (default) picks
  // 2, 3 or 4 for large calls by timing each (xdgcu_set_tuning)
  int32_t host_direct = 5;
  int32_t walk_edge_table = 1;  // mixed walk: FP64 edge coordinates from the edge table
  int32_t trace_edge_table = 1;  // mixed traversal: FP64 triangle terms from d_tri_prime
  int32_t closest_bound = 1;     // mixed closest: FP32 triangle bound from d_tri_cb
  int32_t closest_node_steps = 4;       // closest: inner-node steps between leaf phases (mixed)
  int32_t closest_node_steps_fp64 = 1;  // the same, all-FP64 path
  int32_t find_node_steps_fp64 = 16;    // find_element in phases (all-FP64, or find_phased): the same
  int32_t find_phased = 0;  // mixed find_element: 1 runs warp-synchronous phases, 0 one lane per point
  int32_t packed_passes = 1;  // packed walk: 1 walk in resumed rounds, 2 a count walk and an emit walk
  int32_t closest_budget = 1024;  // closest: steps of one lane before a warp takes the point (0: never)
  int64_t closest_sort_min = 65536;  // closest: batches of at least this many points run in Morton order (0 = never)
  int64_t find_sort_min = 65536;  // find_element: the same
  int32_t segments_walk_cap = 0;  // segments_global: segments per walk and round (0 = automatic)
  bool pageable_direct = false;
  // host_direct 5: trial calls of the policies kAutoPolicies (in place,
  // staged, inputs in place with outputs staged), their summed seconds per
  // ray, and the policy chosen (-1 until each has kAutoTrials)
  std::mutex hd_mu;
  int32_t hd_trials = 0;
  int32_t hd_timed[3] = {0, 0, 0};
  double hd_sec_per_ray[3] = {0.0, 0.0, 0.0};
  int32_t hd_choice = -1;
  int64_t walk_sort_min = 16384;  // tracks; 0 disables the length order
  // diagnostics
  bool counting = false;
  DevMem<unsigned long long> d_counters;
  cudaStream_t counter_stream = nullptr;
  // per-thread staging for host-pointer calls
  std::mutex slot_mu;
  std::unordered_map<std::thread::id, std::unique_ptr<Slot>> slots;
  cudaStream_t build_stream = nullptr;
  // the calls' stream-ordered scratch comes from this pool, which keeps up to
  // keep_bytes of freed memory for later calls instead of returning it to the
  // driver at each synchronisation as the device's default pool does (the
  // global track loop on 1e6 tracks: 36.7 -> 33.0 ms); null: the default pool
  cudaMemPool_t pool = nullptr;
  int64_t keep_bytes = int64_t(8) << 30;
};

namespace {

// Stream-ordered scratch of a call, from the context's pool.
cudaError_t scratch_alloc(const xdgcu_ctx* c, void** p, size_t bytes, cudaStream_t s) {
  return c->pool ? cudaMallocFromPoolAsync(p, bytes, c->pool, s) : cudaMallocAsync(p, bytes, s);
}

int sync_surfaces(xdgcu_ctx* c) {
  if (c->tri_dirty) {
    const int64_t nt = (int64_t)c->h_tri_face.size();
    API_CUDA(c->d_tri_xyz.alloc(std::max<int64_t>(1, 9 * nt)), "alloc triangles");
    API_CUDA(c->d_tri_face.alloc(std::max<int64_t>(1, nt)), "alloc face ids");
    API_CUDA(c->d_tri_surf.alloc(std::max<int64_t>(1, nt)), "alloc surface index");
    if (nt) {
      API_CUDA(cudaMemcpy(c->d_tri_xyz.p, c->h_tri_xyz.data(), sizeof(double) * 9 * nt,
                          cudaMemcpyHostToDevice), "upload triangles");
      API_CUDA(cudaMemcpy(c->d_tri_face.p, c->h_tri_face.data(), sizeof(int32_t) * nt,
                          cudaMemcpyHostToDevice), "upload face ids");
      API_CUDA(cudaMemcpy(c->d_tri_surf.p, c->h_tri_surf.data(), sizeof(int32_t) * nt,
                          cudaMemcpyHostToDevice), "upload surface index");
      API_CUDA(c->d_tri_prime.alloc(kTriPrimeStride * nt), "alloc triangle terms");
      k_tri_prime<<<grid(nt), 256, 0, c->build_stream>>>(c->d_tri_xyz.p, nt, c->d_tri_prime.p);
      API_CUDA(cudaGetLastError(), "triangle terms");
      API_CUDA(c->d_tri_cb.alloc(4 * nt), "alloc triangle bound planes");
      k_tri_cbound<<<grid(nt), 256, 0, c->build_stream>>>(c->d_tri_xyz.p, nt, c->d_tri_cb.p);
      API_CUDA(cudaGetLastError(), "triangle bound planes");
      API_CUDA(cudaStreamSynchronize(c->build_stream), "triangle terms");
    }
    c->tri_dirty = false;
  }
  if (c->surf_dirty) {
    const int64_t ns = (int64_t)c->surfs.size();
    const size_t m = (size_t)std::max<int64_t>(1, ns);
    std::vector<int32_t> ids(m), rev(m), fwd(m), bc(m);
    for (int64_t s = 0; s < ns; ++s) {
      ids[s] = c->surfs[s].id;
      rev[s] = c->surfs[s].rev_tree;
      fwd[s] = c->surfs[s].fwd_tree;
      bc[s] = c->surfs[s].bc;
    }
    API_CUDA(c->d_surf_id.alloc((int64_t)m), "alloc surfaces");
    API_CUDA(c->d_surf_rev.alloc((int64_t)m), "alloc surfaces");
    API_CUDA(c->d_surf_fwd.alloc((int64_t)m), "alloc surfaces");
    API_CUDA(c->d_surf_bc.alloc((int64_t)m), "alloc surfaces");
    API_CUDA(cudaMemcpy(c->d_surf_id.p, ids.data(), sizeof(int32_t) * m, cudaMemcpyHostToDevice),
             "upload surfaces");
    API_CUDA(cudaMemcpy(c->d_surf_rev.p, rev.data(), sizeof(int32_t) * m, cudaMemcpyHostToDevice),
             "upload surfaces");
    API_CUDA(cudaMemcpy(c->d_surf_fwd.p, fwd.data(), sizeof(int32_t) * m, cudaMemcpyHostToDevice),
             "upload surfaces");
    API_CUDA(cudaMemcpy(c->d_surf_bc.p, bc.data(), sizeof(int32_t) * m, cudaMemcpyHostToDevice),
             "upload surfaces");
    c->surf_dirty = false;
  }
  return XDGCU_OK;
}

int sync_tree_tables(xdgcu_ctx* c) {
  if (c->surf_trees_dirty) {
    std::vector<TreeDev> t;
    c->surf_stack_bound = 0;
    for (auto& p : c->surf_trees) {
      t.push_back(p->dev);
      // a traversal holds at most (width - 1) entries per inner level
      c->surf_stack_bound = std::max(c->surf_stack_bound, (p->dev.width - 1) * p->depth);
    }
    if (t.empty()) t.push_back(TreeDev{});
    API_CUDA(c->d_surf_trees.alloc((int64_t)t.size()), "alloc tree table");
    API_CUDA(cudaMemcpy(c->d_surf_trees.p, t.data(), sizeof(TreeDev) * t.size(),
                        cudaMemcpyHostToDevice), "upload tree table");
    c->surf_trees_dirty = false;
  }
  if (c->elem_trees_dirty) {
    std::vector<TreeDev> t;
    for (auto& p : c->elem_trees) t.push_back(p->dev);
    if (t.empty()) t.push_back(TreeDev{});
    API_CUDA(c->d_elem_trees.alloc((int64_t)t.size()), "alloc tree table");
    API_CUDA(cudaMemcpy(c->d_elem_trees.p, t.data(), sizeof(TreeDev) * t.size(),
                        cudaMemcpyHostToDevice), "upload tree table");
    c->elem_trees_dirty = false;
  }
  return XDGCU_OK;
}

void fill_dev(TreeHost& t, const BuiltTree& b, double min_bump) {
  t.n32 = b.n32;
  t.n64 = b.n64;
  t.n_nodes = b.n_nodes;
  t.depth = b.depth;
  TreeDev& d = t.dev;
  d.n32 = b.n32;
  d.n64 = b.n64;
  d.prim32 = t.prim32.p;
  d.prim64 = t.prim64.p;
  d.prim_ref = t.prim_ref.p;
  d.root = b.root;
  d.n_prims = (int32_t)t.prim_ref.n;
  d.depth = b.depth;
  d.tree_id = t.id;
  d.kind = t.kind;
  d.width = b.width;
  double m = 0.0;
  for (int k = 0; k < 6; ++k) m = std::max(m, std::fabs(b.bounds[k]));
  d.max_abs = (float)(m * (1.0 + 1e-6));
  // FP32 safety check compares against the smallest dilation in the tree
  float bf = (float)min_bump;
  if ((double)bf > min_bump) bf = std::nextafter(bf, 0.0f);
  d.bump = bf;
}

// Build the BVH over `tris` (global triangle indices) with per-triangle bumps.
int build_surface_bvh(xdgcu_ctx* c, TreeHost& t, const std::vector<int32_t>& tris,
                      const std::vector<double>& bumps) {
  const int32_t n = (int32_t)tris.size();
  cudaStream_t st = c->build_stream;
  DevMem<int32_t> d_tris(std::max(1, n));
  DevMem<double> d_bump(std::max(1, n)), d_box(6 * (int64_t)std::max(1, n));
  API_CUDA(d_tris.alloc(), "alloc");
  API_CUDA(d_bump.alloc(), "alloc");
  API_CUDA(d_box.alloc(), "alloc");
  double min_bump = INFTY;
  for (double b : bumps) min_bump = std::min(min_bump, b);
  if (n > 0) {
    API_CUDA(cudaMemcpyAsync(d_tris.p, tris.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, st),
             "upload");
    API_CUDA(cudaMemcpyAsync(d_bump.p, bumps.data(), sizeof(double) * n, cudaMemcpyHostToDevice, st),
             "upload");
    k_tri_boxes<<<grid(n), 256, 0, st>>>(c->d_tri_xyz.p, d_tris.p, d_bump.p, n, d_box.p);
    API_CUDA(cudaGetLastError(), "triangle boxes");
  }
  BuiltTree b;
  const BvhCost cost{1.0, c->bvh_prim_cost * 1e-3};
  API_CUDA(build_wide_bvh(d_box.p, n, c->leaf_max, c->node_width, c->bvh_sah ? &cost : nullptr,
                          st, &b),
           "bvh build");
  API_CUDA(t.prim32.alloc(3 * (int64_t)std::max(1, n)), "alloc prims");
  API_CUDA(t.prim64.alloc(kPrim64Stride * (int64_t)std::max(1, n)), "alloc prims");
  API_CUDA(t.prim_ref.alloc(std::max(1, n)), "alloc prims");
  if (n > 0) {
    k_tri_gather<<<grid(n), 256, 0, st>>>(c->d_tri_xyz.p, d_tris.p, b.order, n, t.prim32.p,
                                          t.prim64.p, t.prim_ref.p);
    API_CUDA(cudaGetLastError(), "gather");
  }
  API_CUDA(cudaStreamSynchronize(st), "build sync");
  if (b.order) cudaFree(b.order);
  t.prim_ref.n = n;
  fill_dev(t, b, n > 0 ? min_bump : 1e-3);
  return XDGCU_OK;
}

int build_element_bvh(xdgcu_ctx* c, TreeHost& t, const std::vector<int32_t>& tets) {
  const int32_t n = (int32_t)tets.size();
  cudaStream_t st = c->build_stream;
  DevMem<int32_t> d_tets(std::max(1, n));
  DevMem<double> d_box(6 * (int64_t)std::max(1, n));
  API_CUDA(d_tets.alloc(), "alloc");
  API_CUDA(d_box.alloc(), "alloc");
  if (n > 0) {
    API_CUDA(cudaMemcpyAsync(d_tets.p, tets.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, st),
             "upload");
    k_tet_boxes<<<grid(n), 256, 0, st>>>(c->d_xyz.p, c->d_conn.p, d_tets.p, n, d_box.p);
    API_CUDA(cudaGetLastError(), "tet boxes");
  }
  BuiltTree b;
  const BvhCost cost{1.0, c->bvh_prim_cost * 1e-3};
  API_CUDA(build_wide_bvh(d_box.p, n, c->leaf_max, c->node_width, c->bvh_sah ? &cost : nullptr,
                          st, &b),
           "bvh build");
  API_CUDA(t.prim64.alloc(12 * (int64_t)std::max(1, n)), "alloc prims");
  API_CUDA(t.prim32.alloc(4 * (int64_t)std::max(1, n)), "alloc prims");
  API_CUDA(t.prim_ref.alloc(std::max(1, n)), "alloc prims");
  if (n > 0) {
    k_tet_gather<<<grid(n), 256, 0, st>>>(c->d_xyz.p, c->d_conn.p, d_tets.p, b.order, n,
                                          t.prim64.p, t.prim32.p, t.prim_ref.p);
    API_CUDA(cudaGetLastError(), "gather");
  }
  API_CUDA(cudaStreamSynchronize(st), "build sync");
  if (b.order) cudaFree(b.order);
  t.prim_ref.n = n;
  fill_dev(t, b, 0.0);
  return XDGCU_OK;
}

// ---------------------------------------------------------------------------
// host/device staging
// ---------------------------------------------------------------------------

struct Arr {
  const void* host_in = nullptr;  // input to copy H2D
  void* host_out = nullptr;       // output to copy D2H
  size_t bytes = 0;
  void* dev = nullptr;
  bool no_direct = false;  // kernels update it atomically: always staged
  bool direct = false;     // dev is the host array's own device address
};

// The device address of host array p when the kernels read and write it in
// place (page-locked memory mapped into the device's address space, or
// pageable memory on a device that walks the host's page tables), else
// nullptr: the array is staged.  In-place access moves each byte over the
// host link once, inside the kernel, with no staging copies or chunking.
// `pipelined`: the call is large enough for the staged chunk pipeline to
// overlap its copies with compute; under host_direct 3 page-locked arrays
// are staged then, under host_direct 4 only its outputs (`input` false).
// `hd` is the policy in force for the call (host_direct, or under 5 the
// policy the automatic choice picked for it).  Measured on ray_fire over
// 1e7 host rays with the bench's launch settings, the policies interleaved
// in one process (medians of 24 calls each): page-locked in place 8.14 ms,
// staged 7.44 ms, inputs in place and outputs staged 7.65 ms, against 6.73
// ms for device arrays; with the default launch settings in place was ahead
// (7.55 against 7.70 ms), hence the automatic choice.
void* direct_ptr(const xdgcu_ctx* c, const void* p, bool pipelined, bool input = true,
                 int hd = -1) {
  if (hd < 0) hd = c->host_direct == 5 ? 2 : c->host_direct;
  if (!p || hd <= 0) return nullptr;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (at.type == cudaMemoryTypeHost) {
    const bool staged = pipelined && (hd == 3 || (hd == 4 && !input));
    return staged ? nullptr : at.devicePointer;
  }
  if (at.type == cudaMemoryTypeUnregistered && hd >= 2 && c->pageable_direct)
    return const_cast<void*>(p);
  return nullptr;
}

// Marks the arrays the kernels address in place (direct_ptr); an array that
// is both read and written must be addressable for both.
void resolve_direct(const xdgcu_ctx* c, Arr* a, bool pipelined = false, int hd = -1) {
  if (a->no_direct || a->bytes == 0) return;
  const void* p = a->host_in ? a->host_in : a->host_out;
  if (!p || (a->host_in && a->host_out && a->host_in != a->host_out)) return;
  void* d = direct_ptr(c, p, pipelined, true, hd);
  if (d) {
    a->dev = d;
    a->direct = true;
  }
}

// Decide the pointer kind of a call: 1 device, 0 host, -1 mixed (error).
int classify(std::initializer_list<const void*> ptrs) {
  int kind = -2;
  for (const void* p : ptrs) {
    if (!p) continue;
    const int k = is_device_ptr(p) ? 1 : 0;
    if (kind == -2) kind = k;
    else if (kind != k) return -1;
  }
  return kind == -2 ? 1 : kind;
}

Slot* get_slot(xdgcu_ctx* c) {
  std::lock_guard<std::mutex> g(c->slot_mu);
  auto& s = c->slots[std::this_thread::get_id()];
  if (!s) {
    s.reset(new Slot());
    if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&s->stream2, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&s->copy_in, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&s->copy_out, cudaStreamNonBlocking) != cudaSuccess) {
      s.reset();
      return nullptr;
    }
  }
  return s.get();
}

// Allocate device images of the arrays in the slot's workspace, upload inputs.
int stage_in(const xdgcu_ctx* c, Slot* s, std::vector<Arr*> arrs, cudaStream_t st) {
  size_t total = 0;
  for (Arr* a : arrs) {
    resolve_direct(c, a);
    if (!a->direct) total += (a->bytes + 255) & ~(size_t)255;
  }
  if ((int64_t)total > s->buf.n) {
    API_CUDA(s->buf.alloc((int64_t)std::max<size_t>(total, 1 << 20)), "workspace");
  }
  size_t off = 0;
  for (Arr* a : arrs) {
    if (a->bytes == 0 || a->direct) continue;
    a->dev = s->buf.p + off;
    off += (a->bytes + 255) & ~(size_t)255;
    if (a->host_in)
      API_CUDA(cudaMemcpyAsync(a->dev, a->host_in, a->bytes, cudaMemcpyHostToDevice, st), "H2D");
  }
  return XDGCU_OK;
}

// A per-ray array of a host call: `per_ray` bytes for each of the n rays.
struct RayArr {
  const void* host_in = nullptr;
  void* host_out = nullptr;
  size_t per_ray = 0;
  char* dev = nullptr;
  bool direct = false;  // dev is the host array's own device address
};

// Staged calls run in chunks of this many rays, at most kMaxChunks: 2^21 per
// chunk ran ray_fire over 1e7 host rays in 10.1 ms, 2^20 in 10.7 ms and 2^19
// in 12.6 ms with one launch stream (each chunk's launch ends with a tail of
// a few slow rays); two alternating streams overlap those tails.
constexpr int64_t kChunkRays = 1 << 21;
constexpr int64_t kMaxChunks = 16;
// host_direct 5: timed calls of each policy before the choice
constexpr int kAutoTrials = 2;
// host_direct 5: the policies it chooses among (the fastest differed from one
// GB300 machine to another: staged on some, in place or inputs in place with
// outputs staged on others)
constexpr int kAutoPolicies[3] = {2, 3, 4};
// work-queue grab of a chunk's traversal launch (when a call runs in chunks)
constexpr int32_t kChunkGrab = 64;

// Runs a per-ray query over host arrays in chunks: the inputs of chunk k+1
// are copied in while chunk k computes and chunk k-1 is copied out.  `whole`
// arrays (exclusion lists) are copied once before the first chunk.
// launch(first, count, stream) enqueues the kernel for rays [first,
// first+count) with the device pointers of the RayArr entries offset by
// `first`.  Returns when all results are in host memory.
int begin_query(xdgcu_ctx* c, cudaStream_t st, unsigned long long** counters);

template <typename Launch>
int run_staged(xdgcu_ctx* c, Slot* s, cudaStream_t user, int64_t n, std::vector<Arr*> whole,
               std::vector<RayArr*> rays, unsigned long long** counters, Launch launch) {
  // arrays the kernels address in place take no workspace and no copies
  const bool pipelined = n > 2 * kChunkRays;
  // host_direct 5: the first large calls take the policies kAutoPolicies in
  // turn and are timed; then every large call takes the fastest
  int hd = c->host_direct;
  int trial = -1;
  if (hd == 5) {
    hd = 2;
    if (pipelined) {
      std::lock_guard<std::mutex> g(c->hd_mu);
      if (c->hd_choice >= 0) {
        hd = c->hd_choice;
      } else {
        // the first call of each policy is not timed: it pays one-time
        // costs (the staging workspace's allocation, first touches)
        const int32_t k = c->hd_trials++;
        hd = kAutoPolicies[k % 3];
        trial = k >= 3 ? k % 3 : -1;
      }
    }
  }
  const auto t_start = std::chrono::steady_clock::now();
  bool all_direct = true;
  for (Arr* a : whole) {
    resolve_direct(c, a, pipelined, hd);
    if (a->bytes && !a->direct) all_direct = false;
  }
  for (RayArr* r : rays) {
    if (r->per_ray == 0) continue;
    const void* p = r->host_in ? r->host_in : r->host_out;
    void* d = (r->host_in && r->host_out && r->host_in != r->host_out)
                  ? nullptr
                  : direct_ptr(c, p, pipelined, r->host_in != nullptr, hd);
    if (d) {
      r->dev = (char*)d;
      r->direct = true;
    } else {
      all_direct = false;
    }
  }
  size_t total = 0;
  for (Arr* a : whole)
    if (!a->direct) total += (a->bytes + 255) & ~(size_t)255;
  for (RayArr* r : rays)
    if (!r->direct) total += (r->per_ray * (size_t)n + 255) & ~(size_t)255;
  if ((int64_t)total > s->buf.n)
    API_CUDA(s->buf.alloc((int64_t)std::max<size_t>(total, 1 << 20)), "workspace");
  size_t off = 0;
  for (Arr* a : whole) {
    if (a->bytes == 0 || a->direct) continue;
    a->dev = s->buf.p + off;
    off += (a->bytes + 255) & ~(size_t)255;
  }
  for (RayArr* r : rays) {
    if (r->per_ray == 0 || r->direct) continue;
    r->dev = s->buf.p + off;
    off += (r->per_ray * (size_t)n + 255) & ~(size_t)255;
  }
  // chunks only overlap staging copies with compute: one launch when nothing is staged
  const int64_t chunks =
      all_direct || n <= 2 * kChunkRays
          ? 1
          : std::min<int64_t>(kMaxChunks, (n + kChunkRays - 1) / kChunkRays);
  // chunk k covers rays [starts[k], starts[k+1]).  With more than one, a
  // first chunk of a quarter of the others starts the kernels after a short
  // copy (ray_fire over 1e7 page-locked host rays: 1202 -> 1246 Mrays/s).
  // Shorter first and last chunks (2^17 rays doubling up to 2^21 and back)
  // were slower, 7.55 against 7.40 ms per call: a small chunk's launch is
  // as long as its slowest rays, and two streams overlap only two launches.
  std::vector<int64_t> starts;
  if (chunks == 1) {
    starts = {0, n};
  } else {
    const int64_t per = (n + chunks - 1) / chunks;
    const int64_t f = std::max<int64_t>(1 << 18, per / 4);
    const int64_t per2 = (n - f + chunks - 1) / chunks;
    starts.push_back(0);
    for (int64_t k = 0; k <= chunks; ++k) starts.push_back(std::min<int64_t>(n, f + k * per2));
  }
  const int64_t nch = (int64_t)starts.size() - 1;
  if (!s->events((size_t)(2 * nch + 2))) return set_err(XDGCU_ERR_CUDA, "event creation");
  // order after the caller's stream (if any)
  if (user) {
    API_CUDA(cudaEventRecord(s->ev[2 * nch], user), "event");
    API_CUDA(cudaStreamWaitEvent(s->copy_in, s->ev[2 * nch], 0), "event wait");
  }
  for (Arr* a : whole)
    if (a->host_in && a->bytes && !a->direct)
      API_CUDA(cudaMemcpyAsync(a->dev, a->host_in, a->bytes, cudaMemcpyHostToDevice, s->copy_in),
               "H2D");
  int rc = begin_query(c, s->stream, counters);
  if (rc) return rc;
  // consecutive chunks' kernels alternate between two compute streams, so
  // the tail of one launch (its last, slow rays) overlaps the next launch
  if (nch > 1) {
    API_CUDA(cudaEventRecord(s->ev[2 * nch + 1], s->stream), "event");
    API_CUDA(cudaStreamWaitEvent(s->stream2, s->ev[2 * nch + 1], 0), "event wait");
  }
  for (int64_t k = 0; k < nch; ++k) {
    const int64_t first = starts[k];
    const int64_t cnt = starts[k + 1] - first;
    if (cnt <= 0) continue;
    cudaStream_t cs = (k & 1) ? s->stream2 : s->stream;
    for (RayArr* r : rays)
      if (r->host_in && r->per_ray && !r->direct)
        API_CUDA(cudaMemcpyAsync(r->dev + r->per_ray * first,
                                 (const char*)r->host_in + r->per_ray * first, r->per_ray * cnt,
                                 cudaMemcpyHostToDevice, s->copy_in),
                 "H2D");
    API_CUDA(cudaEventRecord(s->ev[2 * k], s->copy_in), "event");
    API_CUDA(cudaStreamWaitEvent(cs, s->ev[2 * k], 0), "event wait");
    API_CUDA(launch(first, cnt, cs, nch > 1), "query launch");
    API_CUDA(cudaEventRecord(s->ev[2 * k + 1], cs), "event");
    API_CUDA(cudaStreamWaitEvent(s->copy_out, s->ev[2 * k + 1], 0), "event wait");
    for (RayArr* r : rays)
      if (r->host_out && r->per_ray && !r->direct)
        API_CUDA(cudaMemcpyAsync((char*)r->host_out + r->per_ray * first,
                                 r->dev + r->per_ray * first, r->per_ray * cnt,
                                 cudaMemcpyDeviceToHost, s->copy_out),
                 "D2H");
  }
  API_CUDA(cudaStreamSynchronize(s->copy_out), "sync");
  API_CUDA(cudaStreamSynchronize(s->stream), "sync");
  API_CUDA(cudaStreamSynchronize(s->stream2), "sync");
  API_CUDA(cudaStreamSynchronize(s->copy_in), "sync");
  if (trial >= 0) {
    const double sec =
        std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
    std::lock_guard<std::mutex> g(c->hd_mu);
    c->hd_sec_per_ray[trial] += sec / (double)n;
    c->hd_timed[trial]++;
    bool all = c->hd_choice < 0;
    for (int k = 0; k < 3; ++k) all = all && c->hd_timed[k] >= kAutoTrials;
    if (all) {
      int best = 0;
      for (int k = 1; k < 3; ++k)
        if (c->hd_sec_per_ray[k] / c->hd_timed[k] < c->hd_sec_per_ray[best] / c->hd_timed[best])
          best = k;
      c->hd_choice = kAutoPolicies[best];
    }
  }
  return XDGCU_OK;
}

int stage_out(std::vector<Arr*> arrs, cudaStream_t st) {
  for (Arr* a : arrs)
    if (a->host_out && a->bytes && !a->direct)
      API_CUDA(cudaMemcpyAsync(a->host_out, a->dev, a->bytes, cudaMemcpyDeviceToHost, st), "D2H");
  API_CUDA(cudaStreamSynchronize(st), "sync");
  return XDGCU_OK;
}

int begin_query(xdgcu_ctx* c, cudaStream_t st, unsigned long long** counters) {
  *counters = nullptr;
  if (c->counting) {
    if (!c->d_counters.p) API_CUDA(c->d_counters.alloc(CNT_N), "counters");
    API_CUDA(cudaMemsetAsync(c->d_counters.p, 0, sizeof(unsigned long long) * CNT_N, st), "counters");
    *counters = c->d_counters.p;
    c->counter_stream = st;
  }
  return XDGCU_OK;
}

// Runs `body` with a.order set to the tracks sorted by decreasing length when
// the batch is large enough (scratch allocated on the stream), else without.
template <typename Body>
int with_length_order(xdgcu_ctx* c, WalkArgs& a, cudaStream_t s, Body body) {
  if (c->walk_sort_min <= 0 || a.n < c->walk_sort_min || a.n >= ((int64_t)1 << 31)) return body();
  const size_t ord_bytes = ((sizeof(int32_t) * (size_t)a.n + 255) & ~(size_t)255);
  const size_t scr = walk_order_scratch_bytes(a.n);
  char* buf = nullptr;
  API_CUDA(scratch_alloc(c, (void**)&buf, ord_bytes + scr, s), "walk order scratch");
  cudaError_t e = walk_order(a.dist, a.n, (int32_t*)buf, buf + ord_bytes, scr, s);
  if (e != cudaSuccess) {
    cudaFreeAsync(buf, s);
    return cuda_err(e, "walk order");
  }
  a.order = (const int32_t*)buf;
  const int rc = body();
  a.order = nullptr;
  cudaFreeAsync(buf, s);
  return rc;
}

// Stream-ordered scratch of one call, freed on every return path.
struct CallScratch {
  cudaStream_t st;
  cudaMemPool_t pool;
  std::vector<void*> ptrs;
  CallScratch(cudaStream_t s, cudaMemPool_t p) : st(s), pool(p) {}
  ~CallScratch() {
    for (void* p : ptrs) cudaFreeAsync(p, st);
  }
  template <typename T>
  cudaError_t get(T** out, int64_t count) {
    *out = nullptr;
    void* p = nullptr;
    const size_t bytes = sizeof(T) * (size_t)std::max<int64_t>(1, count);
    const cudaError_t e =
        pool ? cudaMallocFromPoolAsync(&p, bytes, pool, st) : cudaMallocAsync(&p, bytes, st);
    if (e != cudaSuccess) return e;
    ptrs.push_back(p);
    *out = static_cast<T*>(p);
    return cudaSuccess;
  }
};

// The K-strided walk buffer of xdgcu_segments_global (12 bytes per slot)
// holds at most about this many bytes.
constexpr int64_t kSegStridedBytes = int64_t(1) << 30;

// D2H of one counter, waited for.
cudaError_t read_count(const int32_t* d, int32_t* h, cudaStream_t st) {
  cudaError_t e = cudaMemcpyAsync(h, d, sizeof(int32_t), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return e;
}

// Rounds of single-pass walks (the global track loop and the packed walk):
// the K-strided buffer of n tracks holds seg_strided_cap entries, about
// kSegStridedBytes (at least 16 per track, 256 at most), or fixed_k per track
// when that is set; a round of `walks` walks takes the largest K <= 256 (a
// power of two) that fits, so rounds with fewer walks pause fewer of them.
int64_t seg_strided_cap(int64_t n, int64_t fixed_k) {
  return fixed_k > 0 ? fixed_k * n
                     : std::max<int64_t>(16 * n, std::min<int64_t>(256 * n, kSegStridedBytes / 12));
}
int32_t seg_round_k(int64_t walks, int64_t cap, int64_t fixed_k, int32_t max_segs) {
  int32_t K = (int32_t)(fixed_k > 0 ? fixed_k : 256);
  while (fixed_k <= 0 && K > 16 && (int64_t)K * walks > cap) K >>= 1;
  return std::min(K, max_segs);
}

// One round's walked tracks and where their kept segments wait, packed, for
// the final placement.
struct SegRound {
  int64_t m, total;
  int32_t* walk_t;
  int64_t *off, *dst_rel;
  int32_t* seg_elem;
  double* seg_len;
};

// Per-walk-entry buffers of the rounds (n entries each) and the K-strided
// segment buffer of strided_cap entries: the walk list (track, start
// element), the walk's inputs from the tracks' walk state, and what the walk
// kernel reports (status, count, where it stopped, its running length sum).
struct SegWalkBufs {
  int32_t *walk_t, *walk_start, *wst, *wcnt, *wstop, *sk_elem;
  double *wr, *wu, *wd, *wsum_in, *wsum_out, *wend_r, *wend_d, *sk_len;
  int64_t strided_cap;
};

// One round of the capped single-pass walk for the m entries of the walk
// list: walk_elements from each track's walk state, at most K segments per
// track into the K-strided buffer, the kept counts scanned into R->off, the
// kept segments packed into a buffer of the round (R, kept for the final
// placement), the walk state advanced and the tracks still active appended to
// act_next (seg_advance; walk_only: an ended walk finishes its track).
// Synchronises `st` once, for the round's total.  On an allocation failure
// sets *no_memory (when given).
int seg_walk_round(xdgcu_ctx* c, bool mixed, const SegState& ss, const WalkArgs& geo,
                   const SegWalkBufs& B, int32_t m, int32_t max_segs, bool walk_only,
                   int32_t* act_next, int32_t* n_act, CallScratch& S, cudaStream_t st,
                   bool* no_memory, SegRound* R) {
  auto get = [&](auto** p, int64_t count) -> bool {
    if (S.get(p, count) == cudaSuccess) return true;
    cudaGetLastError();  // the failed allocation is not a pending launch error
    if (no_memory) *no_memory = true;
    return false;
  };
  const int32_t K = seg_round_k(m, B.strided_cap, c->segments_walk_cap, max_segs);
  *R = SegRound{};
  R->m = m;
  if (!get(&R->walk_t, m) || !get(&R->off, (int64_t)m + 1) || !get(&R->dst_rel, m))
    return set_err(XDGCU_ERR_CUDA, "walk rounds: temporary memory");
  API_CUDA(cudaMemcpyAsync(R->walk_t, B.walk_t, sizeof(int32_t) * m, cudaMemcpyDeviceToDevice, st),
           "D2D");
  API_CUDA(seg_walk_inputs(ss, B.walk_t, m, B.wr, B.wu, B.wd, B.wsum_in, st), "walk inputs");
  WalkArgs w = geo;
  w.n = m;
  w.start = B.walk_start;
  w.org = B.wr;
  w.dir = B.wu;
  w.dist = B.wd;
  w.max_segs = K;
  w.status = B.wst;
  w.seg_count = B.wcnt;
  w.stop_elem = B.wstop;
  w.sum_in = B.wsum_in;
  w.sum_out = B.wsum_out;
  w.end_r = B.wend_r;
  w.end_dist = B.wend_d;
  w.seg_elem = B.sk_elem;
  w.seg_len = B.sk_len;
  w.offsets = nullptr;
  w.out_mode = WALK_STRIDED;
  int rc = with_length_order(c, w, st, [&]() -> int {
    API_CUDA(launch_walk(mixed, c->face_order, w, st), "walk");
    return XDGCU_OK;
  });
  if (rc) return rc;
  // the segments each track keeps (max_segs per walk), packed
  API_CUDA(seg_round_counts(ss, R->walk_t, m, B.wcnt, max_segs, R->off, st), "walk round counts");
  int64_t* sums = nullptr;
  if (!get(&sums, scan_scratch_entries(m))) return set_err(XDGCU_ERR_CUDA, "walk rounds: scan scratch");
  API_CUDA(scan_offsets(R->off, m, sums, st), "scan");
  API_CUDA(cudaMemcpyAsync(&R->total, R->off + m, sizeof(int64_t), cudaMemcpyDeviceToHost, st),
           "D2H");
  API_CUDA(cudaStreamSynchronize(st), "sync");
  if (!get(&R->seg_elem, R->total) || !get(&R->seg_len, R->total))
    return set_err(XDGCU_ERR_CUDA, "walk rounds: temporary memory");
  API_CUDA(seg_pack(m, K, B.sk_elem, B.sk_len, R->off, R->seg_elem, R->seg_len, st), "walk pack");
  API_CUDA(seg_advance(ss, R->walk_t, m, K, B.sk_elem, B.wcnt, B.wst, B.wstop, B.wend_r, B.wend_d,
                       B.wsum_out, max_segs, R->off, R->dst_rel, act_next, n_act, st, walk_only),
           "walk advance");
  return XDGCU_OK;
}

// xdgcu_walk_elements_packed with one walk of every track instead of a count
// walk and an emit walk: rounds of single-pass walks capped at K segments per
// track (as the global track loop's walk step), each round's kept segments
// packed into a buffer of the round; a track that reaches K pauses and the
// next round resumes it where the walk kernel stopped (same element, position
// and distance, so the same segments).  The tracks' totals then give the
// offsets, and every round's segments go to their place.  Statuses follow the
// two-pass walk: RAY_WALK_LIMIT past max_segs, RAY_OUTPUT_FULL (replacing OK)
// for a track with segments that do not fit in `capacity`.  `a` holds device
// arrays.  Sets *no_memory when a temporary buffer could not be allocated (about the
// output's size plus the strided buffer); nothing has then been written that
// the two-pass walk does not overwrite.
int walk_packed_rounds(xdgcu_ctx* c, bool mixed, const WalkArgs& a, cudaStream_t st,
                       bool* no_memory) {
  *no_memory = false;
  const int64_t n = a.n;
  CallScratch S(st, c->pool);
  bool ok = true;
  auto get = [&](auto** p, int64_t count) {
    if (ok && S.get(p, count) != cudaSuccess) {
      ok = false;
      *no_memory = true;
      cudaGetLastError();  // the failed allocation is not a pending launch error
    }
  };
  SegState ss{};
  ss.n = n;
  ss.status = a.status;
  if (!ss.status) get(&ss.status, n);
  get(&ss.written, n);
  get(&ss.last, n);
  get(&ss.stopped, n);
  get(&ss.u, 3 * n);
  get(&ss.wr, 3 * n);
  get(&ss.wd, n);
  get(&ss.wsum, n);
  get(&ss.wcount, n);
  get(&ss.welem, n);
  get(&ss.paused, n);
  int32_t *act = nullptr, *act_next = nullptr, *counters = nullptr, *loc = nullptr;
  get(&act, n);
  get(&act_next, n);
  get(&counters, 4);
  get(&loc, n);
  SegWalkBufs B{};
  get(&B.walk_t, n);
  get(&B.walk_start, n);
  get(&B.wst, n);
  get(&B.wcnt, n);
  get(&B.wstop, n);
  get(&B.wr, 3 * n);
  get(&B.wu, 3 * n);
  get(&B.wd, n);
  get(&B.wsum_in, n);
  get(&B.wsum_out, n);
  get(&B.wend_r, 3 * n);
  get(&B.wend_d, n);
  B.strided_cap = seg_strided_cap(n, c->segments_walk_cap);
  get(&B.sk_elem, B.strided_cap);
  get(&B.sk_len, B.strided_cap);
  if (!ok) return set_err(XDGCU_ERR_CUDA, "walk_elements_packed: temporary memory");
  int32_t* n_act = counters;
  int32_t* n_walk = counters + 1;
  int32_t* n_loc = counters + 3;
  API_CUDA(seg_walk_init(ss, a.start, a.org, a.dir, a.dist, act, st), "packed walk init");
  std::vector<SegRound> rounds;
  int32_t m = (int32_t)n;
  while (m > 0) {
    // every active track is a paused walk: all go to the walk list
    API_CUDA(cudaMemsetAsync(counters, 0, 4 * sizeof(int32_t), st), "memset");
    API_CUDA(seg_split(ss, act, m, B.walk_t, B.walk_start, n_walk, loc, n_loc, st),
             "packed walk split");
    SegRound R{};
    const int rc = seg_walk_round(c, mixed, ss, a, B, m, a.max_segs, true, act_next, n_act, S, st,
                                  no_memory, &R);
    if (rc) return rc;
    rounds.push_back(R);
    API_CUDA(read_count(n_act, &m, st), "packed walk count");
    std::swap(act, act_next);
  }
  // offsets from the tracks' totals, then every round's segments to their place
  API_CUDA(seg_counts(ss, a.offsets, st), "packed walk totals");
  int64_t* sums = nullptr;
  get(&sums, scan_scratch_entries(n));
  if (!ok) return set_err(XDGCU_ERR_CUDA, "walk_elements_packed: temporary memory");
  API_CUDA(scan_offsets(a.offsets, n, sums, st), "scan");
  API_CUDA(seg_mark_full(ss, a.offsets, a.capacity, st), "packed walk capacity");
  for (const SegRound& R : rounds)
    API_CUDA(seg_scatter(ss, R.walk_t, R.m, R.off, R.dst_rel, R.seg_elem, R.seg_len, a.offsets,
                         a.capacity, a.seg_elem, a.seg_len, st),
             "packed walk scatter");
  return XDGCU_OK;
}

// Enqueues one traversal launch with the context's work distribution: when
// the device work queue is on (trace_grab > 0) a zeroed cursor, and when the
// batch is large enough (trace_sort_min) a coherent ray order, both in one
// stream-ordered scratch allocation freed after the launch.
// Stack entries of a traversal launch: the requested depth, raised to the
// surface trees' bound (width - 1) * depth -- which no traversal can exceed --
// as far as the 64-entry maximum allows.
int32_t trace_stack_for(const xdgcu_ctx* c) {
  const int32_t need = std::min(64, (c->surf_stack_bound + 7) / 8 * 8);
  return std::max(c->trace_stack, need);
}

cudaError_t launch_trace(xdgcu_ctx* c, int mode, bool mixed, SurfArgs a, double extent,
                         cudaStream_t s, int32_t min_grab = 0) {
  if (a.n <= 0) return cudaSuccess;
  const bool sort = c->trace_sort_min > 0 && a.n >= c->trace_sort_min && a.n < ((int64_t)1 << 31) &&
                    extent > 0.0;
  a.grab = std::max(c->trace_grab, min_grab);
  a.work = nullptr;
  a.order = nullptr;
  if (a.grab == 0 && !sort) return launch_surface_query(mode, mixed, a, s);
  const size_t ord_bytes = sort ? ((sizeof(int32_t) * (size_t)a.n + 255) & ~(size_t)255) : 0;
  const size_t scr = sort ? ray_order_scratch_bytes(a.n) : 0;
  char* buf = nullptr;
  cudaError_t e = scratch_alloc(c, (void**)&buf, 256 + ord_bytes + scr, s);
  if (e != cudaSuccess) return e;
  if (a.grab > 0) {
    a.work = (unsigned long long*)buf;
    e = cudaMemsetAsync(buf, 0, sizeof(unsigned long long), s);
  }
  if (e == cudaSuccess && sort) {
    a.order = (const int32_t*)(buf + 256);
    const int32_t* trees = (mode == MODE_FIND_VOLUME) ? nullptr : a.ray_trees;
    e = ray_order(a.org, a.dir, trees, a.n_trees, a.n, extent, (int32_t*)(buf + 256),
                  buf + 256 + ord_bytes, scr, s);
  }
  if (e == cudaSuccess) e = launch_surface_query(mode, mixed, a, s);
  const cudaError_t f = cudaFreeAsync(buf, s);
  return e != cudaSuccess ? e : f;
}

// Entry points run with the context's device current and give the caller's
// current device back on return (DeviceGuard).
#define CHECK_CTX(c)                                                            \
  if (!(c)) return set_err(XDGCU_ERR_INVALID_ARG, "null context");              \
  DeviceGuard device_guard_((c)->device);                                       \
  if (!device_guard_.ok()) return set_err(XDGCU_ERR_CUDA, "cudaSetDevice failed")

}  // namespace

// Helpers for the allocation-free walk entry point (noalloc.cu).
namespace xdgcu {

int set_last_error(int code, const char* msg) { return set_err(code, msg); }

int ctx_device(const xdgcu_ctx* c) { return c->device; }

const char* walk_args_for(const xdgcu_ctx* c, WalkArgs* a, int* face_order, int* device) {
  if (!c->has_tets) return "no tet mesh set";
  a->xyz = c->d_xyz.p;
  a->xyz32 = c->d_xyz32.p;
  a->edge = c->walk_edge_table ? c->d_edge.p : nullptr;
  a->tet_edge = c->d_tet_edge.p;
  a->conn = c->d_conn.p;
  a->adj = c->d_adj.p;
  a->elem_ids = c->d_elem_ids.p;
  a->n_tets = (int32_t)c->n_tet;
  std::memcpy(a->face, c->face, sizeof(a->face));
  a->walk_queue = c->walk_queue;
  a->flush_wait = c->walk_flush_wait;
  *face_order = c->face_order;
  *device = c->device;
  return nullptr;
}

}  // namespace xdgcu

// ===========================================================================
// C ABI
// ===========================================================================

extern "C" {

int xdgcu_version(void) { return 100; }

const char* xdgcu_last_error(const xdgcu_ctx*) { return g_last_error.c_str(); }

int xdgcu_create(xdgcu_ctx** out, int device) {
  if (!out) return set_err(XDGCU_ERR_INVALID_ARG, "null output pointer");
  *out = nullptr;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) return set_err(XDGCU_ERR_CUDA, "no CUDA device available");
  if (device < 0 || device >= n) return set_err(XDGCU_ERR_INVALID_ARG, "device out of range");
  DeviceGuard guard(device);
  if (!guard.ok()) return set_err(XDGCU_ERR_CUDA, "cudaSetDevice failed");
  auto* c = new xdgcu_ctx();
  c->device = device;
  int ats = 0;
  if (cudaDeviceGetAttribute(&ats, cudaDevAttrPageableMemoryAccessUsesHostPageTables, device) !=
      cudaSuccess) {
    cudaGetLastError();
    ats = 0;
  }
  c->pageable_direct = ats == 1;
  if (cudaStreamCreateWithFlags(&c->build_stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    return set_err(XDGCU_ERR_CUDA, "stream creation failed");
  }
  // the scratch pool (without one the calls use the device's default pool).
  // XDGCU_SCRATCH_POOL=0 in the environment leaves it out: a profiler's
  // kernel replay, which saves and restores the device memory around each
  // pass, ended in a GPU memory fault in a process with such a pool
  cudaMemPoolProps props{};
  props.allocType = cudaMemAllocationTypePinned;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = device;
  const char* want_pool = std::getenv("XDGCU_SCRATCH_POOL");
  if (want_pool && std::strcmp(want_pool, "0") == 0) {
    c->pool = nullptr;
  } else if (cudaMemPoolCreate(&c->pool, &props) == cudaSuccess) {
    uint64_t keep = (uint64_t)c->keep_bytes;
    cudaMemPoolSetAttribute(c->pool, cudaMemPoolAttrReleaseThreshold, &keep);
  } else {
    cudaGetLastError();
    c->pool = nullptr;
  }
  *out = c;
  return XDGCU_OK;
}

int xdgcu_destroy(xdgcu_ctx* c) {
  if (!c) return XDGCU_OK;
  DeviceGuard guard(c->device);
  cudaDeviceSynchronize();
  if (c->build_stream) cudaStreamDestroy(c->build_stream);
  if (c->pool) cudaMemPoolDestroy(c->pool);
  delete c;
  return XDGCU_OK;
}

int xdgcu_register_surface(xdgcu_ctx* c, int32_t surface_id, int64_t n_faces, const double* tri_xyz,
                           const int32_t* face_ids) {
  CHECK_CTX(c);
  std::lock_guard<std::mutex> g(c->mu);
  if (n_faces < 0 || (n_faces > 0 && (!tri_xyz || !face_ids)))
    return set_err(XDGCU_ERR_INVALID_ARG, "register_surface: bad arrays");
  if (c->surf_index.count(surface_id))
    return set_err(XDGCU_ERR_STATE, "register_surface: surface already registered");
  if ((int64_t)c->h_tri_face.size() + n_faces > (int64_t)(1 << 27))
    return set_err(XDGCU_ERR_INVALID_ARG, "register_surface: more than 2^27 triangles");
  for (int64_t i = 0; i < 9 * n_faces; ++i)
    if (!(std::fabs(tri_xyz[i]) < 0x1p300))
      return set_err(XDGCU_ERR_INVALID_ARG,
                     "register_surface: coordinates must be finite and below 2^300 in magnitude");
  SurfaceRec r;
  r.id = surface_id;
  r.first = (int64_t)c->h_tri_face.size();
  r.count = n_faces;
  const int32_t sidx = (int32_t)c->surfs.size();
  c->surf_index[surface_id] = sidx;
  c->surfs.push_back(r);
  c->h_tri_xyz.insert(c->h_tri_xyz.end(), tri_xyz, tri_xyz + 9 * n_faces);
  c->h_tri_face.insert(c->h_tri_face.end(), face_ids, face_ids + n_faces);
  c->h_tri_surf.insert(c->h_tri_surf.end(), (size_t)n_faces, sidx);
  c->tri_dirty = true;
  c->surf_dirty = true;
  return XDGCU_OK;
}

static int create_surface_tree_impl(xdgcu_ctx* c, const std::vector<int32_t>& sidx,
                                    const std::vector<int32_t>& sense, double bump, bool global,
                                    int32_t* tree_out) {
  auto t = std::make_unique<TreeHost>();
  t->id = (int32_t)c->surf_trees.size() + 1;
  t->kind = TREE_SURFACE;
  t->members = sidx;
  t->bump_arg = bump;
  // parent tree ids and box dilation (embree/ray_tracer.cpp:76-99)
  if (!global) {
    for (size_t k = 0; k < sidx.size(); ++k) {
      SurfaceRec& s = c->surfs[sidx[k]];
      s.bump = std::max(s.bump, bump);
      if (sense[k] == 0) s.fwd_tree = t->id;
      else s.rev_tree = t->id;
    }
    c->surf_dirty = true;
  }
  int rc = sync_surfaces(c);
  if (rc) return rc;
  std::vector<int32_t> tris;
  std::vector<double> bumps;
  for (int32_t s : sidx) {
    const SurfaceRec& r = c->surfs[s];
    const double b = r.bump > 0 ? r.bump : (bump > 0 ? bump : 1e-3);
    for (int64_t k = 0; k < r.count; ++k) {
      tris.push_back((int32_t)(r.first + k));
      bumps.push_back(b);
    }
  }
  rc = build_surface_bvh(c, *t, tris, bumps);
  if (rc) return rc;
  *tree_out = t->id;
  c->surf_trees.push_back(std::move(t));
  c->surf_trees_dirty = true;
  return sync_tree_tables(c);
}

int xdgcu_create_surface_tree(xdgcu_ctx* c, const int32_t* surface_ids, const int32_t* sense,
                              int32_t n_surfaces, double bump, int32_t* tree_out) {
  CHECK_CTX(c);
  std::lock_guard<std::mutex> g(c->mu);
  if (!tree_out || n_surfaces < 0 || (n_surfaces > 0 && (!surface_ids || !sense)))
    return set_err(XDGCU_ERR_INVALID_ARG, "create_surface_tree: bad arguments");
  if (!(bump >= 0.0) || !std::isfinite(bump))
    return set_err(XDGCU_ERR_INVALID_ARG, "create_surface_tree: bump must be finite and >= 0");
  std::vector<int32_t> sidx, sn;
  for (int32_t k = 0; k < n_surfaces; ++k) {
    auto it = c->surf_index.find(surface_ids[k]);
    if (it == c->surf_index.end())
      return set_err(XDGCU_ERR_NOT_FOUND, "create_surface_tree: surface " +
                                              std::to_string(surface_ids[k]) + " not registered");
    if (sense[k] != 0 && sense[k] != 1)
      return set_err(XDGCU_ERR_INVALID_ARG, "create_surface_tree: sense must be 0 or 1");
    sidx.push_back(it->second);
    sn.push_back(sense[k]);
  }
  return create_surface_tree_impl(c, sidx, sn, bump, false, tree_out);
}

int xdgcu_create_global_surface_tree(xdgcu_ctx* c, int32_t* tree_out) {
  CHECK_CTX(c);
  std::lock_guard<std::mutex> g(c->mu);
  if (!tree_out) return set_err(XDGCU_ERR_INVALID_ARG, "null tree_out");
  std::vector<int32_t> sidx(c->surfs.size()), sn(c->surfs.size(), 0);
  for (size_t k = 0; k < sidx.size(); ++k) sidx[k] = (int32_t)k;
  return create_surface_tree_impl(c, sidx, sn, 0.0, true, tree_out);
}

int xdgcu_set_tet_mesh(xdgcu_ctx* c, int64_t n_vertices, const double* xyz, int64_t n_tets,
                       const int32_t* conn, const int32_t* adj, const int32_t* elem_ids,
                       const int32_t face_table[12]) {
  CHECK_CTX(c);
  std::lock_guard<std::mutex> g(c->mu);
  if (c->has_tets) return set_err(XDGCU_ERR_STATE, "set_tet_mesh: mesh already set");
  if (n_vertices < 0 || n_tets < 0 || n_tets >= (1ll << 31) || !face_table ||
      (n_vertices > 0 && !xyz) || (n_tets > 0 && (!conn || !adj || !elem_ids)))
    return set_err(XDGCU_ERR_INVALID_ARG, "set_tet_mesh: bad arrays");
  for (int k = 0; k < 12; ++k)
    if (face_table[k] < 0 || face_table[k] > 3)
      return set_err(XDGCU_ERR_INVALID_ARG, "set_tet_mesh: face table entries must be 0..3");
  for (int64_t i = 0; i < 3 * n_vertices; ++i)
    if (!(std::fabs(xyz[i]) < 0x1p300))
      return set_err(XDGCU_ERR_INVALID_ARG,
                     "set_tet_mesh: coordinates must be finite and below 2^300 in magnitude");
  for (int64_t i = 0; i < 4 * n_tets; ++i) {
    if (conn[i] < 0 || conn[i] >= n_vertices)
      return set_err(XDGCU_ERR_INVALID_ARG, "set_tet_mesh: connectivity out of range");
    if (adj[i] < -1 || adj[i] >= n_tets)
      return set_err(XDGCU_ERR_INVALID_ARG, "set_tet_mesh: adjacency out of range");
  }
  c->n_vert = n_vertices;
  c->n_tet = n_tets;
  API_CUDA(c->d_xyz.alloc(std::max<int64_t>(1, 3 * n_vertices)), "alloc vertices");
  API_CUDA(c->d_xyz32.alloc(std::max<int64_t>(1, n_vertices)), "alloc vertices");
  API_CUDA(c->d_conn.alloc(std::max<int64_t>(1, n_tets)), "alloc tets");
  API_CUDA(c->d_adj.alloc(std::max<int64_t>(1, n_tets)), "alloc tets");
  API_CUDA(c->d_elem_ids.alloc(std::max<int64_t>(1, n_tets)), "alloc tets");
  if (n_vertices) {
    API_CUDA(cudaMemcpy(c->d_xyz.p, xyz, sizeof(double) * 3 * n_vertices, cudaMemcpyHostToDevice),
             "upload vertices");
    k_vert32<<<grid(n_vertices), 256, 0, c->build_stream>>>(c->d_xyz.p, n_vertices, c->d_xyz32.p);
    API_CUDA(cudaGetLastError(), "vertices");
    API_CUDA(cudaStreamSynchronize(c->build_stream), "vertices");
  }
  if (n_tets) {
    API_CUDA(cudaMemcpy(c->d_conn.p, conn, sizeof(int32_t) * 4 * n_tets, cudaMemcpyHostToDevice),
             "upload tets");
    API_CUDA(cudaMemcpy(c->d_adj.p, adj, sizeof(int32_t) * 4 * n_tets, cudaMemcpyHostToDevice),
             "upload tets");
    API_CUDA(cudaMemcpy(c->d_elem_ids.p, elem_ids, sizeof(int32_t) * n_tets, cudaMemcpyHostToDevice),
             "upload tets");
    // meshes of 6 * n_tets >= 2^31 vertex pairs walk without the table
    if (6 * n_tets < (1ll << 31)) {
      double* edge = nullptr;
      int32_t* tet_edge = nullptr;
      int64_t ne = 0;
      // without memory for it the walk computes the edges from the vertices
      if (build_edge_table(c->d_xyz.p, c->d_conn.p, n_tets, &edge, &tet_edge, &ne,
                           c->build_stream) != cudaSuccess)
        cudaGetLastError();
      c->d_edge.p = edge;
      c->d_edge.n = 6 * ne;
      c->d_tet_edge.p = tet_edge;
      c->d_tet_edge.n = 6 * n_tets;
      c->n_edges = ne;
    }
  }
  std::memcpy(c->face, face_table, sizeof(c->face));
  c->face_order = std::memcmp(face_table, kMoabFaces, sizeof(kMoabFaces)) == 0 ? 0 : 1;
  c->has_tets = true;
  return XDGCU_OK;
}

int xdgcu_create_element_tree(xdgcu_ctx* c, const int32_t* tet_indices, int64_t n, int32_t* tree_out) {
  CHECK_CTX(c);
  std::lock_guard<std::mutex> g(c->mu);
  if (!tree_out || n < 0 || (n > 0 && !tet_indices))
    return set_err(XDGCU_ERR_INVALID_ARG, "create_element_tree: bad arguments");
  if (!c->has_tets) return set_err(XDGCU_ERR_STATE, "create_element_tree: no tet mesh set");
  if (n > (1 << 27)) return set_err(XDGCU_ERR_INVALID_ARG, "create_element_tree: too many tets");
  std::vector<int32_t> tets(tet_indices, tet_indices + n);
  for (int32_t t : tets)
    if (t < 0 || t >= c->n_tet)
      return set_err(XDGCU_ERR_INVALID_ARG, "create_element_tree: tet index out of range");
  auto t = std::make_unique<TreeHost>();
  t->id = (int32_t)c->elem_trees.size() + 1;
  t->kind = TREE_ELEMENT;
  t->members = tets;
  int rc = build_element_bvh(c, *t, tets);
  if (rc) return rc;
  *tree_out = t->id;
  c->elem_trees.push_back(std::move(t));
  c->elem_trees_dirty = true;
  return sync_tree_tables(c);
}

int xdgcu_create_global_element_tree(xdgcu_ctx* c, int32_t* tree_out) {
  CHECK_CTX(c);
  std::lock_guard<std::mutex> g(c->mu);
  if (!tree_out) return set_err(XDGCU_ERR_INVALID_ARG, "null tree_out");
  if (!c->has_tets) {
    // the reference builds an empty global scene (embree/ray_tracer.cpp:208-224)
  }
  std::vector<int32_t> tets;
  for (auto& t : c->elem_trees) tets.insert(tets.end(), t->members.begin(), t->members.end());
  auto t = std::make_unique<TreeHost>();
  t->id = (int32_t)c->elem_trees.size() + 1;
  t->kind = TREE_ELEMENT;
  t->members = tets;
  int rc = build_element_bvh(c, *t, tets);
  if (rc) return rc;
  *tree_out = t->id;
  c->elem_trees.push_back(std::move(t));
  c->elem_trees_dirty = true;
  return sync_tree_tables(c);
}

int xdgcu_num_surface_trees(const xdgcu_ctx* c) { return c ? (int)c->surf_trees.size() : 0; }
int xdgcu_num_element_trees(const xdgcu_ctx* c) { return c ? (int)c->elem_trees.size() : 0; }

static int tree_info(const std::vector<std::unique_ptr<TreeHost>>& v, int32_t tree, int64_t out[8]) {
  if (!out) return set_err(XDGCU_ERR_INVALID_ARG, "null output");
  if (tree < 1 || tree > (int32_t)v.size()) return set_err(XDGCU_ERR_NOT_FOUND, "no such tree");
  const TreeHost& t = *v[tree - 1];
  for (int k = 0; k < 8; ++k) out[k] = 0;
  out[0] = t.n_nodes;
  out[1] = t.prim_ref.n;
  out[2] = t.depth;
  out[3] = (int64_t)sizeof(Node32) * t.n_nodes * (t.dev.width / kWidth);
  out[4] = (int64_t)sizeof(Node64) * t.n_nodes * (t.dev.width / kWidth);
  out[5] = t.dev.width;
  return XDGCU_OK;
}

int xdgcu_surface_tree_info(const xdgcu_ctx* c, int32_t tree, int64_t out[8]) {
  if (!c) return set_err(XDGCU_ERR_INVALID_ARG, "null context");
  return tree_info(c->surf_trees, tree, out);
}
int xdgcu_element_tree_info(const xdgcu_ctx* c, int32_t tree, int64_t out[8]) {
  if (!c) return set_err(XDGCU_ERR_INVALID_ARG, "null context");
  return tree_info(c->elem_trees, tree, out);
}

int xdgcu_rebuild_trees(xdgcu_ctx* c, int32_t kinds) {
  CHECK_CTX(c);
  if (kinds < 0 || kinds > 3) return set_err(XDGCU_ERR_INVALID_ARG, "kinds must be 0..3");
  std::lock_guard<std::mutex> g(c->mu);
  int rc = sync_surfaces(c);
  if (rc) return rc;
  for (auto& tp : c->surf_trees) {
    if (!(kinds & 1)) break;
    TreeHost& t = *tp;
    std::vector<int32_t> tris;
    std::vector<double> bumps;
    for (int32_t sx : t.members) {
      const SurfaceRec& r = c->surfs[sx];
      const double b = r.bump > 0 ? r.bump : (t.bump_arg > 0 ? t.bump_arg : 1e-3);
      for (int64_t k = 0; k < r.count; ++k) {
        tris.push_back((int32_t)(r.first + k));
        bumps.push_back(b);
      }
    }
    if (t.n32) cudaFree(t.n32);
    if (t.n64) cudaFree(t.n64);
    t.n32 = nullptr;
    t.n64 = nullptr;
    rc = build_surface_bvh(c, t, tris, bumps);
    if (rc) return rc;
  }
  for (auto& tp : c->elem_trees) {
    if (!(kinds & 2)) break;
    TreeHost& t = *tp;
    if (t.n32) cudaFree(t.n32);
    if (t.n64) cudaFree(t.n64);
    t.n32 = nullptr;
    t.n64 = nullptr;
    rc = build_element_bvh(c, t, t.members);
    if (rc) return rc;
  }
  c->surf_trees_dirty = true;
  c->elem_trees_dirty = true;
  return sync_tree_tables(c);
}

int xdgcu_set_tuning(xdgcu_ctx* c, const char* key, int64_t value) {
  if (!c || !key) return set_err(XDGCU_ERR_INVALID_ARG, "null argument");
  const std::string k(key);
  if (k == "trace_occupancy") {
    if (value < 2 || value > 4) return set_err(XDGCU_ERR_INVALID_ARG, "trace_occupancy must be 2..4");
    c->trace_occupancy = (int32_t)value;
  } else if (k == "trace_node_iters" || k == "trace_node_iters_fp64" ||
             k == "trace_node_iters_direct") {
    if (value < 1 || value > 64) return set_err(XDGCU_ERR_INVALID_ARG, k + " must be 1..64");
    (k == "trace_node_iters" ? c->trace_node_iters
                             : (k == "trace_node_iters_fp64" ? c->trace_node_iters_fp64
                                                             : c->trace_node_iters_direct)) =
        (int32_t)value;
  } else if (k == "trace_flush_wait") {
    if (value < 1 || value > 32) return set_err(XDGCU_ERR_INVALID_ARG, "trace_flush_wait must be 1..32");
    c->trace_flush_wait = (int32_t)value;
  } else if (k == "trace_stack") {
    if (value < 16 || value > 64 || value % 8 != 0)
      return set_err(XDGCU_ERR_INVALID_ARG, "trace_stack must be 16..64 in steps of 8");
    c->trace_stack = (int32_t)value;
  } else if (k == "trace_grab") {
    if (value < 0 || value > (1 << 20) || value % 32 != 0)
      return set_err(XDGCU_ERR_INVALID_ARG, "trace_grab must be 0 or a multiple of 32 up to 2^20");
    c->trace_grab = (int32_t)value;
  } else if (k == "transport_event_wait") {
    if (value < 1 || value > 32)
      return set_err(XDGCU_ERR_INVALID_ARG, "transport_event_wait must be 1..32");
    c->transport_event_wait = (int32_t)value;
  } else if (k == "particle_event_wait") {
    if (value < 1 || value > 32)
      return set_err(XDGCU_ERR_INVALID_ARG, "particle_event_wait must be 1..32");
    c->particle_event_wait = (int32_t)value;
  } else if (k == "trace_sort_min") {
    if (value < 0) return set_err(XDGCU_ERR_INVALID_ARG, "trace_sort_min must be >= 0");
    c->trace_sort_min = value;
  } else if (k == "node_width") {
    if (value != 4 && value != 8) return set_err(XDGCU_ERR_INVALID_ARG, "node_width must be 4 or 8");
    c->node_width = (int32_t)value;
  } else if (k == "leaf_max") {
    if (value < 1 || value > 4) return set_err(XDGCU_ERR_INVALID_ARG, "leaf_max must be 1..4");
    c->leaf_max = (int32_t)value;
  } else if (k == "bvh_sah") {
    if (value < 0 || value > 1) return set_err(XDGCU_ERR_INVALID_ARG, "bvh_sah must be 0 or 1");
    c->bvh_sah = (int32_t)value;
  } else if (k == "bvh_prim_cost") {
    if (value < 1 || value > 100000)
      return set_err(XDGCU_ERR_INVALID_ARG, "bvh_prim_cost must be 1..100000");
    c->bvh_prim_cost = (int32_t)value;
  } else if (k == "walk_queue") {
    if (value < 0 || value > 1) return set_err(XDGCU_ERR_INVALID_ARG, "walk_queue must be 0 or 1");
    c->walk_queue = (int32_t)value;
  } else if (k == "walk_flush_wait") {
    if (value < 1 || value > 32) return set_err(XDGCU_ERR_INVALID_ARG, "walk_flush_wait must be 1..32");
    c->walk_flush_wait = (int32_t)value;
  } else if (k == "walk_sort_min") {
    if (value < 0) return set_err(XDGCU_ERR_INVALID_ARG, "walk_sort_min must be >= 0");
    c->walk_sort_min = value;
  } else if (k == "trace_edge_table") {
    if (value < 0 || value > 1) return set_err(XDGCU_ERR_INVALID_ARG, "trace_edge_table must be 0 or 1");
    c->trace_edge_table = (int32_t)value;
  } else if (k == "closest_node_steps" || k == "closest_node_steps_fp64" ||
             k == "find_node_steps_fp64") {
    if (value < 1 || value > 64)
      return set_err(XDGCU_ERR_INVALID_ARG, k + " must be 1..64");
    (k == "closest_node_steps"        ? c->closest_node_steps
     : k == "closest_node_steps_fp64" ? c->closest_node_steps_fp64
                                      : c->find_node_steps_fp64) = (int32_t)value;
  } else if (k == "scratch_keep_bytes") {
    if (value < 0) return set_err(XDGCU_ERR_INVALID_ARG, "scratch_keep_bytes must be >= 0");
    c->keep_bytes = value;
    if (c->pool) {
      uint64_t keep = (uint64_t)value;
      API_CUDA(cudaMemPoolSetAttribute(c->pool, cudaMemPoolAttrReleaseThreshold, &keep),
               "scratch pool");
      // memory freed on a stream counts as held until the host has seen the
      // free complete: wait for the device, then release
      DeviceGuard guard(c->device);
      API_CUDA(cudaDeviceSynchronize(), "scratch pool");
      API_CUDA(cudaMemPoolTrimTo(c->pool, (size_t)value), "scratch pool");
    }
  } else if (k == "scratch_bytes_high") {
    if (value != 0) return set_err(XDGCU_ERR_INVALID_ARG, "scratch_bytes_high can only be reset to 0");
    if (c->pool) {
      uint64_t zero = 0;
      API_CUDA(cudaMemPoolSetAttribute(c->pool, cudaMemPoolAttrUsedMemHigh, &zero), "scratch pool");
    }
  } else if (k == "closest_sort_min") {
    if (value < 0) return set_err(XDGCU_ERR_INVALID_ARG, "closest_sort_min must be >= 0");
    c->closest_sort_min = value;
  } else if (k == "find_sort_min") {
    if (value < 0) return set_err(XDGCU_ERR_INVALID_ARG, "find_sort_min must be >= 0");
    c->find_sort_min = value;
  } else if (k == "closest_step_budget") {
    if (value < 0 || value > (1 << 30))
      return set_err(XDGCU_ERR_INVALID_ARG, "closest_step_budget must be 0..2^30");
    c->closest_budget = (int32_t)value;
  } else if (k == "packed_walk_passes") {
    if (value != 1 && value != 2) return set_err(XDGCU_ERR_INVALID_ARG, "packed_walk_passes must be 1 or 2");
    c->packed_passes = (int32_t)value;
  } else if (k == "find_element_phased") {
    if (value < 0 || value > 1)
      return set_err(XDGCU_ERR_INVALID_ARG, "find_element_phased must be 0 or 1");
    c->find_phased = (int32_t)value;
  } else if (k == "segments_walk_cap") {
    if (value < 0 || value > 1024)
      return set_err(XDGCU_ERR_INVALID_ARG, "segments_walk_cap must be 0..1024");
    c->segments_walk_cap = (int32_t)value;
  } else if (k == "closest_bound") {
    if (value < 0 || value > 1) return set_err(XDGCU_ERR_INVALID_ARG, "closest_bound must be 0 or 1");
    c->closest_bound = (int32_t)value;
  } else if (k == "walk_edge_table") {
    if (value < 0 || value > 1) return set_err(XDGCU_ERR_INVALID_ARG, "walk_edge_table must be 0 or 1");
    c->walk_edge_table = (int32_t)value;
  } else if (k == "host_direct") {
    if (value < 0 || value > 5) return set_err(XDGCU_ERR_INVALID_ARG, "host_direct must be 0..5");
    c->host_direct = (int32_t)value;
    if (value == 5) {  // a fresh choice
      std::lock_guard<std::mutex> g(c->hd_mu);
      c->hd_trials = 0;
      for (int k = 0; k < 3; ++k) {
        c->hd_timed[k] = 0;
        c->hd_sec_per_ray[k] = 0.0;
      }
      c->hd_choice = -1;
    }
  } else {
    return set_err(XDGCU_ERR_NOT_FOUND, "unknown tuning key " + k);
  }
  return XDGCU_OK;
}

int xdgcu_get_tuning(const xdgcu_ctx* c, const char* key, int64_t* value) {
  if (!c || !key || !value) return set_err(XDGCU_ERR_INVALID_ARG, "null argument");
  const std::string k(key);
  if (k == "trace_occupancy") *value = c->trace_occupancy;
  else if (k == "trace_node_iters") *value = c->trace_node_iters;
  else if (k == "trace_node_iters_fp64") *value = c->trace_node_iters_fp64;
  else if (k == "trace_node_iters_direct") *value = c->trace_node_iters_direct;
  else if (k == "trace_flush_wait") *value = c->trace_flush_wait;
  else if (k == "trace_stack") *value = c->trace_stack;
  else if (k == "trace_grab") *value = c->trace_grab;
  else if (k == "trace_sort_min") *value = c->trace_sort_min;
  else if (k == "particle_event_wait") *value = c->particle_event_wait;
  else if (k == "transport_event_wait") *value = c->transport_event_wait;
  else if (k == "leaf_max") *value = c->leaf_max;
  else if (k == "node_width") *value = c->node_width;
  else if (k == "bvh_sah") *value = c->bvh_sah;
  else if (k == "bvh_prim_cost") *value = c->bvh_prim_cost;
  else if (k == "walk_queue") *value = c->walk_queue;
  else if (k == "walk_flush_wait") *value = c->walk_flush_wait;
  else if (k == "walk_sort_min") *value = c->walk_sort_min;
  else if (k == "host_direct") *value = c->host_direct;
  else if (k == "walk_edge_table") *value = c->walk_edge_table;
  else if (k == "trace_edge_table") *value = c->trace_edge_table;
  else if (k == "closest_bound") *value = c->closest_bound;
  else if (k == "closest_node_steps") *value = c->closest_node_steps;
  else if (k == "closest_node_steps_fp64") *value = c->closest_node_steps_fp64;
  else if (k == "find_node_steps_fp64") *value = c->find_node_steps_fp64;
  else if (k == "segments_walk_cap") *value = c->segments_walk_cap;
  else if (k == "find_element_phased") *value = c->find_phased;
  else if (k == "packed_walk_passes") *value = c->packed_passes;
  else if (k == "closest_step_budget") *value = c->closest_budget;
  else if (k == "closest_sort_min") *value = c->closest_sort_min;
  else if (k == "find_sort_min") *value = c->find_sort_min;
  else if (k == "scratch_keep_bytes") *value = c->keep_bytes;
  else if (k == "scratch_bytes_reserved" || k == "scratch_bytes_high") {
    uint64_t v = 0;
    if (c->pool &&
        cudaMemPoolGetAttribute(c->pool,
                                k == "scratch_bytes_high" ? cudaMemPoolAttrUsedMemHigh
                                                          : cudaMemPoolAttrReservedMemCurrent,
                                &v) != cudaSuccess)
      return set_err(XDGCU_ERR_CUDA, "scratch pool");
    *value = (int64_t)v;
  }
  else if (k == "walk_edges") *value = c->n_edges;
  else if (k == "pageable_direct") *value = c->pageable_direct ? 1 : 0;
  else if (k == "host_direct_choice") *value = c->hd_choice;
  else return set_err(XDGCU_ERR_NOT_FOUND, "unknown tuning key " + k);
  return XDGCU_OK;
}

int xdgcu_set_counting(xdgcu_ctx* c, int32_t enable) {
  if (!c) return set_err(XDGCU_ERR_INVALID_ARG, "null context");
  c->counting = enable != 0;
  return XDGCU_OK;
}

int xdgcu_get_counters(xdgcu_ctx* c, int64_t counters[8]) {
  CHECK_CTX(c);
  if (!counters) return set_err(XDGCU_ERR_INVALID_ARG, "null output");
  for (int k = 0; k < 8; ++k) counters[k] = 0;
  if (!c->d_counters.p) return XDGCU_OK;
  if (c->counter_stream) API_CUDA(cudaStreamSynchronize(c->counter_stream), "sync");
  unsigned long long h[CNT_N];
  API_CUDA(cudaMemcpy(h, c->d_counters.p, sizeof h, cudaMemcpyDeviceToHost), "counters");
  for (int k = 0; k < 8; ++k) counters[k] = (int64_t)h[k];
  return XDGCU_OK;
}

// ---------------------------------------------------------------------------
// surface queries
// ---------------------------------------------------------------------------

static int surface_query(xdgcu_ctx* c, int mode, int32_t tree, const int32_t* ray_trees, int64_t n,
                         const double* org, const double* dir, const double* tmax,
                         int32_t orientation, const int32_t* excl_off, const int32_t* excl_ids,
                         double* t_out, int32_t* surf_out, int32_t* face_out, int32_t* flag_out,
                         double* dist_out, int32_t* status, int32_t precision, void* stream) {
  CHECK_CTX(c);
  if (n < 0) return set_err(XDGCU_ERR_INVALID_ARG, "negative ray count");
  if (precision != XDGCU_FP64 && precision != XDGCU_MIXED)
    return set_err(XDGCU_ERR_INVALID_ARG, "precision must be XDGCU_FP64 or XDGCU_MIXED");
  if (n == 0) return XDGCU_OK;
  if (!org || (!dir && mode != MODE_PIV && mode != MODE_FIND_VOLUME))
    return set_err(XDGCU_ERR_INVALID_ARG, "null origins/directions");
  if (mode == MODE_RAY_FIRE && (!t_out || !surf_out))
    return set_err(XDGCU_ERR_INVALID_ARG, "ray_fire: t_out and surface_out are required");
  if (mode != MODE_RAY_FIRE && !flag_out) return set_err(XDGCU_ERR_INVALID_ARG, "null output");
  if ((excl_off == nullptr) != (excl_ids == nullptr))
    return set_err(XDGCU_ERR_INVALID_ARG, "exclusions need both offsets and ids");
  if (mode == MODE_RAY_FIRE && orientation != XDGCU_ANY && orientation != XDGCU_EXITING &&
      orientation != XDGCU_ENTERING)
    return set_err(XDGCU_ERR_INVALID_ARG, "bad orientation");
  if (mode != MODE_FIND_VOLUME && !ray_trees && (tree < 1 || tree > (int32_t)c->surf_trees.size()))
    return set_err(XDGCU_ERR_NOT_FOUND, "no such surface tree");
  if (mode == MODE_FIND_VOLUME && !c->has_volume_map)
    return set_err(XDGCU_ERR_STATE, "find_volume: no volume map (xdgcu_set_volume_map)");
  {
    std::lock_guard<std::mutex> g(c->mu);
    int rc = sync_surfaces(c);
    if (rc) return rc;
    rc = sync_tree_tables(c);
    if (rc) return rc;
  }
  const int kind = classify({ray_trees, org, dir, tmax, excl_off, excl_ids, t_out, surf_out,
                             face_out, flag_out, dist_out, status});
  if (kind < 0) return set_err(XDGCU_ERR_INVALID_ARG, "host and device pointers mixed in one call");
  SurfArgs a{};
  a.trees = c->d_surf_trees.p;
  a.n_trees = (int32_t)c->surf_trees.size();
  a.tree = tree;
  a.n = n;
  a.orientation = orientation;
  a.tri_face = c->d_tri_face.p;
  a.tri_surf = c->d_tri_surf.p;
  a.surf_id = c->d_surf_id.p;
  a.surf_rev_tree = c->d_surf_rev.p;
  a.occupancy = c->trace_occupancy;
  a.prim_edges = c->trace_edge_table;
  a.tri_prime = c->d_tri_prime.p;
  a.node_iters = precision == XDGCU_MIXED ? c->trace_node_iters : c->trace_node_iters_fp64;
  a.flush_wait = c->trace_flush_wait;
  a.stack = trace_stack_for(c);
  a.vol_ids = c->d_vol_ids.p;
  a.vol_trees = c->d_vol_trees.p;
  a.n_vols = c->n_vols;
  a.ipc_volume = c->ipc_volume;
  cudaStream_t st = (cudaStream_t)stream;
  // origin extent for the coherent ray order: the bounds of the trees queried
  double extent = 0.0;
  if (mode == MODE_FIND_VOLUME || ray_trees) {
    for (auto& t : c->surf_trees) extent = std::max(extent, (double)t->dev.max_abs);
  } else {
    extent = (double)c->surf_trees[tree - 1]->dev.max_abs;
  }
  const bool mixed = precision == XDGCU_MIXED;
  if (kind == 1) {
    a.ray_trees = ray_trees;
    a.org = org;
    a.dir = dir;
    a.tmax = tmax;
    a.excl_off = excl_off;
    a.excl_ids = excl_ids;
    a.t_out = t_out;
    a.surf_out = surf_out;
    a.face_out = face_out;
    a.flag_out = flag_out;
    a.dist_out = dist_out;
    a.status = status;
    int rc = begin_query(c, st, &a.counters);
    if (rc) return rc;
    API_CUDA(launch_trace(c, mode, mixed, a, extent, st), "query launch");
    return XDGCU_OK;
  }
  Slot* s = get_slot(c);
  if (!s) return set_err(XDGCU_ERR_CUDA, "staging stream creation failed");
  int64_t n_excl = 0;
  if (excl_off) n_excl = excl_off[n];
  if (n_excl < 0) return set_err(XDGCU_ERR_INVALID_ARG, "bad exclusion offsets");
  Arr A_eo{excl_off, nullptr, excl_off ? sizeof(int32_t) * (n + 1) : 0};
  Arr A_ei{excl_ids, nullptr, excl_ids ? sizeof(int32_t) * std::max<int64_t>(1, n_excl) : 0};
  if (excl_off && n_excl == 0) A_ei.host_in = nullptr;
  RayArr R_trees{ray_trees, nullptr, ray_trees ? sizeof(int32_t) : 0};
  RayArr R_org{org, nullptr, sizeof(double) * 3}, R_dir{dir, nullptr, dir ? sizeof(double) * 3 : 0};
  RayArr R_tmax{tmax, nullptr, tmax ? sizeof(double) : 0};
  RayArr R_t{nullptr, t_out, t_out ? sizeof(double) : 0};
  RayArr R_s{nullptr, surf_out, surf_out ? sizeof(int32_t) : 0};
  RayArr R_f{nullptr, face_out, face_out ? sizeof(int32_t) : 0};
  RayArr R_fl{nullptr, flag_out, flag_out ? sizeof(int32_t) : 0};
  RayArr R_d{nullptr, dist_out, dist_out ? sizeof(double) : 0};
  RayArr R_st{nullptr, status, status ? sizeof(int32_t) : 0};
  auto at = [](const RayArr& r, int64_t first) -> char* {
    return r.dev ? r.dev + r.per_ray * first : nullptr;
  };
  return run_staged(
      c, s, st, n, {&A_eo, &A_ei},
      {&R_trees, &R_org, &R_dir, &R_tmax, &R_t, &R_s, &R_f, &R_fl, &R_d, &R_st}, &a.counters,
      [&](int64_t first, int64_t cnt, cudaStream_t cs, bool chunked) {
        SurfArgs b = a;
        b.n = cnt;
        b.ray_trees = (const int32_t*)at(R_trees, first);
        b.org = (const double*)at(R_org, first);
        b.dir = (const double*)at(R_dir, first);
        b.tmax = (const double*)at(R_tmax, first);
        b.excl_off = A_eo.dev ? (const int32_t*)A_eo.dev + first : nullptr;
        b.excl_ids = (const int32_t*)A_ei.dev;
        b.t_out = (double*)at(R_t, first);
        b.surf_out = (int32_t*)at(R_s, first);
        b.face_out = (int32_t*)at(R_f, first);
        b.flag_out = (int32_t*)at(R_fl, first);
        b.dist_out = (double*)at(R_d, first);
        b.status = (int32_t*)at(R_st, first);
        // rays read in place from host memory take their own node steps per
        // leaf phase (1e7 rays: 6 steps 6.93 ms, 8 7.03, 4 7.39, 12 7.48,
        // while from device arrays 4 steps were best, 6.45 ms)
        if (mixed && R_org.direct) b.node_iters = c->trace_node_iters_direct;
        // a chunk's launch takes rays from the work queue, so its tail is short
        return launch_trace(c, mode, mixed, b, extent, cs, chunked ? kChunkGrab : 0);
      });
}

int xdgcu_ray_fire(xdgcu_ctx* c, int32_t tree, const int32_t* ray_trees, int64_t n,
                   const double* origins, const double* directions, const double* dist_limit,
                   int32_t orientation, const int32_t* excl_offsets, const int32_t* excl_ids,
                   double* t_out, int32_t* surface_out, int32_t* face_out, int32_t* status,
                   int32_t precision, void* stream) {
  return surface_query(c, MODE_RAY_FIRE, tree, ray_trees, n, origins, directions, dist_limit,
                       orientation, excl_offsets, excl_ids, t_out, surface_out, face_out, nullptr,
                       nullptr, status, precision, stream);
}

int xdgcu_point_in_volume(xdgcu_ctx* c, int32_t tree, const int32_t* ray_trees, int64_t n,
                          const double* points, const double* directions,
                          const int32_t* excl_offsets, const int32_t* excl_ids, int32_t* inside_out,
                          int32_t* status, int32_t precision, void* stream) {
  return surface_query(c, MODE_PIV, tree, ray_trees, n, points, directions, nullptr, XDGCU_ANY,
                       excl_offsets, excl_ids, nullptr, nullptr, nullptr, inside_out, nullptr,
                       status, precision, stream);
}

int xdgcu_set_volume_map(xdgcu_ctx* c, int32_t n_volumes, const int32_t* volume_ids,
                         const int32_t* surface_trees, int32_t implicit_complement) {
  CHECK_CTX(c);
  if (n_volumes < 0 || (n_volumes > 0 && (!volume_ids || !surface_trees)))
    return set_err(XDGCU_ERR_INVALID_ARG, "set_volume_map: bad arguments");
  std::vector<int32_t> ids, trees;
  for (int32_t k = 0; k < n_volumes; ++k) {
    if (volume_ids[k] == implicit_complement) continue;  // xdg.cpp:119
    if (surface_trees[k] < 1 || surface_trees[k] > (int32_t)c->surf_trees.size())
      return set_err(XDGCU_ERR_NOT_FOUND, "set_volume_map: no such surface tree");
    ids.push_back(volume_ids[k]);
    trees.push_back(surface_trees[k]);
  }
  std::lock_guard<std::mutex> g(c->mu);
  const int64_t m = std::max<size_t>(1, ids.size());
  API_CUDA(c->d_vol_ids.alloc(m), "alloc volume map");
  API_CUDA(c->d_vol_trees.alloc(m), "alloc volume map");
  if (!ids.empty()) {
    API_CUDA(cudaMemcpy(c->d_vol_ids.p, ids.data(), sizeof(int32_t) * ids.size(),
                        cudaMemcpyHostToDevice), "upload volume map");
    API_CUDA(cudaMemcpy(c->d_vol_trees.p, trees.data(), sizeof(int32_t) * trees.size(),
                        cudaMemcpyHostToDevice), "upload volume map");
  }
  c->n_vols = (int32_t)ids.size();
  c->ipc_volume = implicit_complement;
  c->has_volume_map = true;
  return XDGCU_OK;
}

int xdgcu_find_volume(xdgcu_ctx* c, int64_t n, const double* points, const double* directions,
                      int32_t* volume_out, int32_t* status, int32_t precision, void* stream) {
  return surface_query(c, MODE_FIND_VOLUME, 0, nullptr, n, points, directions, nullptr, XDGCU_ANY,
                       nullptr, nullptr, nullptr, nullptr, nullptr, volume_out, nullptr, status,
                       precision, stream);
}

int xdgcu_occluded(xdgcu_ctx* c, int32_t tree, const int32_t* ray_trees, int64_t n,
                   const double* origins, const double* directions, int32_t* occluded_out,
                   double* dist_out, int32_t* status, int32_t precision, void* stream) {
  return surface_query(c, MODE_OCCLUDED, tree, ray_trees, n, origins, directions, nullptr,
                       XDGCU_ANY, nullptr, nullptr, nullptr, nullptr, nullptr, occluded_out,
                       dist_out, status, precision, stream);
}

// ---------------------------------------------------------------------------
// point queries
// ---------------------------------------------------------------------------

// A closest or find_element launch over one batch: when the batch has at
// least closest_sort_min (find_sort_min) points, in the order of [tree |
// Morton code of the point] (ray_order without directions, in
// stream-ordered scratch freed after the launch), so that the points of a
// warp share their upper nodes and take similar work.
static cudaError_t launch_points_ordered(xdgcu_ctx* c, bool closest, bool mixed, PointArgs a,
                                         double extent, bool phased, cudaStream_t s) {
  a.order = nullptr;
  const int64_t smin = closest ? c->closest_sort_min : c->find_sort_min;
  const bool sort = smin > 0 && a.n >= smin && a.n < ((int64_t)1 << 31) && extent > 0.0;
  auto launch = [&]() {
    return closest ? launch_closest(mixed, a, s) : launch_find_element(mixed, a, s, phased);
  };
  if (!sort) return launch();
  const size_t ord_bytes = (sizeof(int32_t) * (size_t)a.n + 255) & ~(size_t)255;
  const size_t scr = ray_order_scratch_bytes(a.n);
  char* buf = nullptr;
  cudaError_t e = scratch_alloc(c, (void**)&buf, ord_bytes + scr, s);
  if (e != cudaSuccess) return e;
  e = ray_order(a.pts, nullptr, a.ray_trees, a.n_trees, a.n, extent, (int32_t*)buf,
                buf + ord_bytes, scr, s);
  a.order = (const int32_t*)buf;
  if (e == cudaSuccess) e = launch();
  const cudaError_t f = cudaFreeAsync(buf, s);
  return e != cudaSuccess ? e : f;
}

// phased: the mixed find_element in warp-synchronous phases whatever the
// context's find_element_phased says (points known to lie on tet faces)
static int point_query(xdgcu_ctx* c, bool closest, int32_t tree, const int32_t* ray_trees,
                       int64_t n, const double* pts, double* dist_out, int32_t* id_out,
                       int32_t* index_out, int32_t* status, int32_t precision, void* stream,
                       bool phased = false) {
  CHECK_CTX(c);
  if (n < 0) return set_err(XDGCU_ERR_INVALID_ARG, "negative point count");
  if (precision != XDGCU_FP64 && precision != XDGCU_MIXED)
    return set_err(XDGCU_ERR_INVALID_ARG, "precision must be XDGCU_FP64 or XDGCU_MIXED");
  if (n == 0) return XDGCU_OK;
  if (!pts) return set_err(XDGCU_ERR_INVALID_ARG, "null points");
  if (closest && !dist_out) return set_err(XDGCU_ERR_INVALID_ARG, "closest: dist_out required");
  if (!closest && !id_out && !index_out)
    return set_err(XDGCU_ERR_INVALID_ARG, "find_element: an output is required");
  const int32_t ntrees = (int32_t)(closest ? c->surf_trees.size() : c->elem_trees.size());
  if (!ray_trees && (tree < 1 || tree > ntrees))
    return set_err(XDGCU_ERR_NOT_FOUND, closest ? "no such surface tree" : "no such element tree");
  {
    std::lock_guard<std::mutex> g(c->mu);
    int rc = sync_surfaces(c);
    if (rc) return rc;
    rc = sync_tree_tables(c);
    if (rc) return rc;
  }
  const int kind = classify({ray_trees, pts, dist_out, id_out, index_out, status});
  if (kind < 0) return set_err(XDGCU_ERR_INVALID_ARG, "host and device pointers mixed in one call");
  PointArgs a{};
  a.trees = closest ? c->d_surf_trees.p : c->d_elem_trees.p;
  a.n_trees = ntrees;
  a.tree = tree;
  a.n = n;
  a.tri_face = c->d_tri_face.p;
  a.tri_cb = closest && c->closest_bound ? c->d_tri_cb.p : nullptr;
  a.node_steps = closest ? (precision == XDGCU_MIXED ? c->closest_node_steps
                                                     : c->closest_node_steps_fp64)
                         : c->find_node_steps_fp64;  // find_element in phases
  phased = phased || c->find_phased != 0;
  a.elem_ids = c->d_elem_ids.p;
  cudaStream_t st = (cudaStream_t)stream;
  // closest: a point's search passing closest_step_budget steps is finished
  // by a whole warp; its flag and best so far live in scratch of n entries,
  // allocated on the stream the kernels are ordered after
  auto defer_scratch = [&](CallScratch& S) -> cudaError_t {
    if (!closest || c->closest_budget <= 0) return cudaSuccess;
    cudaError_t e = S.get(&a.deferred, n);
    if (e == cudaSuccess) e = S.get(&a.def_best, n);
    if (e == cudaSuccess) e = S.get(&a.def_face, n);
    if (e == cudaSuccess) a.step_budget = c->closest_budget;
    return e;
  };
  // the bounds of the trees queried, for the points' Morton order
  double extent = 0.0;
  {
    const auto& trees = closest ? c->surf_trees : c->elem_trees;
    if (ray_trees) {
      for (auto& t : trees) extent = std::max(extent, (double)t->dev.max_abs);
    } else {
      extent = (double)trees[tree - 1]->dev.max_abs;
    }
  }
  auto launch = [&]() -> cudaError_t {
    return launch_points_ordered(c, closest, precision == XDGCU_MIXED, a, extent, phased, st);
  };
  if (kind == 1) {
    a.ray_trees = ray_trees;
    a.pts = pts;
    a.dist_out = dist_out;
    a.id_out = id_out;
    a.index_out = index_out;
    a.status = status;
    int rc = begin_query(c, st, &a.counters);
    if (rc) return rc;
    CallScratch S(st, c->pool);
    API_CUDA(defer_scratch(S), "closest scratch");
    API_CUDA(launch(), "query launch");
    return XDGCU_OK;
  }
  Slot* s = get_slot(c);
  if (!s) return set_err(XDGCU_ERR_CUDA, "staging stream creation failed");
  // (the chunks' launches alternate between the slot's streams; the second
  // waits for the first before its first launch)
  CallScratch S(s->stream, c->pool);
  API_CUDA(defer_scratch(S), "closest scratch");
  RayArr R_trees{ray_trees, nullptr, ray_trees ? sizeof(int32_t) : 0};
  RayArr R_p{pts, nullptr, sizeof(double) * 3};
  RayArr R_d{nullptr, dist_out, dist_out ? sizeof(double) : 0};
  RayArr R_i{nullptr, id_out, id_out ? sizeof(int32_t) : 0};
  RayArr R_x{nullptr, index_out, index_out ? sizeof(int32_t) : 0};
  RayArr R_st{nullptr, status, status ? sizeof(int32_t) : 0};
  auto at = [](const RayArr& r, int64_t first) -> char* {
    return r.dev ? r.dev + r.per_ray * first : nullptr;
  };
  return run_staged(c, s, st, n, {}, {&R_trees, &R_p, &R_d, &R_i, &R_x, &R_st}, &a.counters,
                    [&](int64_t first, int64_t cnt, cudaStream_t cs, bool) {
                      PointArgs b = a;
                      b.n = cnt;
                      b.ray_trees = (const int32_t*)at(R_trees, first);
                      b.pts = (const double*)at(R_p, first);
                      b.dist_out = (double*)at(R_d, first);
                      b.id_out = (int32_t*)at(R_i, first);
                      b.index_out = (int32_t*)at(R_x, first);
                      b.status = (int32_t*)at(R_st, first);
                      if (a.deferred) {  // this chunk's slice of the closest scratch
                        b.deferred = a.deferred + first;
                        b.def_best = a.def_best + first;
                        b.def_face = a.def_face + first;
                      }
                      return launch_points_ordered(c, closest, precision == XDGCU_MIXED, b,
                                                   extent, phased, cs);
                    });
}

int xdgcu_closest(xdgcu_ctx* c, int32_t tree, const int32_t* ray_trees, int64_t n,
                  const double* points, double* dist_out, int32_t* face_out, int32_t* status,
                  int32_t precision, void* stream) {
  return point_query(c, true, tree, ray_trees, n, points, dist_out, face_out, nullptr, status,
                     precision, stream);
}

int xdgcu_find_element(xdgcu_ctx* c, int32_t tree, const int32_t* ray_trees, int64_t n,
                       const double* points, int32_t* elem_id_out, int32_t* elem_index_out,
                       int32_t* status, int32_t precision, void* stream) {
  return point_query(c, false, tree, ray_trees, n, points, nullptr, elem_id_out, elem_index_out,
                     status, precision, stream);
}

// ---------------------------------------------------------------------------
// element walk
// ---------------------------------------------------------------------------

static int walk_query(xdgcu_ctx* c, bool walk, int64_t n, const int32_t* start, const double* org,
                      const double* dir, const double* dist, int32_t max_segs, int32_t* seg_elem,
                      double* seg_len, int32_t* seg_count, int32_t* next_out, double* dist_out,
                      int32_t* status, int32_t precision, void* stream) {
  CHECK_CTX(c);
  if (n < 0) return set_err(XDGCU_ERR_INVALID_ARG, "negative track count");
  if (precision != XDGCU_FP64 && precision != XDGCU_MIXED)
    return set_err(XDGCU_ERR_INVALID_ARG, "precision must be XDGCU_FP64 or XDGCU_MIXED");
  if (!c->has_tets) return set_err(XDGCU_ERR_STATE, "no tet mesh set");
  if (n == 0) return XDGCU_OK;
  if (!start || !org || !dir) return set_err(XDGCU_ERR_INVALID_ARG, "null inputs");
  if (walk && (!dist || !seg_elem || !seg_len || !seg_count || max_segs <= 0))
    return set_err(XDGCU_ERR_INVALID_ARG, "walk_elements: bad outputs or max_segs");
  if (!walk && (!next_out || !dist_out))
    return set_err(XDGCU_ERR_INVALID_ARG, "next_element: null outputs");
  const int kind = classify({start, org, dir, dist, seg_elem, seg_len, seg_count, next_out,
                             dist_out, status});
  if (kind < 0) return set_err(XDGCU_ERR_INVALID_ARG, "host and device pointers mixed in one call");
  WalkArgs a{};
  a.xyz = c->d_xyz.p;
  a.xyz32 = c->d_xyz32.p;
  a.edge = c->walk_edge_table ? c->d_edge.p : nullptr;
  a.tet_edge = c->d_tet_edge.p;
  a.conn = c->d_conn.p;
  a.adj = c->d_adj.p;
  a.elem_ids = c->d_elem_ids.p;
  a.n_tets = (int32_t)c->n_tet;
  std::memcpy(a.face, c->face, sizeof(a.face));
  a.walk_queue = c->walk_queue;
  a.flush_wait = c->walk_flush_wait;
  a.n = n;
  a.max_segs = max_segs;
  cudaStream_t st = (cudaStream_t)stream;
  auto launch = [&]() -> cudaError_t {
    return walk ? launch_walk(precision == XDGCU_MIXED, c->face_order, a, st)
                : launch_next_element(precision == XDGCU_MIXED, c->face_order, a, st);
  };
  if (kind == 1) {
    a.start = start;
    a.org = org;
    a.dir = dir;
    a.dist = dist;
    a.seg_elem = seg_elem;
    a.seg_len = seg_len;
    a.seg_count = seg_count;
    a.next_out = next_out;
    a.dist_out = dist_out;
    a.status = status;
    int rc = begin_query(c, st, &a.counters);
    if (rc) return rc;
    if (!walk) {
      API_CUDA(launch(), "walk launch");
      return XDGCU_OK;
    }
    return with_length_order(c, a, st, [&]() -> int {
      API_CUDA(launch(), "walk launch");
      return XDGCU_OK;
    });
  }
  Slot* s = get_slot(c);
  if (!s) return set_err(XDGCU_ERR_CUDA, "staging stream creation failed");
  if (!st) st = s->stream;
  const size_t ns = walk ? (size_t)n * (size_t)max_segs : 0;
  Arr A_s{start, nullptr, sizeof(int32_t) * n};
  Arr A_o{org, nullptr, sizeof(double) * 3 * n}, A_d{dir, nullptr, sizeof(double) * 3 * n};
  Arr A_l{dist, nullptr, walk ? sizeof(double) * n : 0};
  Arr A_se{nullptr, seg_elem, sizeof(int32_t) * ns}, A_sl{nullptr, seg_len, sizeof(double) * ns};
  Arr A_sc{nullptr, seg_count, walk ? sizeof(int32_t) * n : 0};
  Arr A_no{nullptr, next_out, walk ? 0 : sizeof(int32_t) * n};
  Arr A_do{nullptr, dist_out, walk ? 0 : sizeof(double) * n};
  Arr A_st{nullptr, status, status ? sizeof(int32_t) * n : 0};
  std::vector<Arr*> all = {&A_s, &A_o, &A_d, &A_l, &A_se, &A_sl, &A_sc, &A_no, &A_do, &A_st};
  int rc = stage_in(c, s, all, st);
  if (rc) return rc;
  a.start = (const int32_t*)A_s.dev;
  a.org = (const double*)A_o.dev;
  a.dir = (const double*)A_d.dev;
  a.dist = (const double*)A_l.dev;
  a.seg_elem = (int32_t*)A_se.dev;
  a.seg_len = (double*)A_sl.dev;
  a.seg_count = (int32_t*)A_sc.dev;
  a.next_out = (int32_t*)A_no.dev;
  a.dist_out = (double*)A_do.dev;
  a.status = (int32_t*)A_st.dev;
  rc = begin_query(c, st, &a.counters);
  if (rc) return rc;
  if (walk) {
    rc = with_length_order(c, a, st, [&]() -> int {
      API_CUDA(launch(), "walk launch");
      return XDGCU_OK;
    });
    if (rc) return rc;
  } else {
    API_CUDA(launch(), "walk launch");
  }
  return stage_out(all, st);
}

int xdgcu_walk_elements_packed(xdgcu_ctx* c, int64_t n, const int32_t* start_index,
                               const double* start, const double* u, const double* distance,
                               int32_t max_segs, int64_t capacity, int32_t* seg_elem,
                               double* seg_len, int64_t* offsets, int32_t* status,
                               int32_t precision, void* stream) {
  CHECK_CTX(c);
  if (n < 0 || capacity < 0) return set_err(XDGCU_ERR_INVALID_ARG, "negative size");
  if (precision != XDGCU_FP64 && precision != XDGCU_MIXED)
    return set_err(XDGCU_ERR_INVALID_ARG, "precision must be XDGCU_FP64 or XDGCU_MIXED");
  if (!c->has_tets) return set_err(XDGCU_ERR_STATE, "no tet mesh set");
  if (!offsets) return set_err(XDGCU_ERR_INVALID_ARG, "walk_elements_packed: offsets required");
  if (n > 0 && (!start_index || !start || !u || !distance || max_segs <= 0))
    return set_err(XDGCU_ERR_INVALID_ARG, "walk_elements_packed: bad inputs");
  if (capacity > 0 && (!seg_elem || !seg_len))
    return set_err(XDGCU_ERR_INVALID_ARG, "walk_elements_packed: null segment arrays");
  const int kind = classify({start_index, start, u, distance, seg_elem, seg_len, offsets, status});
  if (kind < 0) return set_err(XDGCU_ERR_INVALID_ARG, "host and device pointers mixed in one call");
  WalkArgs a{};
  a.xyz = c->d_xyz.p;
  a.xyz32 = c->d_xyz32.p;
  a.edge = c->walk_edge_table ? c->d_edge.p : nullptr;
  a.tet_edge = c->d_tet_edge.p;
  a.conn = c->d_conn.p;
  a.adj = c->d_adj.p;
  a.elem_ids = c->d_elem_ids.p;
  a.n_tets = (int32_t)c->n_tet;
  std::memcpy(a.face, c->face, sizeof(a.face));
  a.walk_queue = c->walk_queue;
  a.flush_wait = c->walk_flush_wait;
  a.n = n;
  a.max_segs = max_segs;
  a.capacity = capacity;
  cudaStream_t st = (cudaStream_t)stream;
  const bool mixed = precision == XDGCU_MIXED;
  auto run = [&](cudaStream_t s) -> int {
    if (c->packed_passes == 1 && n < ((int64_t)1 << 31)) {
      bool no_memory = false;
      const int rc = walk_packed_rounds(c, mixed, a, s, &no_memory);
      if (!no_memory) return rc;
    }
    // (or without the temporary memory): a count walk, the scan, an emit walk
    return with_length_order(c, a, s, [&]() -> int {
      a.out_mode = WALK_COUNT;
      API_CUDA(launch_walk(mixed, c->face_order, a, s), "walk (count)");
      int64_t* sums = nullptr;
      API_CUDA(scratch_alloc(c, (void**)&sums, sizeof(int64_t) * scan_scratch_entries(n), s),
               "scan scratch");
      cudaError_t e = scan_offsets(a.offsets, n, sums, s);
      cudaFreeAsync(sums, s);
      API_CUDA(e, "scan");
      a.out_mode = WALK_PACKED;
      API_CUDA(launch_walk(mixed, c->face_order, a, s), "walk (emit)");
      return XDGCU_OK;
    });
  };
  if (kind == 1) {
    a.start = start_index;
    a.org = start;
    a.dir = u;
    a.dist = distance;
    a.seg_elem = seg_elem;
    a.seg_len = seg_len;
    a.offsets = offsets;
    a.status = status;
    return n > 0 ? run(st) : (cudaMemsetAsync(offsets, 0, sizeof(int64_t), st) == cudaSuccess
                                  ? XDGCU_OK
                                  : set_err(XDGCU_ERR_CUDA, "memset"));
  }
  if (n == 0) {
    offsets[0] = 0;
    return XDGCU_OK;
  }
  Slot* s = get_slot(c);
  if (!s) return set_err(XDGCU_ERR_CUDA, "staging stream creation failed");
  if (!st) st = s->stream;
  Arr A_s{start_index, nullptr, sizeof(int32_t) * n};
  Arr A_o{start, nullptr, sizeof(double) * 3 * n}, A_d{u, nullptr, sizeof(double) * 3 * n};
  Arr A_l{distance, nullptr, sizeof(double) * n};
  Arr A_off{nullptr, nullptr, sizeof(int64_t) * (n + 1)};
  Arr A_se{nullptr, nullptr, sizeof(int32_t) * capacity}, A_sl{nullptr, nullptr, sizeof(double) * capacity};
  Arr A_st{nullptr, status, status ? sizeof(int32_t) * n : 0};
  std::vector<Arr*> all = {&A_s, &A_o, &A_d, &A_l, &A_off, &A_se, &A_sl, &A_st};
  int rc = stage_in(c, s, all, st);
  if (rc) return rc;
  a.start = (const int32_t*)A_s.dev;
  a.org = (const double*)A_o.dev;
  a.dir = (const double*)A_d.dev;
  a.dist = (const double*)A_l.dev;
  a.offsets = (int64_t*)A_off.dev;
  a.seg_elem = (int32_t*)A_se.dev;
  a.seg_len = (double*)A_sl.dev;
  a.status = (int32_t*)A_st.dev;
  rc = run(st);
  if (rc) return rc;
  API_CUDA(cudaMemcpyAsync(offsets, A_off.dev, sizeof(int64_t) * (n + 1), cudaMemcpyDeviceToHost, st),
           "D2H");
  rc = stage_out({&A_st}, st);
  if (rc) return rc;
  const int64_t used = std::min(offsets[n], capacity);
  if (used > 0) {
    API_CUDA(cudaMemcpyAsync(seg_elem, A_se.dev, sizeof(int32_t) * used, cudaMemcpyDeviceToHost, st),
             "D2H");
    API_CUDA(cudaMemcpyAsync(seg_len, A_sl.dev, sizeof(double) * used, cudaMemcpyDeviceToHost, st),
             "D2H");
    API_CUDA(cudaStreamSynchronize(st), "sync");
  }
  return XDGCU_OK;
}

int xdgcu_next_element(xdgcu_ctx* c, int64_t n, const int32_t* elem_index, const double* positions,
                       const double* directions, int32_t* next_out, double* dist_out,
                       int32_t* status, int32_t precision, void* stream) {
  return walk_query(c, false, n, elem_index, positions, directions, nullptr, 0, nullptr, nullptr,
                    nullptr, next_out, dist_out, status, precision, stream);
}

int xdgcu_walk_elements(xdgcu_ctx* c, int64_t n, const int32_t* start_index, const double* start,
                        const double* u, const double* distance, int32_t max_segs,
                        int32_t* seg_elem, double* seg_len, int32_t* seg_count, int32_t* status,
                        int32_t precision, void* stream) {
  return walk_query(c, true, n, start_index, start, u, distance, max_segs, seg_elem, seg_len,
                    seg_count, nullptr, nullptr, status, precision, stream);
}

int xdgcu_set_boundary_face_elements(xdgcu_ctx* c, int64_t n, const int32_t* face_ids,
                                     const int32_t* elem_index) {
  CHECK_CTX(c);
  if (n < 0 || (n > 0 && (!face_ids || !elem_index)))
    return set_err(XDGCU_ERR_INVALID_ARG, "set_boundary_face_elements: bad arguments");
  if (!c->has_tets) return set_err(XDGCU_ERR_STATE, "set_boundary_face_elements: no tet mesh set");
  std::vector<std::pair<int32_t, int32_t>> m;
  m.reserve((size_t)n);
  for (int64_t k = 0; k < n; ++k) {
    if (elem_index[k] < -1 || elem_index[k] >= c->n_tet)
      return set_err(XDGCU_ERR_INVALID_ARG, "set_boundary_face_elements: tet index out of range");
    if (elem_index[k] >= 0) m.emplace_back(face_ids[k], elem_index[k]);
  }
  std::sort(m.begin(), m.end());
  for (size_t k = 1; k < m.size(); ++k)
    if (m[k].first == m[k - 1].first)
      return set_err(XDGCU_ERR_INVALID_ARG, "set_boundary_face_elements: face id given twice");
  std::vector<int32_t> f(m.size()), e(m.size());
  for (size_t k = 0; k < m.size(); ++k) {
    f[k] = m[k].first;
    e[k] = m[k].second;
  }
  std::lock_guard<std::mutex> g(c->mu);
  const int64_t cnt = std::max<int64_t>(1, (int64_t)m.size());
  API_CUDA(c->d_bfe_face.alloc(cnt), "alloc boundary faces");
  API_CUDA(c->d_bfe_elem.alloc(cnt), "alloc boundary faces");
  if (!m.empty()) {
    API_CUDA(cudaMemcpy(c->d_bfe_face.p, f.data(), sizeof(int32_t) * m.size(), cudaMemcpyHostToDevice),
             "upload boundary faces");
    API_CUDA(cudaMemcpy(c->d_bfe_elem.p, e.data(), sizeof(int32_t) * m.size(), cudaMemcpyHostToDevice),
             "upload boundary faces");
  }
  c->n_bfe = (int64_t)m.size();
  return XDGCU_OK;
}

int xdgcu_segments_global(xdgcu_ctx* c, int32_t ipc_tree, int32_t element_tree, int64_t n,
                          const double* starts, const double* ends, int32_t max_segs,
                          int32_t max_rounds, int64_t capacity, int32_t* seg_elem, double* seg_len,
                          int64_t* offsets, int32_t* status, int32_t precision, void* stream) {
  CHECK_CTX(c);
  if (n < 0 || capacity < 0) return set_err(XDGCU_ERR_INVALID_ARG, "negative size");
  if (n >= ((int64_t)1 << 31)) return set_err(XDGCU_ERR_INVALID_ARG, "segments_global: n >= 2^31");
  if (precision != XDGCU_FP64 && precision != XDGCU_MIXED)
    return set_err(XDGCU_ERR_INVALID_ARG, "precision must be XDGCU_FP64 or XDGCU_MIXED");
  if (!c->has_tets) return set_err(XDGCU_ERR_STATE, "no tet mesh set");
  if (!offsets) return set_err(XDGCU_ERR_INVALID_ARG, "segments_global: offsets required");
  if (max_segs <= 0 || max_rounds <= 0)
    return set_err(XDGCU_ERR_INVALID_ARG, "segments_global: max_segs and max_rounds must be > 0");
  if (n > 0 && (!starts || !ends)) return set_err(XDGCU_ERR_INVALID_ARG, "segments_global: null inputs");
  if (capacity > 0 && (!seg_elem || !seg_len))
    return set_err(XDGCU_ERR_INVALID_ARG, "segments_global: null segment arrays");
  if (ipc_tree < 1 || ipc_tree > (int32_t)c->surf_trees.size())
    return set_err(XDGCU_ERR_NOT_FOUND, "segments_global: no such surface tree");
  if (element_tree < 1 || element_tree > (int32_t)c->elem_trees.size())
    return set_err(XDGCU_ERR_NOT_FOUND, "segments_global: no such element tree");
  const int kind = classify({starts, ends, seg_elem, seg_len, offsets, status});
  if (kind < 0) return set_err(XDGCU_ERR_INVALID_ARG, "host and device pointers mixed in one call");
  cudaStream_t st = (cudaStream_t)stream;
  if (kind == 0 && !st) {
    Slot* sl = get_slot(c);
    if (!sl) return set_err(XDGCU_ERR_CUDA, "staging stream creation failed");
    st = sl->stream;
  }
  if (n == 0) {
    if (kind == 0) {
      offsets[0] = 0;
      return XDGCU_OK;
    }
    API_CUDA(cudaMemsetAsync(offsets, 0, sizeof(int64_t), st), "memset");
    return XDGCU_OK;
  }
  const bool mixed = precision == XDGCU_MIXED;
  CallScratch S(st, c->pool);
  // the caller's arrays, or device images of host arrays
  const double* d_starts = starts;
  const double* d_ends = ends;
  int64_t* d_off = offsets;
  int32_t* d_status = status;
  int32_t* d_se = seg_elem;
  double* d_sl = seg_len;
  if (kind == 0) {
    double *ps = nullptr, *pe = nullptr;
    API_CUDA(S.get(&ps, 3 * n), "segments scratch");
    API_CUDA(S.get(&pe, 3 * n), "segments scratch");
    API_CUDA(cudaMemcpyAsync(ps, starts, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, st), "H2D");
    API_CUDA(cudaMemcpyAsync(pe, ends, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, st), "H2D");
    d_starts = ps;
    d_ends = pe;
    API_CUDA(S.get(&d_off, n + 1), "segments scratch");
    d_status = nullptr;
    API_CUDA(S.get(&d_se, capacity), "segments scratch");
    API_CUDA(S.get(&d_sl, capacity), "segments scratch");
  }
  if (!d_status) API_CUDA(S.get(&d_status, n), "segments scratch");
  SegState ss{};
  ss.n = n;
  ss.status = d_status;
  API_CUDA(S.get(&ss.r, 3 * n), "segments scratch");
  API_CUDA(S.get(&ss.u, 3 * n), "segments scratch");
  API_CUDA(S.get(&ss.dist, n), "segments scratch");
  API_CUDA(S.get(&ss.written, n), "segments scratch");
  API_CUDA(S.get(&ss.last, n), "segments scratch");
  API_CUDA(S.get(&ss.stopped, n), "segments scratch");
  API_CUDA(S.get(&ss.wr, 3 * n), "segments scratch");
  API_CUDA(S.get(&ss.wd, n), "segments scratch");
  API_CUDA(S.get(&ss.wsum, n), "segments scratch");
  API_CUDA(S.get(&ss.wcount, n), "segments scratch");
  API_CUDA(S.get(&ss.welem, n), "segments scratch");
  API_CUDA(S.get(&ss.paused, n), "segments scratch");
  int32_t *act = nullptr, *act_next = nullptr, *counters = nullptr, *eid = nullptr, *eidx = nullptr;
  int32_t *out_t = nullptr, *surf = nullptr, *face = nullptr, *loc = nullptr;
  double *pts = nullptr, *ray_org = nullptr, *ray_dir = nullptr, *t_hit = nullptr;
  API_CUDA(S.get(&act, n), "segments scratch");
  API_CUDA(S.get(&act_next, n), "segments scratch");
  API_CUDA(S.get(&counters, 4), "segments scratch");
  API_CUDA(S.get(&eid, n), "segments scratch");
  API_CUDA(S.get(&eidx, n), "segments scratch");
  API_CUDA(S.get(&out_t, n), "segments scratch");
  API_CUDA(S.get(&surf, n), "segments scratch");
  API_CUDA(S.get(&face, n), "segments scratch");
  API_CUDA(S.get(&loc, n), "segments scratch");
  API_CUDA(S.get(&pts, 3 * n), "segments scratch");
  API_CUDA(S.get(&ray_org, 3 * n), "segments scratch");
  API_CUDA(S.get(&ray_dir, 3 * n), "segments scratch");
  API_CUDA(S.get(&t_hit, n), "segments scratch");
  // the walk list and the rounds' walk buffers (seg_walk_round)
  SegWalkBufs B{};
  B.strided_cap = seg_strided_cap(n, c->segments_walk_cap);
  API_CUDA(S.get(&B.walk_t, n), "segments scratch");
  API_CUDA(S.get(&B.walk_start, n), "segments scratch");
  API_CUDA(S.get(&B.wst, n), "segments scratch");
  API_CUDA(S.get(&B.wcnt, n), "segments scratch");
  API_CUDA(S.get(&B.wstop, n), "segments scratch");
  API_CUDA(S.get(&B.wr, 3 * n), "segments scratch");
  API_CUDA(S.get(&B.wu, 3 * n), "segments scratch");
  API_CUDA(S.get(&B.wd, n), "segments scratch");
  API_CUDA(S.get(&B.wsum_in, n), "segments scratch");
  API_CUDA(S.get(&B.wsum_out, n), "segments scratch");
  API_CUDA(S.get(&B.wend_r, 3 * n), "segments scratch");
  API_CUDA(S.get(&B.wend_d, n), "segments scratch");
  API_CUDA(S.get(&B.sk_elem, B.strided_cap), "segments scratch");
  API_CUDA(S.get(&B.sk_len, B.strided_cap), "segments scratch");
  int32_t* n_act = counters;
  int32_t* n_walk = counters + 1;
  int32_t* n_out = counters + 2;
  int32_t* n_loc = counters + 3;
  // one record per round for the final placement of its segments
  std::vector<SegRound> rounds;
  API_CUDA(cudaMemsetAsync(counters, 0, 4 * sizeof(int32_t), st), "memset");
  API_CUDA(seg_init(ss, d_starts, d_ends, act, n_act, st), "segments init");
  int32_t m = 0;
  API_CUDA(read_count(n_act, &m, st), "segments count");
  WalkArgs geo{};
  {
    int fo = 0, dev = 0;
    if (const char* msg = walk_args_for(c, &geo, &fo, &dev)) return set_err(XDGCU_ERR_STATE, msg);
  }
  int32_t round = 0;
  for (; m > 0 && round < max_rounds; ++round) {
    // paused walks resume; the other active tracks are located
    API_CUDA(cudaMemsetAsync(counters + 1, 0, 3 * sizeof(int32_t), st), "memset");
    API_CUDA(seg_split(ss, act, m, B.walk_t, B.walk_start, n_walk, loc, n_loc, st), "segments split");
    int32_t h3[3] = {0, 0, 0};  // n_walk, n_out, n_loc
    API_CUDA(cudaMemcpyAsync(h3, counters + 1, 3 * sizeof(int32_t), cudaMemcpyDeviceToHost, st), "D2H");
    API_CUDA(cudaStreamSynchronize(st), "sync");
    int32_t m_walk = h3[0];
    const int32_t m_loc = h3[2];
    int rc = XDGCU_OK;
    if (m_loc > 0) {
      // find_element(r) in the element tree.  After the first round the
      // points are where walks left the mesh, on its boundary faces, which
      // the phased kernel locates faster (the global loop on three gapped
      // blocks: 3083 -> 3371 Msegs/s)
      API_CUDA(seg_gather_points(ss, loc, m_loc, pts, st), "segments gather");
      rc = point_query(c, false, element_tree, nullptr, m_loc, pts, nullptr, eid, eidx, nullptr,
                       precision, st, round > 0);
      if (rc) return rc;
      API_CUDA(seg_decide(ss, loc, m_loc, eid, eidx, B.walk_t, B.walk_start, n_walk, out_t, ray_org,
                          ray_dir, n_out, st),
               "segments decide");
      int32_t h2[2] = {0, 0};
      API_CUDA(cudaMemcpyAsync(h2, counters + 1, 2 * sizeof(int32_t), cudaMemcpyDeviceToHost, st),
               "D2H");
      API_CUDA(cudaStreamSynchronize(st), "sync");
      m_walk = h2[0];
      const int32_t m_out = h2[1];
      if (m_out > 0) {
        // ray_fire(ipc, r + u * TINY_BIT, u, INFTY, EXITING), then re-entry
        rc = xdgcu_ray_fire(c, ipc_tree, nullptr, m_out, ray_org, ray_dir, nullptr, XDGCU_EXITING,
                            nullptr, nullptr, t_hit, surf, face, nullptr, precision, st);
        if (rc) return rc;
        API_CUDA(seg_reenter(ss, out_t, m_out, t_hit, surf, face, c->d_bfe_face.p, c->d_bfe_elem.p,
                             c->n_bfe, (int32_t)c->n_tet, B.walk_t, B.walk_start, n_walk, st),
                 "segments re-entry");
        API_CUDA(read_count(n_walk, &m_walk, st), "segments count");
      }
    }
    API_CUDA(cudaMemsetAsync(n_act, 0, sizeof(int32_t), st), "memset");
    if (m_walk > 0) {
      // walk_elements(element, r, u, distance) of the round, one pass, at
      // most K segments per track; the walk reports where it stopped and
      // continues each track's sum of lengths
      SegRound R{};
      rc = seg_walk_round(c, mixed, ss, geo, B, m_walk, max_segs, false, act_next, n_act, S, st,
                          nullptr, &R);
      if (rc) return rc;
      rounds.push_back(R);
    }
    API_CUDA(read_count(n_act, &m, st), "segments count");
    std::swap(act, act_next);
  }
  if (m > 0) API_CUDA(seg_stop_active(ss, act, m, XDGCU_RAY_WALK_LIMIT, st), "segments stop");
  // offsets from the per-track totals, then every round's segments to their place
  API_CUDA(seg_counts(ss, d_off, st), "segments counts");
  {
    int64_t* sums = nullptr;
    API_CUDA(S.get(&sums, scan_scratch_entries(n)), "scan scratch");
    API_CUDA(scan_offsets(d_off, n, sums, st), "scan");
  }
  API_CUDA(seg_mark_full(ss, d_off, capacity, st), "segments capacity");
  for (const SegRound& R : rounds)
    API_CUDA(seg_scatter(ss, R.walk_t, R.m, R.off, R.dst_rel, R.seg_elem, R.seg_len, d_off, capacity,
                         d_se, d_sl, st),
             "segments scatter");
  if (kind == 0) {
    API_CUDA(cudaMemcpyAsync(offsets, d_off, sizeof(int64_t) * (n + 1), cudaMemcpyDeviceToHost, st),
             "D2H");
    if (status)
      API_CUDA(cudaMemcpyAsync(status, d_status, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, st), "D2H");
    API_CUDA(cudaStreamSynchronize(st), "sync");
    const int64_t used = std::min(offsets[n], capacity);
    if (used > 0) {
      API_CUDA(cudaMemcpyAsync(seg_elem, d_se, sizeof(int32_t) * used, cudaMemcpyDeviceToHost, st), "D2H");
      API_CUDA(cudaMemcpyAsync(seg_len, d_sl, sizeof(double) * used, cudaMemcpyDeviceToHost, st), "D2H");
      API_CUDA(cudaStreamSynchronize(st), "sync");
    }
  }
  return XDGCU_OK;
}

// ---------------------------------------------------------------------------
// device particle loop over the tet mesh
// ---------------------------------------------------------------------------

int xdgcu_point_in_volumes(xdgcu_ctx* c, int64_t n, const double* points,
                           const double* directions, int32_t n_trees, const int32_t* trees,
                           uint8_t* inside_out, int32_t* status, int32_t precision,
                           void* stream) {
  CHECK_CTX(c);
  if (n < 0 || n_trees < 0) return set_err(XDGCU_ERR_INVALID_ARG, "negative count");
  if (precision != XDGCU_FP64 && precision != XDGCU_MIXED)
    return set_err(XDGCU_ERR_INVALID_ARG, "precision must be XDGCU_FP64 or XDGCU_MIXED");
  if (n == 0 || n_trees == 0) return XDGCU_OK;
  if (!points || !trees || !inside_out) return set_err(XDGCU_ERR_INVALID_ARG, "null argument");
  for (int32_t k = 0; k < n_trees; ++k)
    if (trees[k] < 1 || trees[k] > (int32_t)c->surf_trees.size())
      return set_err(XDGCU_ERR_NOT_FOUND, "point_in_volumes: no such surface tree");
  {
    std::lock_guard<std::mutex> g(c->mu);
    int rc = sync_surfaces(c);
    if (rc) return rc;
    rc = sync_tree_tables(c);
    if (rc) return rc;
  }
  const int kind = classify({points, directions, inside_out, status});
  if (kind < 0) return set_err(XDGCU_ERR_INVALID_ARG, "host and device pointers mixed in one call");
  SurfArgs a{};
  a.trees = c->d_surf_trees.p;
  a.n_trees = (int32_t)c->surf_trees.size();
  a.n = n;
  a.tri_face = c->d_tri_face.p;
  a.tri_surf = c->d_tri_surf.p;
  a.surf_id = c->d_surf_id.p;
  a.surf_rev_tree = c->d_surf_rev.p;
  a.occupancy = c->trace_occupancy;
  a.prim_edges = c->trace_edge_table;
  a.tri_prime = c->d_tri_prime.p;
  a.node_iters = precision == XDGCU_MIXED ? c->trace_node_iters : c->trace_node_iters_fp64;
  a.flush_wait = c->trace_flush_wait;
  a.stack = trace_stack_for(c);
  a.n_vols = n_trees;
  a.vol_stride = n_trees;
  const bool mixed = precision == XDGCU_MIXED;
  double extent = 0.0;
  for (auto& t : c->surf_trees) extent = std::max(extent, (double)t->dev.max_abs);
  cudaStream_t st = (cudaStream_t)stream;
  Slot* s = nullptr;
  if (kind == 0) {
    s = get_slot(c);
    if (!s) return set_err(XDGCU_ERR_CUDA, "staging stream creation failed");
  }
  // the tree list, in stream order before the launches
  cudaStream_t ls = kind == 1 ? st : s->stream;
  int32_t* d_list = nullptr;
  API_CUDA(scratch_alloc(c, (void**)&d_list, sizeof(int32_t) * n_trees, ls), "tree list");
  API_CUDA(cudaMemcpyAsync(d_list, trees, sizeof(int32_t) * n_trees, cudaMemcpyHostToDevice, ls),
           "tree list");
  a.vol_trees = d_list;
  int rc = XDGCU_OK;
  if (kind == 1) {
    a.org = points;
    a.dir = directions;
    a.vol_inside = inside_out;
    a.status = status;
    rc = begin_query(c, st, &a.counters);
    if (!rc) {
      const cudaError_t e = launch_trace(c, MODE_ALL_VOLUMES, mixed, a, extent, st);
      if (e != cudaSuccess) rc = cuda_err(e, "query launch");
    }
    cudaFreeAsync(d_list, st);
    return rc;
  }
  RayArr R_p{points, nullptr, 24}, R_d{directions, nullptr, directions ? 24u : 0u};
  RayArr R_in{nullptr, inside_out, (size_t)n_trees};
  RayArr R_st{nullptr, status, status ? 4u : 0u};
  auto at = [](const RayArr& r, int64_t first) -> char* {
    return r.dev ? r.dev + r.per_ray * first : nullptr;
  };
  rc = run_staged(c, s, st, n, {}, {&R_p, &R_d, &R_in, &R_st}, &a.counters,
                  [&](int64_t first, int64_t cnt, cudaStream_t cs, bool chunked) {
                    SurfArgs b = a;
                    b.n = cnt;
                    b.org = (const double*)at(R_p, first);
                    b.dir = (const double*)at(R_d, first);
                    b.vol_inside = (uint8_t*)at(R_in, first);
                    b.status = (int32_t*)at(R_st, first);
                    return launch_trace(c, MODE_ALL_VOLUMES, mixed, b, extent, cs,
                                        chunked ? kChunkGrab : 0);
                  });
  cudaFreeAsync(d_list, s->stream);
  return rc;
}

int xdgcu_set_surface_boundary(xdgcu_ctx* c, int32_t n, const int32_t* surface_ids,
                               const int32_t* conditions) {
  CHECK_CTX(c);
  if (n < 0 || (n > 0 && (!surface_ids || !conditions)))
    return set_err(XDGCU_ERR_INVALID_ARG, "bad boundary condition arguments");
  std::lock_guard<std::mutex> g(c->mu);
  for (int32_t k = 0; k < n; ++k) {
    if (conditions[k] < XDGCU_BC_TRANSMISSION || conditions[k] > XDGCU_BC_REFLECTING)
      return set_err(XDGCU_ERR_INVALID_ARG, "unknown boundary condition");
    auto it = c->surf_index.find(surface_ids[k]);
    if (it == c->surf_index.end())
      return set_err(XDGCU_ERR_NOT_FOUND, "boundary condition for an unregistered surface");
  }
  for (int32_t k = 0; k < n; ++k) c->surfs[c->surf_index[surface_ids[k]]].bc = conditions[k];
  c->surf_dirty = true;
  return sync_surfaces(c);
}

int xdgcu_transport_surfaces(xdgcu_ctx* c, int64_t n, int32_t* tree, double* position,
                             double* direction, uint64_t* rng_state, double mean_free_path,
                             int32_t max_events, int32_t graveyard_tree, int32_t history_cap,
                             int32_t* history, int32_t* history_count, double* distance,
                             int32_t* events, double* tree_tally, int32_t* status,
                             int32_t precision, void* stream) {
  CHECK_CTX(c);
  if (n < 0) return set_err(XDGCU_ERR_INVALID_ARG, "negative particle count");
  if (precision != XDGCU_FP64 && precision != XDGCU_MIXED)
    return set_err(XDGCU_ERR_INVALID_ARG, "precision must be XDGCU_FP64 or XDGCU_MIXED");
  if (!(mean_free_path > 0.0) || !(mean_free_path < 1e300))
    return set_err(XDGCU_ERR_INVALID_ARG, "mean_free_path must be positive and finite");
  if (max_events < 0) return set_err(XDGCU_ERR_INVALID_ARG, "max_events must be >= 0");
  if (history_cap < 1 || history_cap > 4096)
    return set_err(XDGCU_ERR_INVALID_ARG, "history_cap must be 1..4096");
  if (n == 0) return XDGCU_OK;
  if (!tree || !position || !direction || !rng_state || !history || !history_count ||
      !distance || !events)
    return set_err(XDGCU_ERR_INVALID_ARG, "null particle state");
  {
    std::lock_guard<std::mutex> g(c->mu);
    int rc = sync_surfaces(c);
    if (rc) return rc;
    rc = sync_tree_tables(c);
    if (rc) return rc;
  }
  const int kind = classify({tree, position, direction, rng_state, history, history_count,
                             distance, events, tree_tally, status});
  if (kind < 0) return set_err(XDGCU_ERR_INVALID_ARG, "host and device pointers mixed in one call");
  SurfArgs a{};
  a.trees = c->d_surf_trees.p;
  a.n_trees = (int32_t)c->surf_trees.size();
  a.n = n;
  a.orientation = XDGCU_EXITING;
  a.tri_face = c->d_tri_face.p;
  a.tri_surf = c->d_tri_surf.p;
  a.surf_id = c->d_surf_id.p;
  a.surf_rev_tree = c->d_surf_rev.p;
  a.surf_fwd_tree = c->d_surf_fwd.p;
  a.surf_bc = c->d_surf_bc.p;
  a.tri_xyz = c->d_tri_xyz.p;
  a.occupancy = c->trace_occupancy;
  a.prim_edges = c->trace_edge_table;
  a.tri_prime = c->d_tri_prime.p;
  a.node_iters = precision == XDGCU_MIXED ? c->trace_node_iters : c->trace_node_iters_fp64;
  a.flush_wait = c->trace_flush_wait;
  a.stack = trace_stack_for(c);
  a.mfp = mean_free_path;
  a.max_events = max_events;
  a.graveyard_tree = graveyard_tree;
  a.hist_cap = history_cap;
  a.event_wait = c->particle_event_wait;
  const bool mixed = precision == XDGCU_MIXED;
  cudaStream_t st = (cudaStream_t)stream;
  auto bind = [&](char* const* p) {
    a.p_tree = (int32_t*)p[0];
    a.p_pos = (double*)p[1];
    a.p_dir = (double*)p[2];
    a.p_rng = (unsigned long long*)p[3];
    a.p_hist = (int32_t*)p[4];
    a.p_hcount = (int32_t*)p[5];
    a.p_dist = (double*)p[6];
    a.p_events = (int32_t*)p[7];
    a.p_tally = (double*)p[8];
    a.status = (int32_t*)p[9];
  };
  if (kind == 1) {
    char* p[10] = {(char*)tree, (char*)position, (char*)direction, (char*)rng_state,
                   (char*)history, (char*)history_count, (char*)distance, (char*)events,
                   (char*)tree_tally, (char*)status};
    bind(p);
    int rc = begin_query(c, st, &a.counters);
    if (rc) return rc;
    // particle histories differ in length by orders of magnitude: warps
    // always take particles from the work queue, 32 at a time at least
    API_CUDA(launch_trace(c, MODE_PARTICLE, mixed, a, 0.0, st, 32), "particle launch");
    return XDGCU_OK;
  }
  Slot* s = get_slot(c);
  if (!s) return set_err(XDGCU_ERR_CUDA, "staging stream creation failed");
  if (!st) st = s->stream;
  const size_t un = (size_t)n;
  Arr A[10] = {{tree, tree, 4 * un},
               {position, position, 24 * un},
               {direction, direction, 24 * un},
               {rng_state, rng_state, 8 * un},
               {history, history, 4 * un * (size_t)history_cap},
               {history_count, history_count, 4 * un},
               {distance, distance, 8 * un},
               {events, events, 4 * un},
               {tree_tally, tree_tally, tree_tally ? 8 * (c->surf_trees.size() + 1) : 0},
               {nullptr, status, status ? 4 * un : 0}};
  A[8].no_direct = true;  // atomic tallies stay in device memory
  std::vector<Arr*> all;
  for (auto& x : A) all.push_back(&x);
  int rc = stage_in(c, s, all, st);
  if (rc) return rc;
  char* p[10];
  for (int k = 0; k < 10; ++k) p[k] = (char*)A[k].dev;
  bind(p);
  rc = begin_query(c, st, &a.counters);
  if (rc) return rc;
  API_CUDA(launch_trace(c, MODE_PARTICLE, mixed, a, 0.0, st, 32), "particle launch");
  return stage_out(all, st);
}

int xdgcu_seed_streams(uint64_t seed, int64_t n, uint64_t* states) {
  if (n < 0 || (n > 0 && !states)) return set_err(XDGCU_ERR_INVALID_ARG, "bad seed arguments");
  for (int64_t i = 0; i < n; ++i) {
    // SplitMix64's output function applied to seed + (i + 1) * golden gamma
    uint64_t z = seed + (uint64_t)(i + 1) * 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    states[i] = z ^ (z >> 31);
  }
  return XDGCU_OK;
}

int xdgcu_transport_elements(xdgcu_ctx* c, int64_t n, int32_t* elem_index, double* position,
                             double* direction, uint64_t* rng_state, double mean_free_path,
                             int32_t max_events, double* distance, int32_t* events,
                             double* elem_tally, int32_t* status, int32_t precision,
                             void* stream) {
  CHECK_CTX(c);
  if (n < 0) return set_err(XDGCU_ERR_INVALID_ARG, "negative particle count");
  if (precision != XDGCU_FP64 && precision != XDGCU_MIXED)
    return set_err(XDGCU_ERR_INVALID_ARG, "precision must be XDGCU_FP64 or XDGCU_MIXED");
  if (!c->has_tets) return set_err(XDGCU_ERR_STATE, "no tet mesh set");
  if (!(mean_free_path > 0.0) || !(mean_free_path < 1e300))
    return set_err(XDGCU_ERR_INVALID_ARG, "mean_free_path must be positive and finite");
  if (max_events < 0) return set_err(XDGCU_ERR_INVALID_ARG, "max_events must be >= 0");
  if (n == 0) return XDGCU_OK;
  if (!elem_index || !position || !direction || !rng_state || !distance || !events)
    return set_err(XDGCU_ERR_INVALID_ARG, "null particle state");
  const int kind = classify({elem_index, position, direction, rng_state, distance, events,
                             elem_tally, status});
  if (kind < 0) return set_err(XDGCU_ERR_INVALID_ARG, "host and device pointers mixed in one call");
  TransportArgs t{};
  WalkArgs& a = t.mesh;
  a.xyz = c->d_xyz.p;
  a.xyz32 = c->d_xyz32.p;
  a.edge = c->walk_edge_table ? c->d_edge.p : nullptr;
  a.tet_edge = c->d_tet_edge.p;
  a.conn = c->d_conn.p;
  a.adj = c->d_adj.p;
  a.elem_ids = c->d_elem_ids.p;
  a.n_tets = (int32_t)c->n_tet;
  std::memcpy(a.face, c->face, sizeof(a.face));
  t.n = n;
  t.mfp = mean_free_path;
  t.max_events = max_events;
  // FP64 steps are FP64-bound themselves: idle waiting lanes cost more than
  // the batching saves, so the all-FP64 loop runs each event at once
  t.event_wait = precision == XDGCU_MIXED ? c->transport_event_wait : 1;
  const bool mixed = precision == XDGCU_MIXED;
  cudaStream_t st = (cudaStream_t)stream;
  if (kind == 1) {
    t.elem = elem_index;
    t.pos = position;
    t.dir = direction;
    t.rng = (unsigned long long*)rng_state;
    t.distance = distance;
    t.events = events;
    t.tally = elem_tally;
    t.status = status;
    int rc = begin_query(c, st, &t.counters);
    if (rc) return rc;
    API_CUDA(launch_transport(mixed, c->face_order, t, st), "transport launch");
    return XDGCU_OK;
  }
  Slot* s = get_slot(c);
  if (!s) return set_err(XDGCU_ERR_CUDA, "staging stream creation failed");
  if (!st) st = s->stream;
  // the particle state is read and written back: copied in and out
  Arr A_e{elem_index, elem_index, sizeof(int32_t) * n};
  Arr A_p{position, position, sizeof(double) * 3 * n}, A_d{direction, direction, sizeof(double) * 3 * n};
  Arr A_r{rng_state, rng_state, sizeof(uint64_t) * n};
  Arr A_l{distance, distance, sizeof(double) * n};
  Arr A_v{events, events, sizeof(int32_t) * n};
  Arr A_t{elem_tally, elem_tally, elem_tally ? sizeof(double) * c->n_tet : 0};
  A_t.no_direct = true;  // atomic tallies stay in device memory
  Arr A_st{nullptr, status, status ? sizeof(int32_t) * n : 0};
  std::vector<Arr*> all = {&A_e, &A_p, &A_d, &A_r, &A_l, &A_v, &A_t, &A_st};
  int rc = stage_in(c, s, all, st);
  if (rc) return rc;
  t.elem = (int32_t*)A_e.dev;
  t.pos = (double*)A_p.dev;
  t.dir = (double*)A_d.dev;
  t.rng = (unsigned long long*)A_r.dev;
  t.distance = (double*)A_l.dev;
  t.events = (int32_t*)A_v.dev;
  t.tally = (double*)A_t.dev;
  t.status = (int32_t*)A_st.dev;
  rc = begin_query(c, st, &t.counters);
  if (rc) return rc;
  API_CUDA(launch_transport(mixed, c->face_order, t, st), "transport launch");
  return stage_out(all, st);
}

}  // extern "C"
