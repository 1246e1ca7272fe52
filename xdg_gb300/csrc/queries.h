// queries.h -- launch interface of the tree-query kernels.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "internal.cuh"

namespace xdgcu {

enum QueryMode : int {
  MODE_RAY_FIRE = 0,
  MODE_PIV = 1,
  MODE_OCCLUDED = 2,
  MODE_FIND_VOLUME = 3,
  MODE_PARTICLE = 4,    // the particle_sim loop: every ray is one flight of a particle
  MODE_ALL_VOLUMES = 5  // point_in_volume of each point in every volume of a list
};

// boundary conditions of the particle loop (MeshManager surface property)
enum : int32_t { BC_TRANSMISSION = 0, BC_VACUUM = 1, BC_REFLECTING = 2 };

struct SurfArgs {
  const TreeDev* trees;  // indexed by tree id - 1
  int32_t n_trees;
  int32_t tree;
  const int32_t* ray_trees;
  int64_t n;
  const double* org;
  const double* dir;
  const double* tmax;
  int32_t orientation;
  const int32_t* excl_off;
  const int32_t* excl_ids;
  // geometry tables (global triangle / surface index)
  const int32_t* tri_face;
  const int32_t* tri_surf;
  const int32_t* surf_id;
  const int32_t* surf_rev_tree;
  // outputs (any may be null where the mode does not write them)
  double* t_out;
  int32_t* surf_out;
  int32_t* face_out;
  int32_t* flag_out;   // PIV inside / occluded flag
  double* dist_out;    // occluded distance
  int32_t* status;
  unsigned long long* counters;
  int32_t occupancy;   // traversal kernel variant: minimum resident blocks per SM (2..4)
  int32_t node_iters;  // inner-node steps per lane between leaf phases (1..64)
  int32_t flush_wait;  // lanes waiting on the FP64 queue that force a partial drain (1..32)
  int32_t stack;       // shared-memory traversal stack entries per lane (16..64, multiple of 8)
  int32_t grab;        // > 0: warps take rays from the device work queue `work`, `grab` at a time
  unsigned long long* work;  // work-queue cursor (zero at launch), used when grab > 0
  const int32_t* order;      // optional ray order (a permutation of 0..n-1), or null
  // MODE_FIND_VOLUME: the volumes tried in order (their surface trees) and
  // the id written when none contains the point; the id goes to flag_out
  const int32_t* vol_ids;
  const int32_t* vol_trees;
  int32_t n_vols;
  int32_t ipc_volume;
  // MODE_ALL_VOLUMES: inside flags, point i's flag for list entry k at
  // vol_inside[i * vol_stride + k] (the list is vol_trees[0 .. n_vols))
  uint8_t* vol_inside;
  int64_t vol_stride;
  // MODE_PARTICLE: per-particle state, read at the start and written back
  // when the particle stops
  double* p_pos;
  double* p_dir;
  int32_t* p_tree;              // surface tree of the particle's volume (-1: ended outside)
  unsigned long long* p_rng;    // SplitMix64 state
  double* p_dist;               // path length so far
  int32_t* p_events;
  int32_t* p_hist;              // exclusion history: hist_cap entries per particle, a ring
  int32_t* p_hcount;            // faces appended since the history was last cleared
  int32_t hist_cap;
  double* p_tally;              // track length per tree id (atomics), or null
  double mfp;
  int32_t max_events;
  int32_t graveyard_tree;       // > 0: a particle that would enter this tree ends
  int32_t event_wait;           // lanes whose flights ended before the warp runs their events
  int32_t prim_edges;           // mixed FP64 tests read tri_prime (1) or the vertices (0)
  const double* tri_prime;      // kTriPrimeStride doubles per global triangle
  const int32_t* surf_fwd_tree;
  const int32_t* surf_bc;
  const double* tri_xyz;        // 9 doubles per global triangle, mesh vertex order
};

struct PointArgs {
  const TreeDev* trees;
  int32_t n_trees;
  int32_t tree;
  const int32_t* ray_trees;
  int64_t n;
  const double* pts;
  const int32_t* tri_face;   // closest: face ids
  // closest, mixed: per global triangle 4 float4 -- unit normal n and n.v0,
  // then for the edges (v0,v1), (v1,v2), (v2,v0) the outward in-plane unit
  // normal m and m.(edge start) -- for a certified FP32 lower bound of the
  // distance (w = NaN for degenerate triangles: never pruned)
  const float4* tri_cb;
  const int32_t* elem_ids;   // find_element: element mesh ids
  int32_t node_steps;        // closest: inner-node steps per lane between leaf phases (1..64)
  // closest, optional: a lane stops a point's search after step_budget node
  // records and triangles (0: no budget), sets deferred[i] and leaves its
  // best so far in def_best / def_face; a warp then finishes each such point
  // (launch_closest).  deferred, def_best and def_face hold n entries.
  int32_t step_budget;
  int8_t* deferred;
  double* def_best;
  int32_t* def_face;
  // optional: position k of the launch takes point order[k] (a permutation
  // of 0..n-1; closest and find_element); results go to the point's own index
  const int32_t* order;
  double* dist_out;
  int32_t* id_out;
  int32_t* index_out;
  int32_t* status;
  unsigned long long* counters;
};

cudaError_t launch_surface_query(int mode, bool mixed, const SurfArgs& a, cudaStream_t st);

// Coherent ray order (order.cu): order = the ray indices sorted by
// [tree | direction octant | Morton code of the origin in [-extent, extent]^3].
// scratch holds ray_order_scratch_bytes(n) bytes; n < 2^31.
size_t ray_order_scratch_bytes(int64_t n);
cudaError_t ray_order(const double* org, const double* dir, const int32_t* ray_trees,
                      int32_t n_trees, int64_t n, double extent, int32_t* order, void* scratch,
                      size_t scratch_bytes, cudaStream_t st);
cudaError_t launch_closest(bool mixed, const PointArgs& a, cudaStream_t st);
// The mixed find_element runs one lane per point on its own unless `phased`
// (warp-synchronous phases, as the all-FP64 path always runs): the faster
// for points on or near tet faces, where the FP32 filter leaves most tets to
// the exact test.
cudaError_t launch_find_element(bool mixed, const PointArgs& a, cudaStream_t st,
                                bool phased = false);

}  // namespace xdgcu
