// walk.h -- launch interface of the tet-walk kernels.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace xdgcu {

struct WalkArgs {
  const double* xyz;     // 3 doubles per vertex
  const float4* xyz32;   // fl32 vertex, w = |v|_inf
  const int4* conn;      // 4 vertex indices per tet
  const int4* adj;       // 4 neighbour tets per tet (-1 boundary), face order
  const int32_t* elem_ids;
  // edge table of the mesh (may be null): 6 doubles per unique edge (e = hi -
  // lo, then e x lo, lo/hi in first() order) and 6 entries per tet for its
  // local vertex pairs (0,1),(0,2),(0,3),(1,2),(1,3),(2,3): the edge index,
  // bit 31 set when the pair's second vertex is the edge's lo
  const double* edge;
  const int32_t* tet_edge;
  int32_t n_tets;
  int32_t face[12];      // local face table
  int64_t n;
  const int32_t* start;  // tet index per track
  const double* org;
  const double* dir;
  const double* dist;    // walk: track lengths
  int32_t max_segs;
  int32_t* seg_elem;
  double* seg_len;
  int32_t* seg_count;
  int32_t* status;
  int32_t* next_out;     // next_element mode
  double* dist_out;
  // walk modes, optional: the tet index a track stopped in (-1 when it left
  // the mesh); for a track stopped by max_segs, where its walk goes on
  int32_t* stop_elem;
  // walk modes, optional (the global track loop): the running sum of a
  // track's segment lengths, added in segment order from sum_in[i] (0 when
  // null) and written to sum_out[i]; and the position (3 doubles at end_r)
  // and distance left (end_dist) where the walk stopped, as its own steps
  // computed them (r += len * u, distance -= len)
  const double* sum_in;
  double* sum_out;
  double* end_r;
  double* end_dist;
  unsigned long long* counters;
  // output layout: 0 = track-major with stride max_segs; 1 = count only
  // (offsets[i] = number of segments of track i); 2 = packed, track i's
  // segments at offsets[i] .. offsets[i+1]-1 of arrays of `capacity` entries
  int32_t out_mode;
  int64_t* offsets;
  int64_t capacity;
  // mixed walk: 1 = per-warp FP64 queue (k_walk_q), 0 = per-lane escalation
  int32_t walk_queue;
  // optional: track indices by decreasing length; the kernels then deal them
  // round-robin to warps, longest first, so warps finish on short tracks
  const int32_t* order;
  int32_t flush_wait;  // queue: lanes waiting that force a partial FP64 round
};

enum : int32_t { WALK_STRIDED = 0, WALK_COUNT = 1, WALK_PACKED = 2 };

// Device particle loop over the tet mesh (tools/walk_elements.h:53-96): the
// per-particle state is read and written back in place.
struct TransportArgs {
  WalkArgs mesh;             // mesh arrays and face table (n, start, ... unused)
  int64_t n;
  int32_t* elem;             // tet index; -1 = outside the mesh
  double* pos;               // 3 per particle
  double* dir;               // 3 per particle (unit)
  unsigned long long* rng;   // SplitMix64 state per particle
  double* distance;          // accumulated path length
  int32_t* events;           // accumulated events
  int32_t* status;           // per particle (may be null)
  double* tally;             // per-tet track length, accumulated with atomics (may be null)
  double mfp;
  int32_t max_events;
  int32_t event_wait;        // lanes gathered before their FP64 event work runs
  unsigned long long* counters;
};

cudaError_t launch_transport(bool mixed, int face_order, const TransportArgs& a, cudaStream_t st);

// In-place exclusive scan of offsets[0..n) with offsets[n] = total.
// block_sums needs scan_scratch_entries(n) int64 entries.
int64_t scan_scratch_entries(int64_t n);
cudaError_t scan_offsets(int64_t* offsets, int64_t n, int64_t* block_sums, cudaStream_t st);

// Length order of n tracks (n < 2^31): order[k] = index of the k-th longest.
// scratch holds walk_order_scratch_bytes(n) bytes.
size_t walk_order_scratch_bytes(int64_t n);
cudaError_t walk_order(const double* dist, int64_t n, int32_t* order, void* scratch,
                       size_t scratch_bytes, cudaStream_t st);

// Builds the edge table of a tet mesh (WalkArgs::edge / tet_edge) on the
// device: sorts the 6 vertex pairs of every tet, numbers the unique ones and
// evaluates each edge's e and e x lo once, with plucker.h:45-62's operations.
// *edge and *tet_edge are cudaMalloc'ed (the caller frees them).  Returns
// cudaErrorInvalidValue without building anything when 6 * n_tets >= 2^31.
cudaError_t build_edge_table(const double* xyz, const int4* conn, int64_t n_tets, double** edge,
                             int32_t** tet_edge, int64_t* n_edges, cudaStream_t st);

// face_order: 0 = the MOAB table {0,1,3},{1,2,3},{2,0,3},{0,2,1} (compiled in),
// 1 = any other table (read from WalkArgs::face).
cudaError_t launch_walk(bool mixed, int face_order, const WalkArgs& a, cudaStream_t st);
cudaError_t launch_next_element(bool mixed, int face_order, const WalkArgs& a, cudaStream_t st);

}  // namespace xdgcu
