// cuda_tools.h -- the particle loops and the overlap check of XDG's tools
// (tools/walk_elements.h, tools/particle_sim.h, tools/overlap.cpp) as C++
// host code over the GB300 engine's C ABI (include/xdgcu.h): every event of
// every particle, and every query of an overlap-check stage, runs in batched
// device launches; the host only does what the tools do between them
// (re-entry through the implicit complement, set bookkeeping).
#pragma once

#include <cstdint>
#include <map>
#include <set>
#include <vector>

#include "cuda_ray_tracer.h"

namespace xdg {

// Per-particle state of the tool loops, one entry per particle, read and
// written back by the loops.
struct ParticleBank {
  // walk_particles: the element (mesh id) the particle is in, ID_NONE once
  // it has left the mesh for good; simulate_particles: its volume, ID_NONE
  // once it entered the graveyard or no volume
  std::vector<MeshID> cell;
  std::vector<double> pos;       // 3 per particle
  std::vector<double> dir;       // 3 per particle (unit)
  std::vector<uint64_t> rng;     // random stream state (seed_streams)
  std::vector<double> distance;  // path length so far
  std::vector<int32_t> events;
  std::vector<int32_t> status;   // XDGCU_RAY_* of the last launch
  size_t size() const { return cell.size(); }
  void resize(size_t n);
};

// n independent random-stream states (xdgcu_seed_streams).
std::vector<uint64_t> seed_streams(uint64_t seed, size_t n);

// The walk_elements tool loop (tools/walk_elements.h:60-96) for particles in
// the element trees' mesh: in-mesh events on the device
// (xdgcu_transport_elements); a particle that leaves the mesh fires a ray in
// the implicit complement's surface tree (EXITING, the faces this search hit
// excluded), moves to the hit and looks for the element at r + u * TINY_BIT
// in the global element tree, as the tool does, and continues if it finds
// one.  element_tally (may be null): path length per engine tet index
// (CudaRayTracer::tet_id maps an index to its element).
void walk_particles(CudaRayTracer& rt, TreeID ipc_surface_tree, ParticleBank& bank, double mfp,
                    int32_t max_events = 1000000, std::vector<double>* element_tally = nullptr,
                    int max_reentries = 64);

// The particle_sim tool loop (tools/particle_sim.h:128-141): surface
// tracking through the volumes' surface trees with the surfaces' boundary
// conditions (MeshManager::get_surface_property), every event on the device
// (xdgcu_transport_surfaces).  volume_trees maps each volume to its surface
// tree; ipc_graveyard ends particles entering the implicit complement (the
// tool's --ipc-graveyard).  cell_tracks (may be null): path length per volume.
void simulate_particles(CudaRayTracer& rt, const MeshManager& mm,
                        const std::map<MeshID, TreeID>& volume_trees, bool ipc_graveyard,
                        ParticleBank& bank, double mfp, int32_t max_events = 1000000,
                        std::map<MeshID, double>* cell_tracks = nullptr,
                        int32_t history_cap = 16);

// Segments of n tracks: track i's are element[offsets[i] .. offsets[i+1]-1]
// with the same lengths; offsets has n + 1 entries.
struct TrackSegments {
  std::vector<MeshID> element;
  std::vector<double> length;
  std::vector<int64_t> offsets;
};

// XDG::segments(start, end) (xdg.cpp:142-198) for the n tracks
// starts[i] -> ends[i] (3 doubles each) across the meshed volumes and the
// implicit complement between them, on the device (xdgcu_segments_global):
// each round locates the active tracks in the global element tree, fires the
// implicit-complement rays of the tracks outside the mesh (EXITING) and
// re-enters through the element behind the hit face
// (MeshManager::get_boundary_face_element, handed to the engine with
// xdgcu_set_boundary_face_elements), then walks the rest in one packed launch.
TrackSegments track_segments(CudaRayTracer& rt, const MeshManager& mm, TreeID ipc_surface_tree,
                             size_t n, const double* starts, const double* ends,
                             int max_rounds = 10000);

// The overlap_check tool (tools/overlap.cpp:62-191): every face vertex moved
// 1e-9 along +/- normalize(0.1, 0.1, 0.1) and tested in every volume
// (xdgcu_point_in_volumes); with check_edges a ray along every face edge in
// every volume that is not a parent of the edge's surface.  Returns each set
// of overlapping volumes with the first location (vertex order, then edge
// order) that found it.
std::map<std::set<MeshID>, Position> check_overlaps(CudaRayTracer& rt, const MeshManager& mm,
                                                    const std::map<MeshID, TreeID>& volume_trees,
                                                    bool check_edges,
                                                    int64_t max_batch = 4000000);

}  // namespace xdg
