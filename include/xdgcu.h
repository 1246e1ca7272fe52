/*
 * xdgcu.h -- C ABI of the GB300 (sm_103a) ray-query engine for XDG.
 *
 * This is the boundary a CUDA backend of XDG's RayTracer plugin API binds
 * (include/xdg/ray_tracing_interface.h:16-147 in the reference).  Each entry
 * point below names the reference interface it replaces.  Plain C types
 * only: pointers, sizes, int32 ids.  No exceptions cross it; every function
 * returns an xdgcu_status and xdgcu_last_error() describes the last failure.
 *
 * Conventions (reference semantics):
 *   - ids are int32 (constants.h:73-87); ID_NONE = TREE_NONE = -1;
 *   - surface and element tree ids are separate counters starting at 1
 *     (ray_tracing_interface.cpp:10-18);
 *   - a miss is {t = INFTY (DBL_MAX), surface = ID_NONE} (embree/ray_tracer.cpp:320-321);
 *   - positions/directions are n x 3 doubles (AoS), as Position/Direction;
 *   - coordinates must be finite with magnitude below 2^300 (so no product of
 *     three of them overflows); rays outside that range get XDGCU_RAY_INVALID.
 *
 * Batched queries take `n` rays and either one tree (`tree` > 0,
 * `ray_trees` = NULL) or one tree per ray (`ray_trees` != NULL, `tree`
 * ignored).  Input and output pointers may be device memory (the fast path:
 * the work is enqueued on `stream` and the call returns without
 * synchronising) or host memory (the call returns when the results are in
 * the caller's arrays).  The two kinds may not be mixed within one call.
 * Host arrays are read and written in place by the kernels where the device
 * can address them (page-locked memory, and pageable memory on systems whose
 * GPU walks the host page tables, such as Grace), except that by default
 * (`host_direct` = 5) a large call's page-locked arrays are staged when
 * timing the first large calls found staging faster.  Memory the device
 * cannot address, or any host array under `host_direct` = 0, is staged
 * through a per-thread device workspace in overlapping chunks.
 *
 * Precision: XDGCU_FP64 evaluates everything in double precision (the plain
 * drop-in); XDGCU_MIXED runs FP32 box tests, an FP32 Plucker pre-filter (the
 * walk: an FP32 face pre-filter; find_element: an FP32 containment
 * pre-filter; closest: FP32 lower bounds of box and triangle distances) with
 * a proven error bound, escalating to the FP64 test wherever the FP32 answer
 * is not certain.  Both return bit-identical ids and distances.
 *
 * Devices: a context belongs to the device it was created on.  Every entry
 * point makes that device current while it runs and makes the caller's
 * current device current again before it returns.
 *
 * Tie rule: when two accepted candidates are at exactly the same distance,
 * the lowest mesh id wins (face id for ray_fire / point_in_volume / closest,
 * element id for find_element).  The reference leaves this to Embree's
 * traversal order.
 */
#ifndef XDGCU_H
#define XDGCU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct xdgcu_ctx xdgcu_ctx;

typedef enum {
  XDGCU_OK = 0,
  XDGCU_ERR_INVALID_ARG = 1,
  XDGCU_ERR_CUDA = 2,
  XDGCU_ERR_NOT_FOUND = 3,
  XDGCU_ERR_OUT_OF_MEMORY = 4,
  XDGCU_ERR_STATE = 5
} xdgcu_status;

/* per-ray status codes written to the optional `status` arrays */
enum {
  XDGCU_RAY_OK = 0,
  XDGCU_RAY_INVALID = 1,        /* NaN/inf origin or direction, or bad tree id */
  XDGCU_RAY_STACK_OVERFLOW = 2, /* traversal stack exhausted (result incomplete) */
  XDGCU_RAY_WALK_LIMIT = 4,     /* walk stopped at max_segs (output truncated) */
  XDGCU_RAY_NO_EXIT_FACE = 5,   /* next_element found no exiting face */
  XDGCU_RAY_OUTPUT_FULL = 6,    /* packed walk output capacity exceeded */
  XDGCU_RAY_EVENT_LIMIT = 7,    /* particle stopped at max_events */
  XDGCU_RAY_LOST = 8,           /* particle found no surface ahead (particle_sim's "lost") */
  XDGCU_RAY_STUCK = 9           /* particle's next surface hit at distance 0 ("stuck") */
};

/* shared_enums.h:11-15 */
enum { XDGCU_ANY = -1, XDGCU_EXITING = 0, XDGCU_ENTERING = 1 };

enum { XDGCU_FP64 = 0, XDGCU_MIXED = 1 };

/* ------------------------------------------------------------------------
 * Context
 * ------------------------------------------------------------------------ */

/* Replaces the backend constructor (embree/ray_tracer.cpp:15-19).  Binds the
 * context to CUDA device `device`. */
int xdgcu_create(xdgcu_ctx** ctx, int device);

/* Replaces the backend destructor (embree/ray_tracer.cpp:21-24). */
int xdgcu_destroy(xdgcu_ctx* ctx);

/* Human-readable description of the last failed call on this context (never
 * NULL; "" when none).  The pointer stays valid until the next call. */
const char* xdgcu_last_error(const xdgcu_ctx* ctx);

/* Library version (major*10000 + minor*100 + patch). */
int xdgcu_version(void);

/* ------------------------------------------------------------------------
 * Geometry registration and tree builds
 * ------------------------------------------------------------------------ */

/* Uploads one surface's triangles: tri_xyz holds 9 doubles per face (the
 * face's three vertices in mesh order, as MeshManager::face_vertices returns
 * them), face_ids the mesh face ids.  Replaces the first-visit branch of
 * EmbreeRayTracer::register_surface (embree/ray_tracer.cpp:107-147).  A
 * surface may be registered once. */
int xdgcu_register_surface(xdgcu_ctx* ctx, int32_t surface_id, int64_t n_faces,
                           const double* tri_xyz, const int32_t* face_ids);

/* Builds a surface tree over the given registered surfaces and returns its
 * tree id.  sense[i] = 0 when the tree's volume is surface i's forward
 * volume, 1 when it is the reverse volume (normals are flipped for that tree,
 * triangle_intersect.cpp:84-87).  bump is the box dilation
 * (ray_tracing_interface.cpp:20-24); the tree's boxes use, per surface, the
 * largest bump of any tree the surface belongs to, as
 * embree/ray_tracer.cpp:76-89 does.  Replaces
 * RayTracer::create_surface_tree (embree/ray_tracer.cpp:49-105). */
int xdgcu_create_surface_tree(xdgcu_ctx* ctx, const int32_t* surface_ids, const int32_t* sense,
                              int32_t n_surfaces, double bump, int32_t* tree_out);

/* Builds the global surface tree over every registered surface (no normal
 * flips).  Replaces create_global_surface_tree (embree/ray_tracer.cpp:190-206). */
int xdgcu_create_global_surface_tree(xdgcu_ctx* ctx, int32_t* tree_out);

/* Uploads the tet mesh used by find_element and the element walk: vertex
 * coordinates (3 per vertex), connectivity (4 vertex indices per tet),
 * adjacency (4 neighbour tet indices per tet, -1 on the boundary, in face
 * order), the per-element mesh ids, and the 4x3 local face table of the mesh
 * library's ElementFaceAccessor (e.g. MOAB's {0,1,3},{1,2,3},{2,0,3},{0,2,1},
 * moab/direct_access.h:181-183).  Replaces what MeshManager::next_element
 * reads through ElementFaceAccessor / adjacent_element
 * (mesh_manager_interface.cpp:149-200).  May be called once. */
int xdgcu_set_tet_mesh(xdgcu_ctx* ctx, int64_t n_vertices, const double* xyz, int64_t n_tets,
                       const int32_t* conn, const int32_t* adj, const int32_t* elem_ids,
                       const int32_t face_table[12]);

/* Builds an element tree over the given tet indices (of the mesh above) and
 * returns its tree id.  Replaces RayTracer::create_element_tree
 * (embree/ray_tracer.cpp:149-188). */
int xdgcu_create_element_tree(xdgcu_ctx* ctx, const int32_t* tet_indices, int64_t n,
                              int32_t* tree_out);

/* Builds the global element tree over all tets in every element tree.
 * Replaces create_global_element_tree (embree/ray_tracer.cpp:208-224). */
int xdgcu_create_global_element_tree(xdgcu_ctx* ctx, int32_t* tree_out);

/* Number of surface / element trees built so far (num_registered_*_trees,
 * ray_tracing_interface.h:121-123). */
int xdgcu_num_surface_trees(const xdgcu_ctx* ctx);
int xdgcu_num_element_trees(const xdgcu_ctx* ctx);

/* ------------------------------------------------------------------------
 * Batched queries
 * ------------------------------------------------------------------------ */

/* RayTracer::ray_fire (ray_tracing_interface.h:81-86; embree/ray_tracer.cpp:
 * 289-326; triangle_intersect.cpp:52-109).  dist_limit: n doubles or NULL
 * (INFTY).  Exclusions in CSR form: excl_offsets (n+1) and excl_ids, or both
 * NULL.  Outputs: t_out (INFTY on a miss), surface_out (ID_NONE on a miss),
 * face_out (the hit face id the reference appends to its exclude list;
 * may be NULL), status (may be NULL). */
int xdgcu_ray_fire(xdgcu_ctx* ctx, int32_t tree, const int32_t* ray_trees, int64_t n,
                   const double* origins, const double* directions, const double* dist_limit,
                   int32_t orientation, const int32_t* excl_offsets, const int32_t* excl_ids,
                   double* t_out, int32_t* surface_out, int32_t* face_out, int32_t* status,
                   int32_t precision, void* stream);

/* RayTracer::point_in_volume (ray_tracing_interface.h:76-79;
 * embree/ray_tracer.cpp:259-287).  directions may be NULL: the reference's
 * default direction (1/sqrt(2), 1/sqrt(2), 0) is used.  inside_out: 1/0. */
int xdgcu_point_in_volume(xdgcu_ctx* ctx, int32_t tree, const int32_t* ray_trees, int64_t n,
                          const double* points, const double* directions,
                          const int32_t* excl_offsets, const int32_t* excl_ids,
                          int32_t* inside_out, int32_t* status, int32_t precision, void* stream);

/* RayTracer::point_in_volume (embree/ray_tracer.cpp:259-287) of each of n
 * points in each of n_trees surface trees (the host array `trees`), in one
 * launch: the lane restarts the point in the next tree.  inside_out[i *
 * n_trees + k] = 1 when point i is inside tree k's volume.  directions may be
 * NULL (the default (1/sqrt(2), 1/sqrt(2), 0)).  This is the inner loop of
 * the overlap_check tool (tools/overlap.cpp:9-60, every volume for every
 * point). */
int xdgcu_point_in_volumes(xdgcu_ctx* ctx, int64_t n, const double* points,
                           const double* directions, int32_t n_trees, const int32_t* trees,
                           uint8_t* inside_out, int32_t* status, int32_t precision,
                           void* stream);

/* Sets the volumes XDG::find_volume tries, in order, with their surface
 * trees (XDG::volume_to_surface_tree_map_, xdg.h:125, filled by
 * prepare_raytracer, xdg.cpp:37-47).  Entries equal to implicit_complement
 * are skipped, as find_volume skips that volume (xdg.cpp:119).  The
 * reference iterates an unordered_map; the order given here is the order
 * tried (for volumes that do not overlap, every order gives the same
 * answer).  Must not be called while queries of this context are running. */
int xdgcu_set_volume_map(xdgcu_ctx* ctx, int32_t n_volumes, const int32_t* volume_ids,
                         const int32_t* surface_trees, int32_t implicit_complement);

/* XDG::find_volume (xdg.cpp:113-128) for n points in one launch: for each
 * point, point_in_volume in the trees of the volume map in order until one
 * holds the point (each lane restarts its traversal in the next tree);
 * volume_out = that volume's id, else the implicit complement.  directions
 * may be NULL (the point_in_volume default direction). */
int xdgcu_find_volume(xdgcu_ctx* ctx, int64_t n, const double* points, const double* directions,
                      int32_t* volume_out, int32_t* status, int32_t precision, void* stream);

/* RayTracer::occluded (ray_tracing_interface.h:112-115; embree/ray_tracer.cpp:
 * 347-370).  occluded_out: 1/0; dist_out (may be NULL): -INFTY when occluded,
 * INFTY otherwise, the value the reference writes through its `dist`. */
int xdgcu_occluded(xdgcu_ctx* ctx, int32_t tree, const int32_t* ray_trees, int64_t n,
                   const double* origins, const double* directions, int32_t* occluded_out,
                   double* dist_out, int32_t* status, int32_t precision, void* stream);

/* RayTracer::closest (ray_tracing_interface.h:109-110; embree/ray_tracer.cpp:
 * 328-345).  Outputs the distance and the nearest face id. */
int xdgcu_closest(xdgcu_ctx* ctx, int32_t tree, const int32_t* ray_trees, int64_t n,
                  const double* points, double* dist_out, int32_t* face_out, int32_t* status,
                  int32_t precision, void* stream);

/* RayTracer::find_element (ray_tracing_interface.h:98-107; embree/ray_tracer.cpp:
 * 226-257).  tree = an element tree id.  Outputs the element mesh id
 * (ID_NONE when no element contains the point) and/or its tet index. */
int xdgcu_find_element(xdgcu_ctx* ctx, int32_t tree, const int32_t* ray_trees, int64_t n,
                       const double* points, int32_t* elem_id_out, int32_t* elem_index_out,
                       int32_t* status, int32_t precision, void* stream);

/* MeshManager::next_element (mesh_manager_interface.cpp:149-200) for n rays:
 * elem_index = tet index; outputs the next tet index (-1 when leaving the
 * mesh) and the exit distance. */
int xdgcu_next_element(xdgcu_ctx* ctx, int64_t n, const int32_t* elem_index,
                       const double* positions, const double* directions, int32_t* next_out,
                       double* dist_out, int32_t* status, int32_t precision, void* stream);

/* MeshManager::walk_elements (mesh_manager_interface.cpp:106-136) for n
 * tracks starting in tet start_index[i] at start[i], direction u[i] (unit),
 * length distance[i].  Output is track-major with stride max_segs:
 * seg_elem[i*max_segs + k] (element MESH ids) and seg_len[...]; seg_count[i]
 * = number of segments (zero-length ones included, as the reference keeps
 * them); status[i] = XDGCU_RAY_WALK_LIMIT when the track needed more than
 * max_segs segments. */
int xdgcu_walk_elements(xdgcu_ctx* ctx, int64_t n, const int32_t* start_index,
                        const double* start, const double* u, const double* distance,
                        int32_t max_segs, int32_t* seg_elem, double* seg_len,
                        int32_t* seg_count, int32_t* status, int32_t precision, void* stream);

/* MeshManager::walk_elements for n tracks with packed, variable-length
 * output -- the form of the reference's per-track
 * std::vector<std::pair<MeshID, double>> (mesh_manager_interface.cpp:106-136).
 * Track i's segments are seg_elem/seg_len[offsets[i] .. offsets[i+1]-1]
 * (element MESH ids, lengths, zero-length segments included); offsets has
 * n+1 entries and offsets[n] is the total.  Arrays hold `capacity` entries:
 * a track whose segments do not fit is not written and gets
 * XDGCU_RAY_OUTPUT_FULL (call again with capacity >= offsets[n]).  max_segs
 * caps the segments of one track (XDGCU_RAY_WALK_LIMIT).  Each track is
 * walked once, in rounds of walks capped at 16..256 segments per track: a
 * walk that reaches the cap pauses and the next round resumes it where it
 * stopped; each round's segments wait in temporary device memory (about the
 * output's size, plus a buffer of up to 1 GiB, allocated on `stream` from
 * the context's scratch pool, "scratch_keep_bytes") until the offsets are
 * known.  Where that memory cannot be
 * had, or with the tuning key "packed_walk_passes" = 2, the tracks are walked
 * twice instead (count, then emit at the scanned offsets), which needs only
 * the scan's scratch.  The results are the same either way. */
int xdgcu_walk_elements_packed(xdgcu_ctx* ctx, int64_t n, const int32_t* start_index,
                               const double* start, const double* u, const double* distance,
                               int32_t max_segs, int64_t capacity, int32_t* seg_elem,
                               double* seg_len, int64_t* offsets, int32_t* status,
                               int32_t precision, void* stream);

/* MeshManager::get_boundary_face_element (mesh_manager_interface.h:153-157)
 * for the global track loop below: face_ids[k] (surface face mesh ids, as
 * ray_fire returns them) -> elem_index[k], the tet index behind the face
 * (-1: none).  Replaces any earlier map.  Host arrays; needs the tet mesh. */
int xdgcu_set_boundary_face_elements(xdgcu_ctx* ctx, int64_t n, const int32_t* face_ids,
                                     const int32_t* elem_index);

/* XDG::segments(start, end) (xdg.cpp:142-198) for n tracks, on the device:
 * u = (end - start) / |end - start|; while distance remains, find_element(r)
 * in `element_tree` (the global element tree in the reference), ignoring the
 * element of the last segment (the track sits on its face); outside the mesh
 * ray_fire(EXITING) in `ipc_tree` (the implicit complement's surface tree)
 * from r + u * TINY_BIT, stop on a miss or a hit beyond the distance, else
 * step to the hit plus TINY_BIT and re-enter through the boundary face's
 * element (xdgcu_set_boundary_face_elements; none: stop); walk_elements;
 * r += u * segment_sum, distance -= segment_sum.  All tracks advance
 * together: each round is one find_element launch for the tracks to locate,
 * one ray_fire launch for those outside the mesh and one walk launch, with
 * the bookkeeping in device kernels.  A round's walk emits at most K
 * segments per track (K = 16..256, chosen so the round buffer stays near
 * 1 GiB); a longer walk pauses and the next round resumes it from where it
 * stopped, with the same operations as one uninterrupted walk.
 * Output as xdgcu_walk_elements_packed: track i's segments (element MESH
 * ids, lengths) at offsets[i] .. offsets[i+1]-1 of arrays of `capacity`
 * entries; a track that does not fit is not written (XDGCU_RAY_OUTPUT_FULL).
 * max_segs caps one walk of a track and max_rounds the rounds (a paused
 * walk's resumption takes a round): a track cut short by either gets
 * XDGCU_RAY_WALK_LIMIT (the reference has no limit).
 * status (may be NULL) also records XDGCU_RAY_NO_EXIT_FACE (the track went
 * on, as the reference's does) and XDGCU_RAY_INVALID (non-finite input).
 * Host or device arrays (not mixed); scratch is allocated on `stream` from
 * the context's scratch pool, and the call waits for a few counters per
 * round. */
int xdgcu_segments_global(xdgcu_ctx* ctx, int32_t ipc_tree, int32_t element_tree, int64_t n,
                          const double* starts, const double* ends, int32_t max_segs,
                          int32_t max_rounds, int64_t capacity, int32_t* seg_elem, double* seg_len,
                          int64_t* offsets, int32_t* status, int32_t precision, void* stream);

/* Fills states[0..n) (host memory) with independent random stream states
 * for the particle loops: SplitMix64's output function of
 * seed + (i + 1) * 0x9E3779B97F4A7C15.  No counterpart in the reference,
 * which draws from one drand48() stream. */
int xdgcu_seed_streams(uint64_t seed, int64_t n, uint64_t* states);

/* The particle loop of the walk_elements tool (tools/walk_elements.h:73-95)
 * on the device, for particles inside the tet mesh: one call runs every
 * event of every particle until it leaves the mesh or reaches max_events.
 * Per event: (next, exit) = next_element(elem, r, u); a collision distance
 * c = -log(1 - U) * mean_free_path; if c < exit the particle moves c and
 * takes a new isotropic direction, else it moves to the exit face and into
 * the next tet; events += 1.  The state is read and written back in place:
 *   elem_index  tet index (-1 = outside the mesh: the particle is skipped);
 *               on return -1 for particles that left the mesh
 *   position, direction (n x 3), distance (path length so far), events;
 *   rng_state   per-particle random stream state (SplitMix64; seed each
 *               particle differently, e.g. with xdgcu_seed_streams).
 * Random numbers come from each particle's own stream, not from the tool's
 * shared drand48(), and directions are sampled by Marsaglia's method instead
 * of rand_dir's acos/sin/cos (the same isotropic distribution), so every
 * particle's history is reproducible.  elem_tally (may be NULL): n_tets
 * doubles, each event adds its length to the tet it was made in (atomic
 * additions, summation order not fixed).  status: XDGCU_RAY_OK (left the
 * mesh, or was outside it), XDGCU_RAY_EVENT_LIMIT, XDGCU_RAY_INVALID.
 * Re-entry after leaving the mesh (the tool's ray_fire in the implicit
 * complement and find_element, :88-94) is the caller's: then call again. */
int xdgcu_transport_elements(xdgcu_ctx* ctx, int64_t n, int32_t* elem_index, double* position,
                             double* direction, uint64_t* rng_state, double mean_free_path,
                             int32_t max_events, double* distance, int32_t* events,
                             double* elem_tally, int32_t* status, int32_t precision,
                             void* stream);

/* Surface boundary conditions of the surface-tracking particle loop
 * (MeshManager::get_surface_property(surface, BOUNDARY_CONDITION),
 * mesh_manager_interface.cpp:98-104: "transmission" unless set). */
enum { XDGCU_BC_TRANSMISSION = 0, XDGCU_BC_VACUUM = 1, XDGCU_BC_REFLECTING = 2 };

/* Sets the boundary condition of n registered surfaces (by surface id). */
int xdgcu_set_surface_boundary(xdgcu_ctx* ctx, int32_t n, const int32_t* surface_ids,
                               const int32_t* conditions);

/* The particle loop of the particle_sim tool (tools/particle_sim.h:128-141)
 * on the device: surface tracking through the volumes' surface trees, every
 * event of every particle in one launch.  Per event: ray_fire in the
 * particle's volume (EXITING, the history of faces crossed since the last
 * collision excluded; the hit face is appended to it); a collision distance
 * c = -log(1 - U) * mean_free_path; if c < hit distance the particle moves c,
 * takes a new isotropic direction and clears its history (collide), else it
 * moves to the surface and crosses it: reflecting -> mirror the direction in
 * the hit face's normal (XDG::surface_normal with the history, xdg.cpp:
 * 272-289) and keep only the last face in the history; vacuum -> the
 * particle ends; transmission -> the other parent volume of the surface
 * (MeshManager::next_volume); entering graveyard_tree (> 0, e.g. the
 * implicit complement's tree, the tool's --ipc-graveyard) or no volume ends
 * the particle.  events += 1 per event.
 * State, read and written back in place (n particles):
 *   tree        surface tree id of the particle's volume; -1 once it ended
 *               (particles with tree -1 are skipped)
 *   position, direction (n x 3), rng_state (as in xdgcu_transport_elements),
 *   history     n x history_cap face ids (the most recent history_cap
 *               crossings are kept: older faces are behind the particle on
 *               the same straight flight and cannot be hit again),
 *   history_count  faces appended since the last clear (start with 0),
 *   distance, events.
 * tree_tally (may be NULL): n_surface_trees + 1 doubles indexed by tree id,
 * the path length per volume (the tool's cell_tracks), atomic additions.
 * status: XDGCU_RAY_OK (ended), XDGCU_RAY_EVENT_LIMIT (stopped alive; call
 * again to continue), XDGCU_RAY_LOST / XDGCU_RAY_STUCK (the tool's fatal
 * errors, :36-45: the particle stops), XDGCU_RAY_INVALID.  The tool reads
 * max_events but never stops on it; here it bounds each call. */
int xdgcu_transport_surfaces(xdgcu_ctx* ctx, int64_t n, int32_t* tree, double* position,
                             double* direction, uint64_t* rng_state, double mean_free_path,
                             int32_t max_events, int32_t graveyard_tree, int32_t history_cap,
                             int32_t* history, int32_t* history_count, double* distance,
                             int32_t* events, double* tree_tally, int32_t* status,
                             int32_t precision, void* stream);

/* Largest batch of xdgcu_walk_elements_packed_noalloc. */
#define XDGCU_NOALLOC_MAX_TRACKS 4194304

/* xdgcu_walk_elements_packed for callers that cannot let the library
 * allocate device memory -- e.g. a transport code or framework whose own
 * allocator owns the device memory (a caching pool that reserves the free
 * memory at start-up, where a foreign cudaMalloc fails or fragments it), or a
 * particle loop that must stay out of the allocator once set up.  This entry
 * point has no counterpart in the reference.  Same arguments and results as
 * xdgcu_walk_elements_packed, with these differences:
 *   - it calls no cudaMalloc/cudaFree/cudaMallocAsync or other allocating
 *     routine: the scan scratch is a static device array of 32 KiB in the
 *     library, which every GPU that loads the library holds until exit;
 *   - n must not exceed XDGCU_NOALLOC_MAX_TRACKS (else XDGCU_ERR_INVALID_ARG);
 *   - all array arguments must be device (or managed) memory;
 *   - all array arguments must be on the context's device;
 *   - it walks every track twice (count, then emit at the scanned offsets:
 *     the allocating walk's resumed rounds keep their segments in scratch
 *     memory), and it never applies the longest-first track order the
 *     allocating walk uses for batches of at least `walk_sort_min` tracks
 *     (that order sorts the tracks into scratch memory), so
 *     `walk_sort_min` has no effect here: the results are the same, and
 *     it runs at about half the allocating walk's rate (2323 against 4664
 *     Msegs/s on 1e6 tracks of a 750,000-tet cube);
 *   - the first call on a device looks up the static array's device address
 *     (cudaGetSymbolAddress); make that first call before any stream capture.
 *     The address stays valid for the device's primary context: after a
 *     cudaDeviceReset the entry point cannot be used on that device again in
 *     the same process;
 *   - all calls share the static array, so calls whose work overlaps on the
 *     GPU (other streams or host threads) race and must be serialised. */
int xdgcu_walk_elements_packed_noalloc(xdgcu_ctx* ctx, int64_t n, const int32_t* start_index,
                                       const double* start, const double* u,
                                       const double* distance, int32_t max_segs,
                                       int64_t capacity, int32_t* seg_elem, double* seg_len,
                                       int64_t* offsets, int32_t* status, int32_t precision,
                                       void* stream);

/* ------------------------------------------------------------------------
 * Diagnostics
 * ------------------------------------------------------------------------ */

/* Per-launch work counters of the last query run with counting enabled:
 * counters[0] = box tests, [1] = node fetches, [2] = primitive tests,
 * [3] = FP64 escalations, [4] = rays, [5] = walk steps.  Counting is enabled
 * with xdgcu_set_counting(ctx, 1) and slows queries down; it exists to
 * compute algorithmic bytes for roofline reports. */
int xdgcu_set_counting(xdgcu_ctx* ctx, int32_t enable);
int xdgcu_get_counters(xdgcu_ctx* ctx, int64_t counters[8]);

/* Launch and build parameters picked by an autotuner (no counterpart in the
 * reference, whose Embree backend has no tunables).  Keys:
 *   "trace_occupancy"  resident blocks per SM the ray-traversal kernel is
 *                      compiled for (2, 3 or 4, default 4; more blocks = fewer
 *                      registers)
 *   "trace_node_iters" inner-node steps a lane takes between two leaf phases
 *                      of the warp-synchronous traversal, mixed precision
 *                      (1..64, default 4; the FP64 path's default is 1).  On
 *                      the nested spheres every query ran fastest with 4 (1e7
 *                      rays, ms with 2/4/8/16 steps: ray_fire 7.36/6.50/
 *                      6.70/8.03, point_in_volume 7.05/6.23/6.41/7.71,
 *                      occluded 5.52/4.90/5.15/6.26, find_volume 22.6/22.1/
 *                      24.5/29.9)
 *   "trace_node_iters_fp64"  the same for the all-FP64 path
 *   "trace_node_iters_direct"  the same for mixed calls whose rays the
 *                      kernel reads in place from host memory (host_direct;
 *                      default 6).  The best setting differs: 1e7 rays of
 *                      the nested spheres ran 6.45 ms from device arrays
 *                      with 4 steps (6.64 with 8) but in place 6.93 ms with
 *                      6, 7.03 with 8, 7.39 with 4 and 7.48 with 12
 *   "trace_flush_wait" number of lanes (1..32, default 4) whose rays wait
 *                      only on queued FP64 candidate tests before the warp
 *                      drains a partly filled queue
 *   "trace_stack"      shared-memory traversal stack entries per ray (16..64,
 *                      steps of 8; default 40).  Deeper stacks take shared
 *                      memory and so resident blocks.  A launch raises it to
 *                      (node width - 1) x (depth of the deepest surface tree),
 *                      which no traversal can exceed, up to 64; only trees
 *                      deeper than that can make a ray end with
 *                      XDGCU_RAY_STACK_OVERFLOW
 *   "trace_grab"       0 (default): each warp walks one contiguous slice of
 *                      the batch fixed at launch; > 0 (a multiple of 32): warps
 *                      take this many rays at a time from a device work queue,
 *                      which balances batches of very uneven per-ray cost
 *   "particle_event_wait"  particle loop of xdgcu_transport_surfaces: lanes
 *                      whose flights have ended that a warp gathers before it
 *                      runs their events together (1..32, default 16)
 *   "transport_event_wait" particle loop of xdgcu_transport_elements, mixed
 *                      precision: lanes whose events need the FP64 sample
 *                      (collisions, uncertain exits) that a warp gathers
 *                      before it runs them together (1..32, default 4)
 *   "trace_sort_min"   batches of at least this many rays (default 0 = never)
 *                      are traversed in a coherent order: sorted on the device
 *                      by tree, direction octant and the Morton code of the
 *                      origin.  Results are written at the callers' indices
 *                      and do not depend on it
 *   "leaf_max"         primitives per BVH leaf for trees built afterwards (1..4,
 *                      default 2)
 *   "node_width"       children per BVH node for trees built (or rebuilt,
 *                      xdgcu_rebuild_trees) afterwards: 4 (default) or 8
 *   "bvh_sah"          how trees built afterwards group the binary tree's
 *                      nodes into wide nodes: 1 (default) at the least
 *                      surface-area cost (a dynamic program over the binary
 *                      tree), 0 greedily opening the largest child.  Results
 *                      do not depend on it
 *   "bvh_prim_cost"    cost of one primitive test relative to one wide-node
 *                      visit in that surface-area cost, in thousandths
 *                      (1..100000, default 300)
 *   "walk_queue"       mixed-precision walk: 1 runs the FP64 face tests of a
 *                      warp's tracks 32 at a time from a per-warp queue, 0
 *                      (default) lets each lane evaluate its own faces
 *   "walk_flush_wait"  number of tracks (1..32) waiting only on queued FP64
 *                      face tests before the warp runs a partly filled round
 *   "walk_sort_min"    batches of at least this many tracks (default 16384;
 *                      0 = never) are walked longest first: the tracks are
 *                      sorted by length on the device and dealt round-robin
 *                      to warps, so warps end on short tracks.  Results do not
 *                      depend on it.
 *   "trace_edge_table" mixed ray_fire / point_in_volume / occluded /
 *                      find_volume / particle loop: 1 (default) takes each
 *                      triangle's ray-independent FP64 terms (edge vectors,
 *                      edge normals, face normal) from a 256-byte record per
 *                      triangle, evaluated once when the surfaces are
 *                      uploaded, with the reference's operations; 0 computes
 *                      them from the vertices.  Results do not depend on it
 *   "closest_bound"    mixed closest: 1 (default) skips the FP64 point-triangle
 *                      test of triangles that a certified FP32 lower bound of
 *                      the distance (four planes per triangle, evaluated once
 *                      when the surfaces are uploaded) proves farther than the
 *                      nearest so far; 0 tests every triangle the box pruning
 *                      reaches.  Results do not depend on it
 *   "closest_node_steps"  closest, mixed: inner-node steps each lane takes
 *                      before the warp's lanes bound and test the triangles of
 *                      the leaves they hold together (1..64, default 4;
 *                      with the points in Morton order 4 ran 1e6 points in
 *                      15.4 ms, 8 in 16.6, 2 in 15.6, 16 in 17.4)
 *   "closest_node_steps_fp64"  the same for the all-FP64 closest (default 1)
 *   "closest_step_budget"  closest: node records and triangles a lane visits
 *                      for one point (default 1024; 0 = no limit) before the
 *                      point is left to a second kernel that searches it with
 *                      a whole warp.  A point almost equidistant from many
 *                      triangles (the centre of a sphere) otherwise holds one
 *                      lane, and the launch, for thousands of steps (1e6
 *                      points of the nested spheres: 25.8 -> 32.0 Mpoints/s
 *                      mixed, 4.45 -> 6.23 FP64).  Results do not depend on
 *                      it
 *   "closest_sort_min"  closest: batches (or staged chunks) of at least this
 *                      many points run in the order of [tree | Morton code
 *                      of the point] (default 65536; 0 = the caller's
 *                      order), so that the points of a warp share their
 *                      upper nodes and take similar work; the order is
 *                      computed in the call's scratch (one radix sort).
 *                      1e6 points of the nested spheres: 35.9 -> 60.5
 *                      Mpoints/s mixed, 155 -> 92 ms FP64.  Results do not
 *                      depend on it
 *   "find_sort_min"    the same for find_element (default 65536; 1e6 points
 *                      of the 750,000-tet cube: 0.723 -> 0.700 ms mixed,
 *                      8.74 -> 8.07 ms FP64).  The ray queries' own order
 *                      (trace_sort_min) stays off by default: with it,
 *                      point_in_volume of 1e7 points took 15.9 instead of
 *                      6.7 ms, the warps' contiguous shares of similar rays
 *                      being unequal work
 *   "find_node_steps_fp64"  the same for the all-FP64 find_element (default
 *                      16), and for the mixed one when it runs in phases
 *   "scratch_keep_bytes"  the calls' temporary device memory (allocated on
 *                      their stream) comes from a memory pool of the
 *                      context that keeps up to this many bytes of it between
 *                      calls (default 8 GiB; 0 returns it to the driver at
 *                      each synchronisation, as the device's default pool
 *                      does); setting it waits for the device and releases
 *                      what exceeds it.  The
 *                      pool is destroyed with the context; with
 *                      XDGCU_SCRATCH_POOL=0 in the environment when the
 *                      context is created, the device's default pool serves
 *                      instead (for tools that save and restore device
 *                      memory, such as a profiler's kernel replay).  Read-only
 *                      "scratch_bytes_reserved" is what the pool holds and
 *                      "scratch_bytes_high" the most it has lent at once
 *                      (set it to 0 to restart the count)
 *   "packed_walk_passes"  xdgcu_walk_elements_packed: 1 (default) walks each
 *                      track once, in resumed rounds; 2 walks it twice (a
 *                      count walk, then an emit walk), without the temporary
 *                      memory of the rounds.  Results do not depend on it
 *   "find_element_phased"  mixed find_element: 0 (default) runs one lane per
 *                      point on its own, the faster for points inside tets
 *                      (1409 against 1249 Mpoints/s on 1e6 uniform points of
 *                      a 750,000-tet cube); 1 runs the warp's lanes in step
 *                      with their exact FP64 tests together, the faster for
 *                      points on tet faces, where the FP32 filter decides
 *                      little (445 against 198 Mpoints/s on the cube's faces).
 *                      xdgcu_segments_global locates in phases after its
 *                      first round whatever this says.  Results do not
 *                      depend on it
 *   "segments_walk_cap"  xdgcu_segments_global and the packed walk's rounds:
 *                      segments a walk emits per
 *                      round before it pauses (1..1024; 0, the default, picks
 *                      per round the largest power of two in 16..256 for which
 *                      that round's walks fit a buffer of about 1 GiB, so
 *                      rounds with fewer walks pause fewer of them).  Results
 *                      do not depend on it
 *   "walk_edge_table"  mixed walk: 1 (default) takes the FP64 Plucker
 *                      coordinates of a face's edges from the edge table built
 *                      with the mesh (each edge's e and e x lo evaluated once,
 *                      the same values), 0 computes them from the vertices;
 *                      read-only "walk_edges" is the table's edge count (0
 *                      when the mesh has none).  Results do not depend on it
 *   "host_direct"      calls with host arrays: 0 stages every host array
 *                      through device memory, in chunks that overlap copies
 *                      with compute; 1 lets the kernels read and write
 *                      page-locked arrays in place (each byte crosses the
 *                      host link once, inside the kernel); 2 does the same
 *                      for pageable memory too when the device reads it
 *                      through the host's page tables (read-only key
 *                      "pageable_direct" = 1, as on Grace systems); 3
 *                      keeps pageable arrays in place and
 *                      page-locked arrays in place unless the call is large
 *                      enough (more than 2 chunks of 2^21 rays) for the
 *                      staged pipeline to overlap its copies; 4 is 2 except
 *                      that such a large call reads its page-locked inputs
 *                      in place and stages its outputs; 5 (the default)
 *                      chooses among 2, 3 and 4 by measurement: the first
 *                      nine large calls with host arrays take them in turn,
 *                      the last six are timed, and every later large call
 *                      takes the fastest (read-only key "host_direct_choice": -1 while
 *                      undecided, then 2, 3 or 4; setting host_direct to 5
 *                      again starts a new choice).  Which is faster depends
 *                      on the machine and the launch settings.  Staged
 *                      chunks' kernels alternate between two streams and take
 *                      their rays from the device work queue, so that one
 *                      launch's tail overlaps the next.  Tallies updated
 *                      atomically are always staged.  Results do not depend
 *                      on it. */
int xdgcu_set_tuning(xdgcu_ctx* ctx, const char* key, int64_t value);
int xdgcu_get_tuning(const xdgcu_ctx* ctx, const char* key, int64_t* value);

/* Queries the traversal autotuner can tune for. */
enum {
  XDGCU_QUERY_RAY_FIRE = 0,
  XDGCU_QUERY_POINT_IN_VOLUME = 1,
  XDGCU_QUERY_OCCLUDED = 2,
  XDGCU_QUERY_FIND_VOLUME = 3
};

/* Autotuner of the traversal launch parameters (no counterpart in the
 * reference).  Runs the sample batch (device arrays; arguments as for the
 * query, EXITING orientation for ray_fire, no exclusions) under settings of
 * trace_occupancy, trace_stack, trace_node_iters (or trace_node_iters_fp64
 * for XDGCU_FP64), trace_flush_wait, trace_grab and, for samples of at least
 * 65,536 rays, trace_sort_min, one key at a time, and leaves the context set
 * to the fastest combination found.  With tune_tree != 0 it does so for
 * every tree shape -- node_width 4 or 8, leaf_max 2, 3 or 4 -- rebuilding
 * the surface trees for each (xdgcu_rebuild_trees), and keeps the fastest.  Each setting is timed as the median of
 * `reps` launches after one untimed launch.  Every setting must reproduce
 * the first run's outputs byte for byte (XDGCU_ERR_STATE otherwise); settings
 * whose smaller stack overflows are skipped.  When the coherent order wins,
 * trace_sort_min is set to max(65536, n/4).  best_ms (may be NULL) receives
 * the sample's time under the chosen settings.  Synchronous; do not run
 * queries of this context meanwhile. */
int xdgcu_autotune_trace(xdgcu_ctx* ctx, int32_t query, int32_t tree, const int32_t* ray_trees,
                         int64_t n, const double* origins, const double* directions,
                         int32_t precision, int32_t reps, int32_t tune_tree, double* best_ms);

/* Autotuner of the walk launch parameters (no counterpart in the reference):
 * walk_queue (mixed precision only), walk_flush_wait and, for samples of at
 * least 16,384 tracks, walk_sort_min, on a sample of xdgcu_walk_elements
 * (device arrays, strided output of max_segs per track allocated by the
 * tuner).  Same search, timing and result check as xdgcu_autotune_trace;
 * when the length order wins, walk_sort_min is set to max(16384, n/4). */
int xdgcu_autotune_walk(xdgcu_ctx* ctx, int64_t n, const int32_t* start_index,
                        const double* start, const double* u, const double* distance,
                        int32_t max_segs, int32_t precision, int32_t reps, double* best_ms);

/* Rebuilds the existing trees (kinds: 1 = surface trees, 2 = element trees,
 * 3 = both) with the current "node_width" and "leaf_max", keeping their ids
 * and members.  No counterpart in the reference (Embree trees are built
 * once); the autotuner uses it to compare node widths.  Must not run while
 * queries of this context are running. */
int xdgcu_rebuild_trees(xdgcu_ctx* ctx, int32_t kinds);

/* Tree statistics: out[0] = nodes, [1] = primitives, [2] = depth,
 * [3] = bytes of FP32 nodes, [4] = bytes of FP64 nodes, [5] = node width. */
int xdgcu_surface_tree_info(const xdgcu_ctx* ctx, int32_t tree, int64_t out[8]);
int xdgcu_element_tree_info(const xdgcu_ctx* ctx, int32_t tree, int64_t out[8]);

#ifdef __cplusplus
}
#endif

#endif /* XDGCU_H */
