/*
 * xdg_oracle.h -- CPU oracle for the XDG ray-query hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library restates, in plain C, the
 * double-precision semantics of the reference's ray queries so that the CUDA
 * engine can be checked against it.  Only tests/, __graft_entry__.smoke() and
 * the cpu_baseline leg of bench.py load it; the product path never does.
 *
 * Every function cites the reference file:line it restates (paths relative to
 * the reference project root).  The library is compiled with
 * -ffp-contract=off so each double operation rounds exactly like the
 * reference's C++ expressions (no fused multiply-add).
 *
 * Tie rules.  The reference resolves exact distance ties by Embree's traversal
 * order, which no test pins.  The oracle (and the CUDA engine) use a fixed
 * rule instead: among accepted candidates with equal distance the lowest mesh
 * id wins (face id for ray_fire/point_in_volume/closest, element id for
 * find_element).
 */
#ifndef XDG_ORACLE_H
#define XDG_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* constants.h:15, 30, 32 */
#define XO_INFTY 1.7976931348623157e+308
#define XO_ID_NONE (-1)

/* shared_enums.h:11-15 */
enum { XO_ANY = -1, XO_EXITING = 0, XO_ENTERING = 1 };

/* per-query status codes (shared meaning with the CUDA engine) */
enum {
  XO_OK = 0,
  XO_WALK_LIMIT = 4,     /* walk stopped at the caller's segment capacity */
  XO_NO_EXIT_FACE = 5,   /* next_element found no exiting face */
  XO_EVENT_LIMIT = 7,    /* particle stopped at max_events */
  XO_LOST = 8,           /* particle_sim: no surface ahead */
};

/* ---- single-primitive kernels ------------------------------------------ */

/* plucker.h:45-62 */
double xo_plucker_edge_test(const double va[3], const double vb[3],
                            const double ray[3], const double ray_normal[3]);

/* plucker.h:64-161; returns hit (0/1), writes t when hit */
int xo_plucker_ray_tri(const double v[9], const double origin[3],
                       const double dir[3], double t_max, double t_min,
                       int use_orientation, int orientation, double* t_out);

/* tetrahedron_contain.cpp:11-43; v = 4 vertices x 3 */
int xo_tet_contains(const double p[3], const double v[12]);

/* closest.cpp:6-28 (region of the projection) */
int xo_closest_region(const double v[9], const double p[3]);

/* closest.cpp:54-183 */
void xo_closest_on_tri(const double v[9], const double p[3], double out[3]);

/* vec3da.h:61-66 (normalize with the min_rcp_input clamp), in place */
void xo_normalize(double v[3]);

/* mesh_manager_interface.cpp:216-220 */
void xo_face_normal(const double v[9], double n[3]);

/* ---- trees ------------------------------------------------------------- */

typedef struct xo_tree xo_tree;

/* A surface tree: n triangles given by their three vertices in mesh order
 * (9 doubles each), mesh face id, surface id, and a per-triangle flag that is
 * 1 when the tree is the surface's reverse-sense volume (the normal is then
 * flipped, triangle_intersect.cpp:84-87).  `bump` is the box dilation of
 * ray_tracing_interface.cpp:20-24.  use_bvh=0 selects brute force. */
xo_tree* xo_tree_create_tris(int64_t n, const double* tri_xyz,
                             const int32_t* face_ids, const int32_t* surf_ids,
                             const uint8_t* flip, double bump, int use_bvh);

/* An element tree: n tets (12 doubles each) and their mesh ids; the box bump
 * is each element's own dilation (tetrahedron_contain.cpp:47-63). */
xo_tree* xo_tree_create_tets(int64_t n, const double* tet_xyz,
                             const int32_t* elem_ids, int use_bvh);

void xo_tree_destroy(xo_tree* tree);

/* embree/ray_tracer.cpp:289-326 + triangle_intersect.cpp:52-109.
 * dist_limit may be NULL (INFTY).  excl_off (n+1) / excl_ids may be NULL.
 * Miss: t = INFTY, surf = face = ID_NONE. */
void xo_ray_fire(const xo_tree* tree, int64_t n, const double* org,
                 const double* dir, const double* dist_limit, int orientation,
                 const int32_t* excl_off, const int32_t* excl_ids,
                 double* t_out, int32_t* surf_out, int32_t* face_out,
                 int n_threads);

/* embree/ray_tracer.cpp:259-287.  dir may be NULL: the default direction
 * (1/sqrt(2), 1/sqrt(2), 0) of :268 is used. */
void xo_point_in_volume(const xo_tree* tree, int64_t n, const double* pts,
                        const double* dir, const int32_t* excl_off,
                        const int32_t* excl_ids, int32_t* inside_out,
                        int n_threads);

/* embree/ray_tracer.cpp:347-370 + triangle_intersect.cpp:139-161:
 * dist = -INFTY on a hit, INFTY otherwise; returns occluded flag. */
void xo_occluded(const xo_tree* tree, int64_t n, const double* org,
                 const double* dir, int32_t* occ_out, double* dist_out,
                 int n_threads);

/* embree/ray_tracer.cpp:328-345 + triangle_intersect.cpp:111-137 */
void xo_closest(const xo_tree* tree, int64_t n, const double* pts,
                double* dist_out, int32_t* face_out, int n_threads);

/* embree/ray_tracer.cpp:226-257 + tetrahedron_contain.cpp:94-114.
 * Writes the element's mesh id and its index within the tree (or -1). */
void xo_find_element(const xo_tree* tree, int64_t n, const double* pts,
                     int32_t* elem_id_out, int32_t* elem_idx_out,
                     int n_threads);

/* ---- tet walk ----------------------------------------------------------- */

typedef struct xo_tetmesh xo_tetmesh;

/* conn: 4 vertex indices per tet; adj: 4 neighbour tet indices per tet in
 * face order (-1 on the boundary); face_table: 4 faces x 3 local vertex
 * indices (the mesh library's ElementFaceAccessor ordering, e.g. MOAB's
 * {0,1,3},{1,2,3},{2,0,3},{0,2,1} in moab/direct_access.h:181-183). */
xo_tetmesh* xo_tetmesh_create(int64_t n_vert, const double* xyz, int64_t n_tet,
                              const int32_t* conn, const int32_t* adj,
                              const int32_t face_table[12]);
void xo_tetmesh_destroy(xo_tetmesh* mesh);

/* mesh_manager_interface.cpp:149-200.  Returns a status: XO_NO_EXIT_FACE when
 * no face is exited (the reference then indexes the adjacency with -1, which
 * is undefined; here next = -1 and dist = INFTY). */
int xo_next_element(const xo_tetmesh* mesh, int32_t elem, const double r[3],
                    const double u[3], int32_t* next_out, double* dist_out);

/* mesh_manager_interface.cpp:106-136 for n tracks.  Output is track-major
 * with stride max_segs: seg_elem[i*max_segs + k], seg_len[...]; seg_count[i]
 * holds the number written and status[i] a status code. */
void xo_walk_elements(const xo_tetmesh* mesh, int64_t n, const int32_t* start_elem,
                      const double* start, const double* u, const double* distance,
                      int32_t max_segs, int32_t* seg_elem, double* seg_len,
                      int32_t* seg_count, int32_t* status, int n_threads);

/* ---- particle loops ------------------------------------------------------ */

/* Random sampling of the engine's particle loops (the engine gives each
 * particle its own SplitMix64 stream where the reference tools share one
 * drand48() stream): uniform in [0,1), -log(1-U)*mfp with the series
 * logarithm, Marsaglia isotropic direction + Vec3da::normalize. */
double xo_uniform(uint64_t* state);
double xo_series_log(double x);
double xo_sample_collision(uint64_t* state, double mfp);
void xo_sample_direction(uint64_t* state, double dir[3]);

/* The in-mesh part of the walk_elements tool loop (tools/walk_elements.h:
 * 73-87): per particle, events until it leaves the mesh (elem = -1) or
 * reaches max_events (XO_EVENT_LIMIT).  State arrays are updated in place;
 * tally (may be NULL) gets each event's length added to its tet. */
void xo_transport_elements(const xo_tetmesh* mesh, int64_t n, int32_t* elem, double* pos,
                           double* dir, uint64_t* rng, double mfp, int32_t max_events,
                           double* distance, int32_t* events, double* tally,
                           int32_t* status, int n_threads);

/* The whole walk_elements tool loop (tools/walk_elements.h:60-96) for
 * particles that start in tet elem[i]: the in-mesh loop above, and after
 * leaving the mesh the re-entry search -- ray_fire in the implicit
 * complement's tree (EXITING, the hit faces of this search excluded), move
 * to the hit, find_element(r + u*TINY_BIT) in elem_tree -- repeated until an
 * element is found or nothing is hit (the particle ends).  events counts one
 * per loop iteration as the tool does; elem_tree's primitive index must be
 * the tet index. */
void xo_walk_particles(const xo_tetmesh* mesh, const struct xo_tree* ipc_tree,
                       const struct xo_tree* elem_tree, int64_t n, int32_t* elem, double* pos,
                       double* dir, uint64_t* rng, double mfp, int32_t max_events,
                       double* distance, int32_t* events, int32_t* status, int n_threads);

/* The particle_sim tool loop (tools/particle_sim.h:128-141) with the
 * engine's per-particle streams: per event ray_fire in the particle's volume
 * tree (EXITING, history excluded, hit appended), collision sampling,
 * advance, then collide (new direction, history cleared) or cross the
 * surface by its boundary condition (surf_bc: 0 transmission -> next volume
 * by surf_fwd/surf_rev tree ids, 1 vacuum, 2 reflecting).  trees[k] is the
 * volume tree of tree id k+1; surface tables are indexed by surface id and
 * face_xyz (9 doubles) by face id.  tally (may be NULL) is indexed by tree
 * id.  Statuses: 0, XO_EVENT_LIMIT, XO_LOST, 9 (stuck), 1 (invalid). */
void xo_transport_surfaces(const xo_tree* const* trees, int32_t n_trees, const int32_t* surf_fwd,
                           const int32_t* surf_rev, const int32_t* surf_bc, int32_t n_surf_ids,
                           const double* face_xyz, int32_t n_face_ids, int64_t n, int32_t* tree,
                           double* pos, double* dir, uint64_t* rng, double mfp,
                           int32_t max_events, int32_t graveyard_tree, double* distance,
                           int32_t* events, double* tally, int32_t* status, int n_threads);

/* Library self-description for tests. */
int xo_version(void);

#ifdef __cplusplus
}
#endif

#endif
