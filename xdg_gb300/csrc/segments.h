// segments.h -- device kernels of the global track loop, XDG::segments(start,
// end) (xdg.cpp:142-198), which xdgcu_segments_global (api.cu) composes with
// find_element, ray_fire and the packed walk.
//
// Every track keeps its state in device arrays indexed by track: position r,
// direction u, remaining distance, the number of segments written so far
// (`written`, so that `written > 0` is the reference's `segments.size() > 0`),
// the mesh id of its last segment and a status.  A round runs, for the
// tracks still active:
//   locate   find_element(r) in the global element tree;
//   decide   the element just left does not count (xdg.cpp:162); tracks in an
//            element go to the walk list, the others fire a ray in the
//            implicit complement from r + u * TINY_BIT;
//   re-enter a hit within the remaining distance moves the track to the hit
//            plus TINY_BIT and continues in the element behind the hit face
//            (get_boundary_face_element); a miss, a hit beyond the distance or
//            a face without an element ends the track (xdg.cpp:166-183);
//   walk     walk_elements(element, r, u, distance) of the walk list, at most
//            K segments per track and round (one pass, K-strided buffer): a
//            walk that reaches K pauses, and the next round resumes it where
//            it stopped (the element, position and remaining distance the
//            walk kernel reports, as its own steps computed them) without
//            locating the track again.  The walk kernel also sums the lengths
//            it emits, in order, continuing the sum of the walk's earlier
//            rounds (std::accumulate across the pauses);
//   advance  the round's segments packed into a buffer of the round (one warp
//            per track); when the walk ends, r += u * segment_sum and
//            distance -= segment_sum (xdg.cpp:188-193); tracks with
//            distance > 0 stay active.
// When no track is active, the per-track totals are scanned into the output
// offsets and every round's segments are copied to their place.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace xdgcu {

struct SegState {
  int64_t n;
  double* r;         // 3 per track
  double* u;         // 3 per track
  double* dist;
  int64_t* written;  // segments emitted so far
  int32_t* last;     // mesh id of the last segment (valid when written > 0)
  int32_t* status;   // per track: XDGCU_RAY_* (OK until something stops it)
  int8_t* stopped;   // the track's loop has returned
  // the walk in progress (walk_elements(element, r, u, distance) of one
  // iteration of the loop): its own position and remaining distance, the
  // sum of its segments so far, their number, where it resumes, and whether
  // it is paused at the per-round segment cap
  double* wr;        // 3 per track
  double* wd;
  double* wsum;
  int32_t* wcount;
  int32_t* welem;
  int8_t* paused;
};

// u = (end - start) / |end - start|, distance = |end - start|, r = start
// (xdg.cpp:148-153); tracks with distance > 0 are appended to `act`.
cudaError_t seg_init(const SegState& s, const double* starts, const double* ends, int32_t* act,
                     int32_t* n_act, cudaStream_t st);

// The packed walk (walk_elements of every track, no global loop around it):
// track t starts as a walk paused at element start[t], position org[t],
// direction dir[t] and distance dist[t]; act[t] = t.  State r and dist are
// not used.
cudaError_t seg_walk_init(const SegState& s, const int32_t* start, const double* org,
                          const double* dir, const double* dist, int32_t* act, cudaStream_t st);

// The active tracks: paused walks to the walk list (resumed at welem), the
// others to `loc` (to be located).
cudaError_t seg_split(const SegState& s, const int32_t* act, int64_t m, int32_t* walk_t,
                      int32_t* walk_start, int32_t* n_walk, int32_t* loc, int32_t* n_loc,
                      cudaStream_t st);

// pts[k] = r[act[k]]
cudaError_t seg_gather_points(const SegState& s, const int32_t* act, int64_t m, double* pts,
                              cudaStream_t st);

// For act[k] with find_element result (eid[k], eidx[k]): to the walk list
// (walk_t, walk_start) when in an element other than the last one walked,
// else to the ray list (out_t, ray origins r + u * TINY_BIT, directions u).
cudaError_t seg_decide(const SegState& s, const int32_t* act, int64_t m, const int32_t* eid,
                       const int32_t* eidx, int32_t* walk_t, int32_t* walk_start,
                       int32_t* n_walk, int32_t* out_t, double* ray_org, double* ray_dir,
                       int32_t* n_out, cudaStream_t st);

// The implicit-complement hits of the ray list: re-entry or end of track.
// bfe_face (ascending face ids) / bfe_elem: get_boundary_face_element.
// Elements outside [0, n_tets) count as none.
cudaError_t seg_reenter(const SegState& s, const int32_t* out_t, int64_t m, const double* t_hit,
                        const int32_t* surf, const int32_t* face, const int32_t* bfe_face,
                        const int32_t* bfe_elem, int64_t n_bfe, int32_t n_tets, int32_t* walk_t,
                        int32_t* walk_start, int32_t* n_walk, cudaStream_t st);

// The walk's inputs for the walk list, from each track's walk state:
// xr[k] = wr[t], xu[k] = u[t], xd[k] = wd[t], xsum[k] = wsum[t].
cudaError_t seg_walk_inputs(const SegState& s, const int32_t* walk_t, int64_t m, double* xr,
                            double* xu, double* xd, double* xsum, cudaStream_t st);

// off[k] = the segments of walk entry k this round keeps: its count, cut
// where the walk would pass max_segs segments.
cudaError_t seg_round_counts(const SegState& s, const int32_t* walk_t, int64_t m,
                             const int32_t* cnt, int32_t max_segs, int64_t* off, cudaStream_t st);

// The kept segments of the round's walk (rows of K in seg_elem / seg_len) to
// out_elem / out_len at off[k] .. off[k+1]-1, one warp per walk entry.
cudaError_t seg_pack(int64_t m, int32_t K, const int32_t* seg_elem, const double* seg_len,
                     const int64_t* off, int32_t* out_elem, double* out_len, cudaStream_t st);

// After the round's walk (K-strided segments seg_elem, counts cnt, statuses
// wst, and per walk entry where it stopped: element wstop, position wend_r,
// distance left wend_d, running length sum wsum) and the scan of the kept
// counts into off[0..m]: the walk state advanced, dst_rel[k] = the track's
// segments written before this round; a walk that ends applies segment_sum
// to r and distance; the tracks still active (paused or with distance left)
// are appended to act_next.  With walk_only (the packed walk) a walk that
// ends finishes its track, with the walk's status.
cudaError_t seg_advance(const SegState& s, const int32_t* walk_t, int64_t m, int32_t K,
                        const int32_t* seg_elem, const int32_t* cnt, const int32_t* wst,
                        const int32_t* wstop, const double* wend_r, const double* wend_d,
                        const double* wsum, int32_t max_segs, const int64_t* off,
                        int64_t* dst_rel, int32_t* act_next, int32_t* n_act, cudaStream_t st,
                        bool walk_only = false);

// Tracks still active after the last allowed round end with `code`.
cudaError_t seg_stop_active(const SegState& s, const int32_t* act, int64_t m, int32_t code,
                            cudaStream_t st);

// offsets[t] = written[t] (the scan then turns them into offsets).
cudaError_t seg_counts(const SegState& s, int64_t* offsets, cudaStream_t st);

// Tracks with segments that end beyond `capacity` get XDGCU_RAY_OUTPUT_FULL.
cudaError_t seg_mark_full(const SegState& s, const int64_t* offsets, int64_t capacity,
                          cudaStream_t st);

// One round's segments to their final place: track t's k-th segment of the
// round goes to offsets[t] + dst_rel + k when the track's segments fit in
// `capacity`; nothing is written for a track that does not fit.  One warp
// per walk entry.
cudaError_t seg_scatter(const SegState& s, const int32_t* walk_t, int64_t m, const int64_t* off,
                        const int64_t* dst_rel, const int32_t* seg_elem, const double* seg_len,
                        const int64_t* offsets, int64_t capacity, int32_t* out_elem,
                        double* out_len, cudaStream_t st);

}  // namespace xdgcu
