// trace.cu -- warp-synchronous BVH traversal for ray_fire, point_in_volume
// and occluded.
//
// GB300 issues FP64 at 1/64 of the FP32 rate, and an FP64 instruction costs
// its full issue slot however few lanes of the warp are active.  So the
// kernel keeps all per-lane work in FP32 and routes every FP64 evaluation
// through a per-warp queue that the whole warp drains together:
//
//   * each lane owns one ray at a time and advances it by one step per loop
//     iteration: either one 4-child node test or one triangle test;
//   * a triangle test runs the certified FP32 Plucker filter (geom.cuh); a
//     candidate it cannot reject is appended to the warp's queue;
//   * when 32 candidates are queued (or lanes are waiting on the queue), all
//     32 lanes evaluate one queued candidate each with the FP64 Plucker test
//     and the hit bookkeeping of triangle_intersect.cpp:52-109, then each ray
//     merges its own results (lowest (t, face id) wins, the fixed tie rule);
//   * a lane whose ray is finished and has nothing queued writes its result
//     and refills from the warp's current chunk of rays, so long rays do not
//     hold a whole warp idle.  Chunks are either one contiguous slice per warp
//     fixed at launch (no global atomics) or, when `grab` > 0, taken `grab`
//     rays at a time from a device work queue (one atomicAdd per chunk), which
//     balances batches whose rays cost very different amounts (many
//     geometries of uneven size in one launch).  An optional permutation
//     `order` (rays sorted by tree, direction octant and origin) makes the
//     rays of a warp coherent; results are written at the original index.
//
// Merging candidates evaluated against an older best distance gives the same
// answer as evaluating them one by one: the Plucker test's tMax only rejects
// t > tMax (plucker.h:158) and every other cull is independent of the best
// hit, so the result is the minimum over all accepted candidates.
//
// The all-FP64 variant (MIXED = false) uses the same loop with FP64 node
// boxes and queues every candidate triangle.
//
// Why the FP32 box test never loses a hit: every primitive box is dilated by
// `bump` (>= 1e-3 for surface trees, ray_tracing_interface.cpp:20-24), so the
// exact slab interval of a ray around any hit point has slack bump/|d|_inf on
// both sides, while the FP32 evaluation errs by at most ~5u(|box| + |o|).  A
// ray for which 8u(max|coordinate| + |o|_inf) is not below the bump tests FP64
// boxes instead (checked per ray, `use64`).
//
// Nodes are 4- or 8-wide per tree (an 8-wide node's two records are tested,
// sorted and merged).
//
// Stack: `stack` entries per lane (16..64, a launch parameter) in dynamic
// shared memory, [entry][thread] so that lanes hit distinct banks; in the
// FP64 traversal each entry keeps a lower bound of its near distance so
// entries beyond a closer hit found meanwhile are discarded without fetching
// the node (stack_keys below).  A deeper stack costs shared memory and so
// resident blocks and L1 capacity; overflow ends the ray with
// RAY_STACK_OVERFLOW.
#include <atomic>

#include "sample.cuh"
#include "traverse.cuh"

namespace xdgcu {

namespace {

constexpr int kTBlock = 128;
constexpr int kTWarps = kTBlock / 32;
constexpr int kTStackMin = 16, kTStackMax = 64;
constexpr int kQ = 256;  // ring buffer, power of two; at most 31 + 4*32 entries live
constexpr unsigned kFull = 0xffffffffu;

// Queue entries pack (owner lane << 27) | leaf-order primitive index (trees
// hold < 2^27 primitives).
struct WarpQueue {
  uint32_t ent[kQ];
  double rt[32];
  int32_t rface[32];
  int32_t rsurf[32];
  int32_t rflags[32];  // bit 0: accepted, bit 1: dot(d, n) > 0
  int32_t rtri[32];    // global triangle of the result (particle mode: face normal)
  uint32_t head, tail;
  int32_t pad[2];
};

// Short-stack entries are node references, with (FP64 traversal only) the
// node's near distance, rounded down to its upper 16 bits (a lower bound of a
// non-negative float), so that a pop skips a node that starts beyond the
// current best hit.  The mixed traversal and occluded keep no distances:
// their FP32 node tests are cheap to repeat, and the smaller stack leaves
// more of the SM's shared-memory/L1 storage to cache nodes and triangles
// (ray_fire on 655k triangles: 1137 Mrays/s without distances, 1122 with
// 16-bit and 1060 with 32-bit ones; FP64: 366 with 16-bit, 353 without).
template <int MODE, bool MIXED>
__host__ __device__ constexpr bool stack_keys() {
  return !MIXED && MODE != MODE_OCCLUDED;
}

// Dynamic shared memory: the warp queues, each lane's FP64 ray (origin and
// direction, [6][kTBlock]), the lanes' LaneCold, then the stack's references
// [stack][kTBlock] and, with keys, near distances [stack][kTBlock].  The FP64 ray is read only
// when a traversal starts (its FP32 forms), by the FP64 tests of the drain
// (any lane of the warp reads the owner's) and by the particle events;
// keeping it out of the registers cut the 4-blocks-per-SM variant's spills
// from 144 to 52 bytes per thread and raised ray_fire on 655k triangles
// from 1275 to 1420 Mrays/s.
constexpr size_t kRayBytes = 6 * sizeof(double) * kTBlock;

// Per-lane state the traversal loop does not touch, in shared memory for the
// same reason: the best hit so far, the tree, the exclusion list and the ray
// index.  The drain reads the owner lane's entries directly instead of
// shuffling them.  ray_fire 1404 -> 1447 Mrays/s (spills at 4 blocks per SM
// 52 -> 16 bytes per thread).
struct LaneCold {
  double bt[kTBlock];
  int64_t ray[kTBlock];
  const TreeDev* tree[kTBlock];
  const int32_t* excl[kTBlock];
  int32_t tid[kTBlock], nexcl[kTBlock], bface[kTBlock], bsurf[kTBlock];
};

// The mixed particle loop's per-particle state, likewise: its random
// stream, path length, events, history count and the triangle of the best
// hit (spills at 4 blocks per SM 40 -> 16 bytes per thread; particle_sim
// loop 468 -> 479 Mevents/s).
struct ParticleCold {
  unsigned long long rs[kTBlock];
  double pdist[kTBlock];
  int32_t pev[kTBlock], hc[kTBlock], btri[kTBlock];
};

__host__ __device__ constexpr size_t trace_smem_bytes(int stack, bool keys, bool particle) {
  return sizeof(WarpQueue) * kTWarps + kRayBytes + sizeof(LaneCold) +
         (particle ? sizeof(ParticleCold) : 0) +
         (size_t)stack * kTBlock * (sizeof(int32_t) + (keys ? sizeof(uint16_t) : 0));
}

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

template <int MODE, bool MIXED, int MINB>
__global__ void __launch_bounds__(kTBlock, MINB) k_trace(SurfArgs a, int64_t chunk) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int tx = threadIdx.x;
  WarpQueue& Q = reinterpret_cast<WarpQueue*>(smem_raw)[wib];
  double* const sray = reinterpret_cast<double*>(smem_raw + sizeof(WarpQueue) * kTWarps);
  LaneCold& LC = *reinterpret_cast<LaneCold*>(smem_raw + sizeof(WarpQueue) * kTWarps + kRayBytes);
  // (the all-FP64 particle loop keeps this state in registers: it has no
  // spills to remove, and the shared memory would cost it L1)
  constexpr bool kPCold = MODE == MODE_PARTICLE && MIXED;
  constexpr size_t kPC = kPCold ? sizeof(ParticleCold) : 0;
  ParticleCold& PC = *reinterpret_cast<ParticleCold*>(smem_raw + sizeof(WarpQueue) * kTWarps +
                                                     kRayBytes + sizeof(LaneCold));
  int32_t* const sref = reinterpret_cast<int32_t*>(smem_raw + sizeof(WarpQueue) * kTWarps +
                                                   kRayBytes + sizeof(LaneCold) + kPC);
  // the FP64 ray of lane slot t (this thread's: tx)
  auto ray_o = [&](int t) { return mk3(sray[t], sray[kTBlock + t], sray[2 * kTBlock + t]); };
  auto ray_d = [&](int t) {
    return mk3(sray[3 * kTBlock + t], sray[4 * kTBlock + t], sray[5 * kTBlock + t]);
  };
  auto set_o = [&](d3 v) {
    sray[tx] = v.x;
    sray[kTBlock + tx] = v.y;
    sray[2 * kTBlock + tx] = v.z;
  };
  auto set_d = [&](d3 v) {
    sray[3 * kTBlock + tx] = v.x;
    sray[4 * kTBlock + tx] = v.y;
    sray[5 * kTBlock + tx] = v.z;
  };
  uint16_t* const stn = reinterpret_cast<uint16_t*>(sref + (size_t)a.stack * kTBlock);
  constexpr bool kKeys = stack_keys<MODE, MIXED>();
  const int kstack = a.stack;
  const bool dyn = a.grab > 0;
  const int64_t gwarp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  int64_t cursor = dyn ? 0 : gwarp * chunk;
  int64_t end = dyn ? 0 : min(a.n, cursor + chunk);
  bool exhausted = false;  // work queue (grab > 0) has no rays left
  if (lane == 0) {
    Q.head = 0u;
    Q.tail = 0u;
  }
  __syncwarp();

  Counters cnt = {0, 0, 0, 0};
  unsigned long long rays_done = 0;

  // ---- lane state ----
  bool has_ray = false, trav = false, use64 = false;
  int32_t status = RAY_OK, npend = 0, vk = 0;
  // (LaneCold entries of this lane)
  int64_t& ray = LC.ray[tx];
  int32_t& tid = LC.tid[tx];
  const TreeDev*& tree = LC.tree[tx];
  double& bt = LC.bt[tx];
  int32_t& bface = LC.bface[tx];
  int32_t& bsurf = LC.bsurf[tx];
  const int32_t*& excl = LC.excl[tx];
  int32_t& nexcl = LC.nexcl[tx];
  ray = 0;
  tid = 0;
  tree = nullptr;
  bt = INFTY;
  bface = -1;
  bsurf = -1;
  excl = nullptr;
  nexcl = 0;
  const Node32* n32 = nullptr;
  const float4* prim32 = nullptr;
  int32_t cur = CHILD_EMPTY, leaf_p = 0, leaf_end = 0;
  int sp = 0;
  float bt32 = INFINITY;
  bool bhas = false, bdot = false;
  bool wide8 = false;  // the lane's tree has 8-wide nodes
  // MODE_PARTICLE: the particle's stream, path length, events, history count
  // and the triangle of the best hit
  unsigned long long rs_r = 0ull;
  double pdist_r = 0.0;
  int32_t pev_r = 0, hc_r = 0, btri_r = -1;
  unsigned long long& rs = kPCold ? PC.rs[tx] : rs_r;
  double& pdist = kPCold ? PC.pdist[tx] : pdist_r;
  int32_t& pev = kPCold ? PC.pev[tx] : pev_r;
  int32_t& hc = kPCold ? PC.hc[tx] : hc_r;
  int32_t& btri = kPCold ? PC.btri[tx] : btri_r;
  if (kPCold) {
    rs = 0ull;
    pdist = 0.0;
    pev = 0;
    hc = 0;
    btri = -1;
  }
  BoxRay32 br32;
  Ray32 r32;
  BoxRay64 br64;

  auto pop = [&]() {
    cur = CHILD_EMPTY;
    while (sp > 0) {
      --sp;
      const int32_t r = sref[sp * kTBlock + tx];
      if (!kKeys || __uint_as_float((uint32_t)stn[sp * kTBlock + tx] << 16) <= bt32) {
        if (ref_is_leaf(r)) {
          leaf_p = leaf_first(r);
          leaf_end = leaf_p + leaf_count(r);
        } else {
          cur = r;
        }
        return;
      }
    }
    trav = false;
  };

  // starts the traversal of the lane's ray in tree `tid` (status RAY_INVALID
  // for an unknown tree)
  auto begin_tree = [&]() {
    if (tid < 1 || tid > a.n_trees) {
      status = RAY_INVALID;
      trav = false;
      return;
    }
    trav = true;
    const TreeDev* T = a.trees + (tid - 1);
    tree = T;
    n32 = T->n32;
    prim32 = T->prim32;
    wide8 = T->width == 8;
    const int32_t root = T->root;
    bt32 = (MODE == MODE_OCCLUDED) ? INFINITY : f32_up(bt);
    if (MIXED) {
      br32 = make_boxray32(ray_o(tx), ray_d(tx));
      r32 = make_ray32(ray_o(tx), ray_d(tx));
      // FP32 box-test safety (see the file comment)
      use64 = !(8.0f * kU32 * (T->max_abs + r32.oabs) < T->bump);
    }
    if (!MIXED) br64 = make_boxray64(ray_o(tx), ray_d(tx));
    if (root == CHILD_EMPTY) {
      trav = false;
    } else if (ref_is_leaf(root)) {
      cur = CHILD_EMPTY;
      leaf_p = leaf_first(root);
      leaf_end = leaf_p + leaf_count(root);
    } else {
      cur = root;
    }
  };

  while (true) {
    // ---- finalize finished rays ----
    bool fin = has_ray && !trav && npend == 0;
    if (MODE == MODE_PARTICLE) {
      // A particle's event (sampling, logarithm, normalisation: ~100 FP64
      // instructions) is run for many lanes at once: a lane whose flight has
      // ended waits until event_wait lanes are ready or no lane of the warp
      // has traversal work left.  FP64 instructions cost the same issue time
      // however few lanes are active.
      const unsigned fm = __ballot_sync(kFull, fin);
      const unsigned wm = __ballot_sync(kFull, has_ray && (trav || npend > 0));
      if (!(__popc(fm) >= a.event_wait || wm == 0u)) fin = false;
    }
    if (fin) {
      bool done = true;
      if (MODE == MODE_RAY_FIRE) {
        a.t_out[ray] = bhas ? bt : INFTY;
        a.surf_out[ray] = bhas ? bsurf : -1;
        if (a.face_out) a.face_out[ray] = bhas ? bface : -1;
      } else if (MODE == MODE_PIV) {
        a.flag_out[ray] = (bhas && bdot) ? 1 : 0;  // embree/ray_tracer.cpp:282-286
      } else if (MODE == MODE_FIND_VOLUME) {
        // xdg.cpp:113-128: the first volume whose point_in_volume is true;
        // otherwise the lane restarts the same point in the next volume
        const bool inside = bhas && bdot;
        if (!inside && status == RAY_OK && vk + 1 < a.n_vols) {
          ++vk;
          tid = a.vol_trees[vk];
          bt = INFTY;
          bhas = false;
          bdot = false;
          bface = -1;
          bsurf = -1;
          sp = 0;
          leaf_p = leaf_end = 0;
          begin_tree();
          done = false;
        } else {
          a.flag_out[ray] = inside ? a.vol_ids[vk] : a.ipc_volume;
        }
      } else if (MODE == MODE_ALL_VOLUMES) {
        // point_in_volume in list entry vk (embree/ray_tracer.cpp:282-286),
        // then the lane restarts the same point in the next entry's tree
        a.vol_inside[ray * a.vol_stride + vk] = (bhas && bdot) ? 1 : 0;
        if (status == RAY_OK && vk + 1 < a.n_vols) {
          ++vk;
          tid = a.vol_trees[vk];
          bt = INFTY;
          bhas = false;
          bdot = false;
          bface = -1;
          bsurf = -1;
          sp = 0;
          leaf_p = leaf_end = 0;
          begin_tree();
          done = false;
        }
      } else if (MODE == MODE_PARTICLE) {
        // one event of tools/particle_sim.h:128-141 after the flight's
        // ray_fire (EXITING, history excluded)
        d3 o = ray_o(tx), d = ray_d(tx);
        bool alive = false;
        if (status == RAY_OK && tid > 0) {
          if (bhas && bt == 0.0) {
            status = RAY_STUCK;  // :36-40
          } else if (!bhas) {
            status = RAY_LOST;   // :41-45
          } else {
            // ray_fire appended the hit face to the history
            a.p_hist[ray * a.hist_cap + (hc % a.hist_cap)] = bface;
            ++hc;
            // :47-49.  The FP64 series logarithm is needed only when the
            // particle may collide: an FP32 logarithm with a certified margin
            // (|c32 - c| <= 6.1e-8 mfp + 3.7e-7 c; margin 1.1e-6 (c32 + mfp))
            // first tests c >= hit distance.
            const double U = uniform53(rs);
            bool cross = false;
            if (a.mfp < 1e30) {
              const float mfp32 = (float)a.mfp;
              const float c32 = -logf(__double2float_rn(1.0 - U)) * mfp32;
              cross = dlt(bt, (double)(c32 - 1.1e-6f * (c32 + mfp32)));
            }
            double c = 0.0;
            if (!cross) c = -series_log(1.0 - U) * a.mfp;  // sample_collision's value
            alive = true;
            if (!cross && dlt(c, bt)) {
              // advance + collide (:66-70, :57-64)
              o = add3(o, scl3(c, d));
              pdist += c;
              if (a.p_tally) atomicAdd(&a.p_tally[tid], c);
              ++pev;
              d = sample_direction(rs);
              hc = 0;
            } else {
              // advance to the surface + cross_surface (:71-75, :78-118)
              o = add3(o, scl3(bt, d));
              pdist += bt;
              if (a.p_tally) atomicAdd(&a.p_tally[tid], bt);
              ++pev;
              const int32_t sidx = __ldg(&a.tri_surf[btri]);
              const int32_t bc = __ldg(&a.surf_bc[sidx]);
              if (bc == BC_REFLECTING) {
                // surface_normal(surface, r, &history) = face_normal(history.back())
                // (xdg.cpp:272-289); reflect and renormalise (:88-96)
                d3 v0, v1, v2;
                const double* tx9 = a.tri_xyz + 9 * (int64_t)btri;
                v0 = mk3(tx9[0], tx9[1], tx9[2]);
                v1 = mk3(tx9[3], tx9[4], tx9[5]);
                v2 = mk3(tx9[6], tx9[7], tx9[8]);
                d3 nrm = face_normal64(v0, v1, v2);
                const double proj = dot3(nrm, d);
                const double mag = sqrt(nrm.x * nrm.x + nrm.y * nrm.y + nrm.z * nrm.z);
                nrm = scl3(2.0 * proj / mag, nrm);
                d = normalize64(sub3(d, nrm));
                a.p_hist[ray * a.hist_cap] = bface;  // history = {history.back()}
                hc = 1;
              } else if (bc == BC_VACUUM) {
                alive = false;
              } else {
                // MeshManager::next_volume (mesh_manager_interface.cpp:202-214)
                const int32_t fwd = __ldg(&a.surf_fwd_tree[sidx]);
                const int32_t rev = __ldg(&a.surf_rev_tree[sidx]);
                if (fwd == tid) {
                  tid = rev;
                } else if (rev == tid) {
                  tid = fwd;
                } else {
                  status = RAY_INVALID;  // not a parent volume of the surface
                  alive = false;
                }
                if (alive && (tid < 1 || tid == a.graveyard_tree)) {
                  tid = -1;  // :112-116
                  alive = false;
                }
              }
            }
            if (alive && pev >= a.max_events) {
              status = RAY_EVENT_LIMIT;
              alive = false;
            }
          }
        }
        set_o(o);
        set_d(d);
        if (alive) {
          // next flight from the new position in the (new) volume
          bt = INFTY;
          bhas = false;
          bdot = false;
          bface = -1;
          bsurf = -1;
          btri = -1;
          sp = 0;
          leaf_p = leaf_end = 0;
          excl = a.p_hist + ray * a.hist_cap;
          nexcl = min(hc, a.hist_cap);
          begin_tree();
          done = false;
        } else {
          a.p_pos[3 * ray] = o.x;
          a.p_pos[3 * ray + 1] = o.y;
          a.p_pos[3 * ray + 2] = o.z;
          a.p_dir[3 * ray] = d.x;
          a.p_dir[3 * ray + 1] = d.y;
          a.p_dir[3 * ray + 2] = d.z;
          a.p_tree[ray] = tid;
          a.p_rng[ray] = rs;
          a.p_dist[ray] = pdist;
          a.p_events[ray] = pev;
          a.p_hcount[ray] = hc;
        }
      } else {
        a.flag_out[ray] = bhas ? 1 : 0;
        if (a.dist_out) a.dist_out[ray] = bhas ? -INFTY : INFTY;  // :368-369
      }
      if (done) {
        if (a.status) a.status[ray] = status;
        has_ray = false;
        rays_done++;
      }
    }
    // ---- refill from the warp's chunk ----
    const unsigned need = __ballot_sync(kFull, !has_ray);
    if (need != 0u && dyn && cursor >= end && !exhausted) {
      // cursor, end and exhausted are warp-uniform
      unsigned long long base = 0ull;
      if (lane == 0) base = atomicAdd(a.work, (unsigned long long)a.grab);
      base = __shfl_sync(kFull, base, 0);
      if ((int64_t)base >= a.n) {
        exhausted = true;
      } else {
        cursor = (int64_t)base;
        end = min(a.n, cursor + (int64_t)a.grab);
      }
    }
    if (need != 0u && cursor < end) {
      if (!has_ray) {
        const int64_t pos = cursor + __popc(need & lanemask_lt());
        const int64_t idx = pos < end ? (a.order ? (int64_t)__ldg(&a.order[pos]) : pos) : -1;
        if (idx >= 0 && idx < a.n) {  // (an order entry out of range names no ray)
          ray = idx;
          has_ray = true;
          status = RAY_OK;
          npend = 0;
          sp = 0;
          bhas = false;
          bdot = false;
          bface = -1;
          bsurf = -1;
          leaf_p = leaf_end = 0;
          vk = 0;
          if (MODE == MODE_PARTICLE) {
            tid = a.p_tree[idx];
            set_o(load3(a.p_pos, idx));
            set_d(load3(a.p_dir, idx));
            rs = a.p_rng[idx];
            pdist = a.p_dist[idx];
            pev = a.p_events[idx];
            hc = a.p_hcount[idx];
            btri = -1;
          } else {
            tid = (MODE == MODE_FIND_VOLUME || MODE == MODE_ALL_VOLUMES)
                      ? (a.n_vols > 0 ? a.vol_trees[0] : 0)
                      : (a.ray_trees ? a.ray_trees[idx] : a.tree);
            set_o(load3(a.org, idx));
            if ((MODE == MODE_PIV || MODE == MODE_FIND_VOLUME || MODE == MODE_ALL_VOLUMES) &&
                a.dir == nullptr)
              set_d(mk3(1. / sqrt(2.0), 1 / sqrt(2.0), 0.0));  // embree/ray_tracer.cpp:268
            else
              set_d(load3(a.dir, idx));
          }
          bt = (MODE == MODE_RAY_FIRE && a.tmax) ? a.tmax[idx] : INFTY;
          excl = nullptr;
          nexcl = 0;
          if (MODE == MODE_PARTICLE) {
            excl = a.p_hist + idx * a.hist_cap;
            nexcl = hc < 0 ? 0 : min(hc, a.hist_cap);
          } else if (MODE != MODE_OCCLUDED && MODE != MODE_FIND_VOLUME &&
                     MODE != MODE_ALL_VOLUMES && a.excl_off) {
            const int32_t e0 = a.excl_off[idx];
            excl = a.excl_ids + e0;
            nexcl = a.excl_off[idx + 1] - e0;
          }
          if (!finite3(ray_o(tx)) || !finite3(ray_d(tx)) || nan_bits(bt) ||
              (MODE == MODE_PARTICLE && (hc < 0 || nan_bits(pdist)))) {
            status = RAY_INVALID;
            trav = false;
          } else if ((MODE == MODE_FIND_VOLUME || MODE == MODE_ALL_VOLUMES) && a.n_vols == 0) {
            trav = false;  // no volume to try (find_volume: the implicit complement)
          } else if (MODE == MODE_PARTICLE && tid < 0) {
            trav = false;  // the particle ended earlier: left as it is
          } else if (MODE == MODE_PARTICLE && pev >= a.max_events) {
            status = RAY_EVENT_LIMIT;
            trav = false;
          } else {
            begin_tree();
          }
        }
      }
      cursor += __popc(need);
    }
    if (__ballot_sync(kFull, has_ray) == 0u) break;

    // ---- one traversal step per active lane ----
    unsigned escm = 0u;   // escalated primitives of this step (bit k -> esc_p0 + k)
    int32_t esc_p0 = 0;
    // node phase: lanes without a pending leaf descend through inner nodes
    // (up to node_iters steps) until they hold a leaf or run out of work
    for (int it = 0; it < a.node_iters; ++it) {
      const bool want = trav && leaf_p >= leaf_end;
      if (__ballot_sync(kFull, want) == 0u) break;
      if (want) {
        cnt.node++;
        cnt.box += wide8 ? 8 : 4;
        // an 8-wide node is two 4-wide records, each tested and sorted, then
        // merged; a 4-wide node leaves the upper half empty
        int32_t cr[8];
        float key[8];
#pragma unroll
        for (int r = 0; r < 2; ++r) {
          if (r == 1 && !wide8) {
#pragma unroll
            for (int k = 4; k < 8; ++k) {
              key[k] = INFINITY;
              cr[k] = CHILD_EMPTY;
            }
            continue;
          }
          const int64_t rec = wide8 ? 2 * (int64_t)cur + r : (int64_t)cur;
          if (MIXED && !use64) {
            node_test32(n32 + rec, br32, bt32, key + 4 * r, cr + 4 * r);
          } else {
            double tn[4];
            if (MIXED) br64 = make_boxray64(ray_o(tx), ray_d(tx));  // rare: rays failing the FP32 safety test
            node_test64(tree->n64 + rec, br64, (MODE == MODE_OCCLUDED) ? INFTY : bt, tn,
                        cr + 4 * r);
#pragma unroll
            for (int k = 0; k < 4; ++k)
              key[4 * r + k] = tn[k] < INFINITY ? __double2float_rd(tn[k]) : INFINITY;
          }
          sort4(key + 4 * r, cr + 4 * r);
        }
        if (wide8) merge8(key, cr);
        int nhit = 0;
#pragma unroll
        for (int k = 0; k < 8; ++k) nhit += key[k] < INFINITY ? 1 : 0;
        if (nhit == 0) {
          pop();
        } else if (sp + nhit - 1 > kstack) {
          status = RAY_STACK_OVERFLOW;
          trav = false;
        } else {
#pragma unroll
          for (int k = 7; k >= 1; --k) {
            if (k < nhit) {  // static indices keep key/cr in registers
              sref[sp * kTBlock + tx] = cr[k];
              if (kKeys) stn[sp * kTBlock + tx] = (uint16_t)(__float_as_uint(key[k]) >> 16);
              ++sp;
            }
          }
          if (ref_is_leaf(cr[0])) {
            cur = CHILD_EMPTY;
            leaf_p = leaf_first(cr[0]);
            leaf_end = leaf_p + leaf_count(cr[0]);
          } else {
            cur = cr[0];
          }
        }
      }
    }
    // leaf phase: the whole leaf (<= 4 primitives) at once, so its loads overlap
    if (trav && leaf_p < leaf_end) {
      const int32_t p0 = leaf_p;
      const int np = leaf_end - leaf_p;
      leaf_p = leaf_end;
      esc_p0 = p0;
      cnt.prim += np;
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        if (k < np) {
          if (MIXED) {
            const int64_t q = 3 * (int64_t)(p0 + k);
            const float4 A = __ldg(&prim32[q]);
            const float4 B = __ldg(&prim32[q + 1]);
            const float4 C = __ldg(&prim32[q + 2]);
            const SignCert c = plucker_filter32(r32, A.x, A.y, A.z, B.x, B.y, B.z, C.x, C.y,
                                                C.z, B.w, A.w);
            if (!certified_miss(c)) escm |= 1u << k;
          } else {
            escm |= 1u << k;
          }
        }
      }
      if (cur == CHILD_EMPTY) pop();
    }
    // ---- enqueue this step's escalations (warp-wide exclusive scan) ----
    {
      const int c = __popc(escm);
      int incl = c;
#pragma unroll
      for (int off = 1; off < 32; off <<= 1) {
        const int y = __shfl_up_sync(kFull, incl, off);
        if (lane >= off) incl += y;
      }
      const int total = __shfl_sync(kFull, incl, 31);
      if (total > 0) {
        const uint32_t tail = Q.tail;
        __syncwarp();
        uint32_t pos = tail + (uint32_t)(incl - c);
        unsigned m = escm;
        while (m) {
          const int k = __ffs(m) - 1;
          m &= m - 1u;
          Q.ent[pos & (kQ - 1)] = ((uint32_t)lane << 27) | (uint32_t)(esc_p0 + k);
          ++pos;
        }
        npend += c;
        cnt.esc += c;
        if (lane == 0) Q.tail = tail + (uint32_t)total;
      }
    }
    __syncwarp();

    // ---- drain the FP64 queue with the whole warp ----
    while (true) {
      const uint32_t head = Q.head;
      const int qn = (int)(Q.tail - head);
      const unsigned act2 = __ballot_sync(kFull, trav);
      const unsigned waiting = __ballot_sync(kFull, has_ray && !trav && npend > 0);
      if (!(qn >= 32 || (qn > 0 && (act2 == 0u || __popc(waiting) >= a.flush_wait)))) break;
      const int nq = min(qn, 32);
      const bool mine = lane < nq;
      const uint32_t ent = mine ? Q.ent[(head + lane) & (kQ - 1)] : ((uint32_t)lane << 27);
      const int owner = (int)(ent >> 27);
      const int32_t prim = (int32_t)(ent & 0x7ffffffu);
      // the owner's ray, tree and current best

      const bool obhas = __shfl_sync(kFull, bhas ? 1 : 0, owner) != 0;
      const int ot = (wib << 5) + owner;
      const double obt = LC.bt[ot];
      const int32_t obface = LC.bface[ot];
      const int32_t otid = LC.tid[ot];
      const TreeDev* otree = LC.tree[ot];
      const int32_t* oexcl = LC.excl[ot];
      const int32_t onexcl = LC.nexcl[ot];
      const d3 oo = ray_o(ot), od = ray_d(ot);
      int32_t flags = 0;
      double rt = 0.0;
      int32_t rface = -1, rsurf = -1, rtri = -1;
      if (mine) {
        const double* op64 = otree->prim64;
        const int32_t* opref = otree->prim_ref;
        // the mixed path reads the triangle's ray-independent FP64 terms
        // (edges, edge normals, face normal) and its vertices from one
        // record per triangle; the all-FP64 path computes the terms from the
        // vertices, as the reference does
        const double* pe = nullptr;
        const double* pv = op64 + kPrim64Stride * (int64_t)prim;
        if (MIXED && a.prim_edges && a.tri_prime) {
          pe = a.tri_prime + kTriPrimeStride * (int64_t)__ldg(&opref[prim]);
          pv = pe + 22;
        }
        d3 v0 = mk3(0, 0, 0), v1 = v0, v2 = v0;
        const d3 rn = cross3(od, oo);  // plucker.h:75
        double t;
        const double tmax = (MODE == MODE_OCCLUDED) ? INFTY : obt;
        bool hit;
        if (pe) {
          const double c0 = plucker_edge_oriented(pe, od, rn);
          const double c1 = plucker_edge_oriented(pe + 6, od, rn);
          const double c2 = plucker_edge_oriented(pe + 12, od, rn);
          const int idx = plucker_axis(od);
          hit = plucker64_coords(c0, c1, c2, __ldg(&pv[idx]), __ldg(&pv[3 + idx]),
                                 __ldg(&pv[6 + idx]), comp3(oo, idx), comp3(od, idx), tmax, 0.0,
                                 false, 0, &t);
        } else {
          load_tri64(pv, v0, v1, v2);
          hit = plucker64(v0, v1, v2, oo, od, rn, tmax, 0.0, false, 0, &t);
        }
        if (hit) {
          if (MODE == MODE_OCCLUDED) {
            flags = 1;
          } else if (!dlt(obt, t)) {  // triangle_intersect.cpp:78: t > dtfar rejects
            const int32_t gtri = __ldg(&opref[prim]);
            const int32_t fid = __ldg(&a.tri_face[gtri]);
            if (!(obhas && okey(t) == okey(obt) && fid >= obface)) {
              // sign of dot(d, normal), normal flipped in the surface's
              // reverse-sense tree (:80, :84-87)
              const int32_t sidx = __ldg(&a.tri_surf[gtri]);
              int sg;
              if (pe) {
                const double2 cxy = __ldg(reinterpret_cast<const double2*>(pe + 18));
                sg = normal_dot_sign_c(od, mk3(cxy.x, cxy.y, __ldg(&pe[20])));
              } else {
                sg = normal_dot_sign(od, v0, v1, v2);
              }
              if (__ldg(&a.surf_rev_tree[sidx]) == otid) sg = -sg;
              bool keep = true;
              if (MODE == MODE_RAY_FIRE || MODE == MODE_PARTICLE) {  // orientation_cull, :12-24
                if (a.orientation == 0 && sg < 0) keep = false;   // dot < 0
                if (a.orientation == 1 && sg >= 0) keep = false;  // dot >= 0
              }
              for (int32_t k = 0; keep && k < onexcl; ++k)  // primitive_mask_cull, :26-34
                if (__ldg(&oexcl[k]) == fid) keep = false;
              if (keep) {
                flags = 1 | (sg > 0 ? 2 : 0);
                rt = t;
                rface = fid;
                rsurf = __ldg(&a.surf_id[sidx]);
                rtri = gtri;
              }
            }
          }
        }
      }
      Q.rflags[lane] = flags;
      Q.rt[lane] = rt;
      Q.rface[lane] = rface;
      Q.rsurf[lane] = rsurf;
      if (MODE == MODE_PARTICLE) Q.rtri[lane] = rtri;
      const int my_owner = owner;
      __syncwarp();
      // each ray merges its own results in queue order
      bool changed = false;
      for (int j = 0; j < nq; ++j) {
        if (__shfl_sync(kFull, my_owner, j) != lane) continue;
        npend--;
        const int32_t fl = Q.rflags[j];
        if (!(fl & 1)) continue;
        if (MODE == MODE_OCCLUDED) {
          bhas = true;
          trav = false;
          continue;
        }
        const double t = Q.rt[j];
        const int32_t f = Q.rface[j];
        const long long kt = okey(t), kb = okey(bt);
        if (!bhas || kt < kb || (kt == kb && f < bface)) {
          bhas = true;
          bt = t;
          bface = f;
          bsurf = Q.rsurf[j];
          if (MODE == MODE_PARTICLE) btri = Q.rtri[j];
          bdot = (fl & 2) != 0;
          changed = true;
        }
      }
      if (changed) bt32 = f32_up(bt);
      __syncwarp();
      if (lane == 0) Q.head = head + (uint32_t)nq;
      __syncwarp();
    }
  }
  if (a.counters) {
    // rays_done is per lane; flush_counters sums lanes
    flush_counters(a.counters, cnt, rays_done);
  }
}

// resident blocks per SM, by kernel variant, MINB and stack depth (8..64
// step 8), per device, and whether the variant's shared-memory limit is
// raised on a device; filled on first use, from any host thread
std::atomic<int> g_blocks_per_sm[12][3][kTStackMax / 8 + 1][kMaxDevices];
std::atomic<bool> g_smem_attr[12][3][kMaxDevices];

template <int MODE, bool MIXED, int MINB>
cudaError_t launch_minb(const SurfArgs& a, cudaStream_t st, int slot) {
  if (a.stack < kTStackMin || a.stack > kTStackMax || a.stack % 8 != 0) return cudaErrorInvalidValue;
  if (a.grab > 0 && (a.work == nullptr || a.grab % 32 != 0)) return cudaErrorInvalidValue;
  constexpr bool keys = stack_keys<MODE, MIXED>();
  const size_t smem = trace_smem_bytes(a.stack, keys, MODE == MODE_PARTICLE && MIXED);
  auto kern = k_trace<MODE, MIXED, MINB>;
  const int dev = current_device();
  const bool known = dev >= 0 && dev < kMaxDevices;
  if (!known || !g_smem_attr[slot][MINB - 2][dev].load(std::memory_order_acquire)) {
    cudaError_t e = cudaFuncSetAttribute(
        kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
        (int)trace_smem_bytes(kTStackMax, keys, MODE == MODE_PARTICLE && MIXED));
    if (e != cudaSuccess) return e;
    if (known) g_smem_attr[slot][MINB - 2][dev].store(true, std::memory_order_release);
  }
  int per_sm = 0;
  {
    const cudaError_t e =
        occupancy_cached(g_blocks_per_sm[slot][MINB - 2][a.stack / 8], kern, kTBlock, smem, per_sm);
    if (e != cudaSuccess) return e;
  }
  const int64_t warps_needed = (a.n + 31) / 32;
  int64_t blocks = (int64_t)device_sm_count() * per_sm;
  const int64_t max_blocks = (warps_needed + kTWarps - 1) / kTWarps;
  if (blocks > max_blocks) blocks = max_blocks;
  if (blocks < 1) blocks = 1;
  const int64_t warps = blocks * kTWarps;
  const int64_t chunk = a.grab > 0 ? 0 : (a.n + warps - 1) / warps;
  kern<<<(unsigned)blocks, kTBlock, smem, st>>>(a, chunk);
  return cudaGetLastError();
}

template <int MODE, bool MIXED>
cudaError_t launch_one(const SurfArgs& a, cudaStream_t st, int slot) {
  switch (a.occupancy) {
    case 2: return launch_minb<MODE, MIXED, 2>(a, st, slot);
    case 4: return launch_minb<MODE, MIXED, 4>(a, st, slot);
    default: return launch_minb<MODE, MIXED, 3>(a, st, slot);
  }
}

}  // namespace

cudaError_t launch_surface_query(int mode, bool mixed, const SurfArgs& a, cudaStream_t st) {
  if (a.n <= 0) return cudaSuccess;
  switch (mode * 2 + (mixed ? 1 : 0)) {
    case 0: return launch_one<MODE_RAY_FIRE, false>(a, st, 0);
    case 1: return launch_one<MODE_RAY_FIRE, true>(a, st, 1);
    case 2: return launch_one<MODE_PIV, false>(a, st, 2);
    case 3: return launch_one<MODE_PIV, true>(a, st, 3);
    case 4: return launch_one<MODE_OCCLUDED, false>(a, st, 4);
    case 5: return launch_one<MODE_OCCLUDED, true>(a, st, 5);
    case 6: return launch_one<MODE_FIND_VOLUME, false>(a, st, 6);
    case 7: return launch_one<MODE_FIND_VOLUME, true>(a, st, 7);
    case 8: return launch_one<MODE_PARTICLE, false>(a, st, 8);
    case 9: return launch_one<MODE_PARTICLE, true>(a, st, 9);
    case 10: return launch_one<MODE_ALL_VOLUMES, false>(a, st, 10);
    case 11: return launch_one<MODE_ALL_VOLUMES, true>(a, st, 11);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace xdgcu
