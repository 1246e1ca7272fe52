"""Host-side mirror of XDG's RayTracer plugin API and XDG facade over the
CUDA engine (C ABI in include/xdgcu.h).

``CudaRayTracer`` follows xdg::RayTracer (include/xdg/ray_tracing_interface.h:
16-147): register_volume / create_*_tree / ray_fire / point_in_volume /
occluded / closest / find_element, tree ids counted from 1 per kind.  ``XDG``
follows the facade in src/xdg.cpp (prepare_raytracer, per-volume dispatch,
find_volume, segments).  Every query is batched: arrays of n rays in, arrays
out.  NumPy inputs run through the host-staging path of the C ABI; torch CUDA
tensors run on the device without copies, on torch's current stream.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import ANY, ENTERING, EXITING, FP64, MIXED, check  # noqa: F401
from ._lib import (QUERY_FIND_VOLUME, QUERY_OCCLUDED, QUERY_POINT_IN_VOLUME,  # noqa: F401
                   QUERY_RAY_FIRE, BC_REFLECTING, BC_TRANSMISSION, BC_VACUUM)

# keys of xdgcu_set_tuning / xdgcu_get_tuning
TUNING_KEYS = ("trace_occupancy", "trace_node_iters", "trace_node_iters_fp64",
               "trace_flush_wait", "trace_stack", "trace_grab", "trace_sort_min",
               "particle_event_wait", "transport_event_wait", "leaf_max", "node_width",
               "walk_queue", "walk_flush_wait", "walk_sort_min", "walk_edge_table",
               "trace_edge_table", "host_direct", "closest_bound", "bvh_sah", "bvh_prim_cost",
               "closest_node_steps", "closest_node_steps_fp64", "find_node_steps_fp64",
               "segments_walk_cap", "find_element_phased", "packed_walk_passes",
               "closest_step_budget", "scratch_keep_bytes", "closest_sort_min",
               "find_sort_min", "trace_node_iters_direct")

INFTY = np.finfo(np.float64).max
TINY_BIT = 1e-10  # constants.h:32
ID_NONE = -1
TREE_NONE = -1


def _is_torch(x) -> bool:
    return type(x).__module__.startswith("torch")


def _addr(x):
    """Device/host address of an array argument (None stays None)."""
    if x is None:
        return None
    if _is_torch(x):
        return ctypes.c_void_p(x.data_ptr())
    return x.ctypes.data_as(ctypes.c_void_p)


def _host(a, dtype, shape=None):
    a = np.ascontiguousarray(a, dtype=dtype)
    return a.reshape(shape) if shape is not None else a


class _Out:
    """Allocates outputs of the same kind as the inputs: NumPy arrays, torch
    CUDA tensors, or torch CPU tensors (page-locked when the input is, so
    that the kernels write them in place)."""

    def __init__(self, like):
        self.torch = _is_torch(like)
        if self.torch:
            import torch
            self._torch = torch
            self.device = like.device
            self.cuda = like.is_cuda
            self.pin = (not like.is_cuda) and like.is_pinned()

    def empty(self, shape, dtype):
        if self.torch:
            return self._torch.empty(shape, dtype=dtype, device=self.device, pin_memory=self.pin)
        return np.empty(shape, dtype=dtype)

    def zeros(self, shape, dtype):
        if self.torch:
            return self._torch.zeros(shape, dtype=dtype, device=self.device, pin_memory=self.pin)
        return np.zeros(shape, dtype=dtype)

    def f64(self, *shape):
        return self.empty(shape, self._torch.float64 if self.torch else np.float64)

    def i32(self, *shape):
        return self.empty(shape, self._torch.int32 if self.torch else np.int32)

    def stream(self):
        if self.torch and self.cuda:
            return ctypes.c_void_p(self._torch.cuda.current_stream(self.device).cuda_stream)
        return None


def _prep(x, dtype, cols=None):
    if x is None:
        return None
    if _is_torch(x):
        return x.contiguous()
    return _host(x, dtype, (-1, cols) if cols else (-1,))


def _csr(exclude, n, torch_like=None):
    if exclude is None:
        return None, None
    off = np.zeros(n + 1, dtype=np.int32)
    off[1:] = np.cumsum([len(e) for e in exclude])
    ids = (np.concatenate([np.asarray(e, dtype=np.int32) for e in exclude]) if off[-1]
           else np.zeros(1, dtype=np.int32))
    ids = np.ascontiguousarray(ids, dtype=np.int32)
    if torch_like is not None and _is_torch(torch_like):
        import torch
        return (torch.from_numpy(off).to(torch_like.device),
                torch.from_numpy(ids).to(torch_like.device))
    return off, ids


def volume_bounding_box(model, volume):
    """MeshManager::volume_bounding_box (mesh_manager_interface.cpp:236-267).

    Its BoundingBox starts at all zeros (bbox.h:17-25) and is then grown, so
    the box always contains the origin; that quirk is kept.
    """
    lo = np.zeros(3)
    hi = np.zeros(3)
    for s, _ in model.volume_surfaces(volume):
        x = s.vertices[s.triangles.reshape(-1)]
        lo = np.minimum(lo, x.min(0))
        hi = np.maximum(hi, x.max(0))
    return lo, hi


def bounding_box_bump(model, volume, numerical_precision=1e-3):
    """RayTracer::bounding_box_bump (ray_tracing_interface.cpp:20-24)."""
    lo, hi = volume_bounding_box(model, volume)
    w = hi - lo
    chord = np.sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2])
    return max(chord * 1e-6, numerical_precision)


class CudaRayTracer:
    """The CUDA backend behind XDG's RayTracer interface."""

    def __init__(self, device: int = 0):
        self.L = _lib.load()
        h = ctypes.c_void_p()
        rc = self.L.xdgcu_create(ctypes.byref(h), device)
        check(rc, None, "xdgcu_create")
        self.ctx = h
        self.device = device
        self._registered = set()
        self._tets_set = False
        self.global_surface_tree = TREE_NONE
        self.global_element_tree = TREE_NONE
        self.surface_trees = []
        self.element_trees = []

    def close(self):
        if getattr(self, "ctx", None):
            self.L.xdgcu_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc, what):
        check(rc, self.ctx, what)

    def library(self):
        return "CUDA"

    # ---- registration -------------------------------------------------

    def register_surface(self, surface):
        """First-visit registration of a surface (embree/ray_tracer.cpp:107-147)."""
        if surface.surface_id in self._registered:
            return
        xyz = surface.tri_xyz()
        fid = _host(surface.face_ids, np.int32)
        self._check(self.L.xdgcu_register_surface(self.ctx, int(surface.surface_id), len(fid),
                                                   _addr(xyz), _addr(fid)),
                    "register_surface")
        self._registered.add(surface.surface_id)

    def create_surface_tree(self, model, volume):
        """RayTracer::create_surface_tree (embree/ray_tracer.cpp:49-105)."""
        pairs = model.volume_surfaces(volume)
        for s, _ in pairs:
            self.register_surface(s)
        ids = np.array([s.surface_id for s, _ in pairs], dtype=np.int32)
        sense = np.array([sn for _, sn in pairs], dtype=np.int32)
        bump = bounding_box_bump(model, volume)
        tree = ctypes.c_int32(-1)
        self._check(self.L.xdgcu_create_surface_tree(self.ctx, _addr(ids), _addr(sense), len(ids),
                                                      float(bump), ctypes.byref(tree)),
                    "create_surface_tree")
        self.surface_trees.append(tree.value)
        return tree.value

    def set_tet_mesh(self, tets):
        if self._tets_set:
            return
        v = _host(tets.vertices, np.float64, (-1, 3))
        c = _host(tets.conn, np.int32, (-1, 4))
        a = _host(tets.adj, np.int32, (-1, 4))
        ids = _host(tets.elem_ids, np.int32)
        ft = _host(tets.face_table, np.int32, (12,))
        self._check(self.L.xdgcu_set_tet_mesh(self.ctx, len(v), _addr(v), len(c), _addr(c), _addr(a),
                                               _addr(ids), _addr(ft)), "set_tet_mesh")
        self._tets_set = True

    def create_element_tree(self, model, volume):
        """RayTracer::create_element_tree (embree/ray_tracer.cpp:149-188)."""
        elems = model.volume_elements(volume)
        if elems is None or len(elems) == 0:
            return TREE_NONE
        self.set_tet_mesh(model.tets)
        e = _host(elems, np.int32)
        tree = ctypes.c_int32(-1)
        self._check(self.L.xdgcu_create_element_tree(self.ctx, _addr(e), len(e), ctypes.byref(tree)),
                    "create_element_tree")
        self.element_trees.append(tree.value)
        return tree.value

    def register_volume(self, model, volume):
        """RayTracer::register_volume (embree/ray_tracer.cpp:38-47)."""
        return self.create_surface_tree(model, volume), self.create_element_tree(model, volume)

    def create_global_surface_tree(self):
        tree = ctypes.c_int32(-1)
        self._check(self.L.xdgcu_create_global_surface_tree(self.ctx, ctypes.byref(tree)),
                    "create_global_surface_tree")
        self.surface_trees.append(tree.value)
        self.global_surface_tree = tree.value
        return tree.value

    def create_global_element_tree(self):
        tree = ctypes.c_int32(-1)
        self._check(self.L.xdgcu_create_global_element_tree(self.ctx, ctypes.byref(tree)),
                    "create_global_element_tree")
        self.element_trees.append(tree.value)
        self.global_element_tree = tree.value
        return tree.value

    def init(self):
        pass

    def num_registered_trees(self):
        return self.num_registered_surface_trees() + self.num_registered_element_trees()

    def num_registered_surface_trees(self):
        return int(self.L.xdgcu_num_surface_trees(self.ctx))

    def num_registered_element_trees(self):
        return int(self.L.xdgcu_num_element_trees(self.ctx))

    def tree_info(self, tree, element=False):
        out = (ctypes.c_int64 * 8)()
        fn = self.L.xdgcu_element_tree_info if element else self.L.xdgcu_surface_tree_info
        self._check(fn(self.ctx, int(tree), out), "tree_info")
        return dict(nodes=out[0], prims=out[1], depth=out[2], bytes32=out[3], bytes64=out[4],
                    width=out[5])

    def set_tuning(self, key: str, value: int):
        self._check(self.L.xdgcu_set_tuning(self.ctx, key.encode(), int(value)), "set_tuning")

    def get_tuning(self, key: str) -> int:
        v = ctypes.c_int64()
        self._check(self.L.xdgcu_get_tuning(self.ctx, key.encode(), ctypes.byref(v)), "get_tuning")
        return int(v.value)

    def tuning(self) -> dict:
        """Every tuning key with its current value."""
        return {k: self.get_tuning(k) for k in TUNING_KEYS}

    def rebuild_trees(self, kinds=3):
        """xdgcu_rebuild_trees (1 surface, 2 element, 3 both) with the
        current node_width / leaf_max."""
        self._check(self.L.xdgcu_rebuild_trees(self.ctx, int(kinds)), "rebuild_trees")

    def autotune_trace(self, query, tree, origins, dirs=None, precision=MIXED, ray_trees=None,
                       reps=5, tune_tree=True):
        """xdgcu_autotune_trace on a sample batch (torch CUDA tensors).  Leaves
        the context tuned; returns (sample ms under the chosen settings,
        tuning dict)."""
        o = _prep(origins, np.float64, 3)
        d = _prep(dirs, np.float64, 3)
        rt = _prep(ray_trees, np.int32)
        ms = ctypes.c_double()
        self._check(self.L.xdgcu_autotune_trace(self.ctx, int(query), int(tree or 0), _addr(rt),
                                                o.shape[0], _addr(o), _addr(d), int(precision),
                                                int(reps), 1 if tune_tree else 0,
                                                ctypes.byref(ms)), "autotune_trace")
        return ms.value, self.tuning()

    def autotune_walk(self, start_index, start, u, distance, max_segs=256, precision=MIXED,
                      reps=5):
        """xdgcu_autotune_walk on a sample of tracks (torch CUDA tensors)."""
        si = _prep(start_index, np.int32)
        r = _prep(start, np.float64, 3)
        uu = _prep(u, np.float64, 3)
        dist = _prep(distance, np.float64)
        ms = ctypes.c_double()
        self._check(self.L.xdgcu_autotune_walk(self.ctx, si.shape[0], _addr(si), _addr(r),
                                               _addr(uu), _addr(dist), int(max_segs),
                                               int(precision), int(reps), ctypes.byref(ms)),
                    "autotune_walk")
        return ms.value, self.tuning()

    def set_counting(self, on: bool):
        self._check(self.L.xdgcu_set_counting(self.ctx, 1 if on else 0), "set_counting")

    def counters(self):
        out = (ctypes.c_int64 * 8)()
        self._check(self.L.xdgcu_get_counters(self.ctx, out), "get_counters")
        return dict(box=out[0], node=out[1], prim=out[2], escalate=out[3], rays=out[4],
                    steps=out[5])

    # ---- queries ------------------------------------------------------

    def ray_fire(self, tree, origins, dirs, dist_limit=None, orientation=EXITING, exclude=None,
                 precision=MIXED, ray_trees=None, status=False, stream=None):
        """Batched RayTracer::ray_fire.  Returns (t, surface, face[, status]).

        ``exclude`` is a list of per-ray face-id lists (the reference's
        exclude_primitives); the reference appends the hit face to it, which
        the caller can do with the returned face ids."""
        o = _prep(origins, np.float64, 3)
        d = _prep(dirs, np.float64, 3)
        n = o.shape[0]
        dl = None
        if dist_limit is not None:
            dl = dist_limit if _is_torch(dist_limit) else _host(np.broadcast_to(dist_limit, (n,)),
                                                                 np.float64)
        rt = _prep(ray_trees, np.int32)
        eo, ei = _csr(exclude, n, o)
        out = _Out(o)
        t, s, f, st = out.f64(n), out.i32(n), out.i32(n), out.i32(n)
        self._check(self.L.xdgcu_ray_fire(self.ctx, int(tree or 0), _addr(rt), n, _addr(o), _addr(d),
                                          _addr(dl), int(orientation), _addr(eo), _addr(ei),
                                          _addr(t), _addr(s), _addr(f), _addr(st), int(precision),
                                          stream if stream is not None else out.stream()),
                    "ray_fire")
        return (t, s, f, st) if status else (t, s, f)

    def point_in_volume(self, tree, points, dirs=None, exclude=None, precision=MIXED,
                        ray_trees=None, stream=None):
        p = _prep(points, np.float64, 3)
        d = _prep(dirs, np.float64, 3)
        n = p.shape[0]
        rt = _prep(ray_trees, np.int32)
        eo, ei = _csr(exclude, n, p)
        out = _Out(p)
        r = out.i32(n)
        self._check(self.L.xdgcu_point_in_volume(self.ctx, int(tree or 0), _addr(rt), n, _addr(p),
                                                 _addr(d), _addr(eo), _addr(ei), _addr(r), None,
                                                 int(precision),
                                                 stream if stream is not None else out.stream()),
                    "point_in_volume")
        return r

    def point_in_volumes(self, points, trees, dirs=None, precision=MIXED, stream=None):
        """xdgcu_point_in_volumes: (n, len(trees)) uint8 inside flags."""
        p = _prep(points, np.float64, 3)
        d = _prep(dirs, np.float64, 3)
        n = p.shape[0]
        tl = np.ascontiguousarray(trees, dtype=np.int32)
        out = _Out(p)
        res = out.zeros((n, len(tl)), out._torch.uint8 if out.torch else np.uint8)
        self._check(self.L.xdgcu_point_in_volumes(self.ctx, n, _addr(p), _addr(d), len(tl),
                                                  _addr(tl), _addr(res), None, int(precision),
                                                  stream if stream is not None else out.stream()),
                    "point_in_volumes")
        return res

    def set_volume_map(self, volume_ids, surface_trees, implicit_complement):
        """The volumes find_volume tries, in order, and their surface trees."""
        ids = _host(volume_ids, np.int32)
        trees = _host(surface_trees, np.int32)
        self._check(self.L.xdgcu_set_volume_map(self.ctx, len(ids), _addr(ids), _addr(trees),
                                                 int(implicit_complement)), "set_volume_map")

    def find_volume(self, points, dirs=None, precision=MIXED, status=False, stream=None):
        """XDG::find_volume for n points in one launch (volume map order)."""
        p = _prep(points, np.float64, 3)
        d = _prep(dirs, np.float64, 3)
        n = p.shape[0]
        out = _Out(p)
        vol, st = out.i32(n), out.i32(n)
        self._check(self.L.xdgcu_find_volume(self.ctx, n, _addr(p), _addr(d), _addr(vol), _addr(st),
                                             int(precision),
                                             stream if stream is not None else out.stream()),
                    "find_volume")
        return (vol, st) if status else vol

    def occluded(self, tree, origins, dirs, precision=MIXED, ray_trees=None, stream=None):
        o = _prep(origins, np.float64, 3)
        d = _prep(dirs, np.float64, 3)
        n = o.shape[0]
        rt = _prep(ray_trees, np.int32)
        out = _Out(o)
        occ, dist = out.i32(n), out.f64(n)
        self._check(self.L.xdgcu_occluded(self.ctx, int(tree or 0), _addr(rt), n, _addr(o), _addr(d),
                                          _addr(occ), _addr(dist), None, int(precision),
                                          stream if stream is not None else out.stream()),
                    "occluded")
        return occ, dist

    def closest(self, tree, points, precision=MIXED, ray_trees=None, stream=None):
        p = _prep(points, np.float64, 3)
        n = p.shape[0]
        rt = _prep(ray_trees, np.int32)
        out = _Out(p)
        dist, face = out.f64(n), out.i32(n)
        self._check(self.L.xdgcu_closest(self.ctx, int(tree or 0), _addr(rt), n, _addr(p),
                                         _addr(dist), _addr(face), None, int(precision),
                                         stream if stream is not None else out.stream()),
                    "closest")
        return dist, face

    def find_element(self, tree, points, precision=MIXED, ray_trees=None, stream=None):
        """Returns (element mesh id, tet index); tree None -> global tree."""
        if tree is None:
            tree = self.global_element_tree
        p = _prep(points, np.float64, 3)
        n = p.shape[0]
        rt = _prep(ray_trees, np.int32)
        out = _Out(p)
        eid, eidx = out.i32(n), out.i32(n)
        self._check(self.L.xdgcu_find_element(self.ctx, int(tree or 0), _addr(rt), n, _addr(p),
                                              _addr(eid), _addr(eidx), None, int(precision),
                                              stream if stream is not None else out.stream()),
                    "find_element")
        return eid, eidx

    def next_element(self, elem_index, positions, dirs, precision=MIXED, stream=None):
        e = _prep(elem_index, np.int32)
        r = _prep(positions, np.float64, 3)
        u = _prep(dirs, np.float64, 3)
        n = r.shape[0]
        out = _Out(r)
        nxt, dist, st = out.i32(n), out.f64(n), out.i32(n)
        self._check(self.L.xdgcu_next_element(self.ctx, n, _addr(e), _addr(r), _addr(u), _addr(nxt),
                                              _addr(dist), _addr(st), int(precision),
                                              stream if stream is not None else out.stream()),
                    "next_element")
        return nxt, dist, st

    def walk_elements(self, start_index, start, u, distance, max_segs=256, precision=MIXED,
                      stream=None):
        """Returns (seg_elem [n, max_segs], seg_len, seg_count, status)."""
        e = _prep(start_index, np.int32)
        r = _prep(start, np.float64, 3)
        uu = _prep(u, np.float64, 3)
        n = r.shape[0]
        dist = distance if _is_torch(distance) else _host(np.broadcast_to(distance, (n,)),
                                                           np.float64)
        out = _Out(r)
        se, sl, sc, st = out.i32(n, max_segs), out.f64(n, max_segs), out.i32(n), out.i32(n)
        self._check(self.L.xdgcu_walk_elements(self.ctx, n, _addr(e), _addr(r), _addr(uu),
                                               _addr(dist), int(max_segs), _addr(se), _addr(sl),
                                               _addr(sc), _addr(st), int(precision),
                                               stream if stream is not None else out.stream()),
                    "walk_elements")
        return se, sl, sc, st


    def seed_streams(self, seed, n):
        """xdgcu_seed_streams: n independent random-stream states (uint64)."""
        st = np.zeros(int(n), dtype=np.uint64)
        self._check(self.L.xdgcu_seed_streams(ctypes.c_uint64(int(seed) & (2**64 - 1)), int(n),
                                              _addr(st)), "seed_streams")
        return st

    def transport_elements(self, elem_index, pos, dirs, rng, mfp, max_events, distance, events,
                           tally=None, precision=MIXED, stream=None):
        """xdgcu_transport_elements: updates the particle state in place
        (torch CUDA tensors or NumPy arrays; rng as int64/uint64 bits).
        Returns the per-particle status array."""
        n = len(elem_index)
        out = _Out(pos)
        st = out.i32(n)
        self._check(self.L.xdgcu_transport_elements(
            self.ctx, n, _addr(elem_index), _addr(pos), _addr(dirs), _addr(rng), float(mfp),
            int(max_events), _addr(distance), _addr(events), _addr(tally), _addr(st),
            int(precision), stream if stream is not None else out.stream()), "transport_elements")
        return st

    def set_surface_boundary(self, conditions: dict):
        """xdgcu_set_surface_boundary: {surface id: BC_TRANSMISSION /
        BC_VACUUM / BC_REFLECTING}."""
        ids = np.array(list(conditions.keys()), dtype=np.int32)
        bc = np.array([conditions[k] for k in conditions], dtype=np.int32)
        self._check(self.L.xdgcu_set_surface_boundary(self.ctx, len(ids), _addr(ids), _addr(bc)),
                    "set_surface_boundary")

    def transport_surfaces(self, tree, pos, dirs, rng, mfp, max_events, history, history_count,
                           distance, events, tally=None, graveyard_tree=0, precision=MIXED,
                           stream=None):
        """xdgcu_transport_surfaces: updates the particle state in place
        (torch CUDA tensors or NumPy arrays).  ``history`` is n x cap.
        Returns the per-particle status array."""
        n = len(tree)
        out = _Out(pos)
        st = out.i32(n)
        cap = int(history.shape[1])
        self._check(self.L.xdgcu_transport_surfaces(
            self.ctx, n, _addr(tree), _addr(pos), _addr(dirs), _addr(rng), float(mfp),
            int(max_events), int(graveyard_tree), cap, _addr(history), _addr(history_count),
            _addr(distance), _addr(events), _addr(tally), _addr(st), int(precision),
            stream if stream is not None else out.stream()), "transport_surfaces")
        return st

    def walk_elements_packed(self, start_index, start, u, distance, capacity, max_segs=4096,
                             precision=MIXED, stream=None):
        """Packed walk: returns (seg_elem [capacity], seg_len, offsets [n+1], status)."""
        e = _prep(start_index, np.int32)
        r = _prep(start, np.float64, 3)
        uu = _prep(u, np.float64, 3)
        n = r.shape[0]
        dist = distance if _is_torch(distance) else _host(np.broadcast_to(distance, (n,)),
                                                           np.float64)
        out = _Out(r)
        se, sl, st = out.i32(max(1, capacity)), out.f64(max(1, capacity)), out.i32(n)
        off = out.empty(n + 1, out._torch.int64 if out.torch else np.int64)
        self._check(self.L.xdgcu_walk_elements_packed(self.ctx, n, _addr(e), _addr(r), _addr(uu),
                                                      _addr(dist), int(max_segs), int(capacity),
                                                      _addr(se), _addr(sl), _addr(off), _addr(st),
                                                      int(precision),
                                                      stream if stream is not None else out.stream()),
                    "walk_elements_packed")
        return se, sl, off, st


    def set_boundary_face_elements(self, face_ids, elem_index):
        """MeshManager::get_boundary_face_element for the global track loop:
        face mesh id -> tet index behind it (-1: none)."""
        f = _host(face_ids, np.int32)
        e = _host(elem_index, np.int32)
        self._check(self.L.xdgcu_set_boundary_face_elements(self.ctx, len(f), _addr(f), _addr(e)),
                    "set_boundary_face_elements")

    def segments_global(self, ipc_tree, element_tree, starts, ends, capacity, max_segs=4096,
                        max_rounds=10_000, precision=MIXED, stream=None):
        """xdgcu_segments_global: XDG::segments(start, end) for n tracks on the
        device.  Returns (seg_elem [capacity], seg_len, offsets [n+1], status)."""
        s = _prep(starts, np.float64, 3)
        e = _prep(ends, np.float64, 3)
        n = s.shape[0]
        out = _Out(s)
        se, sl, st = out.i32(max(1, capacity)), out.f64(max(1, capacity)), out.i32(n)
        off = out.empty(n + 1, out._torch.int64 if out.torch else np.int64)
        self._check(self.L.xdgcu_segments_global(self.ctx, int(ipc_tree), int(element_tree), n,
                                                 _addr(s), _addr(e), int(max_segs), int(max_rounds),
                                                 int(capacity), _addr(se), _addr(sl), _addr(off),
                                                 _addr(st), int(precision),
                                                 stream if stream is not None else out.stream()),
                    "segments_global")
        return se, sl, off, st


class XDG:
    """The XDG facade (src/xdg.cpp) over a model and the CUDA ray tracer."""

    def __init__(self, model, device: int = 0, ray_tracer: CudaRayTracer | None = None):
        self.model = model
        self.rti = ray_tracer or CudaRayTracer(device)
        self.volume_to_surface_tree = {}
        self.volume_to_point_location_tree = {}
        self._volume_map_set = False

    def ray_tracing_interface(self):
        return self.rti

    def prepare_volume_for_raytracing(self, volume):
        self._volume_map_set = False
        st, et = self.rti.register_volume(self.model, volume)
        self.volume_to_surface_tree[volume] = st
        self.volume_to_point_location_tree[volume] = et

    def prepare_raytracer(self):
        """xdg.cpp:37-47; also hands the engine the mesh's boundary-face
        elements (MeshManager::get_boundary_face_element) for the global
        track loop."""
        for v in self.model.volumes:
            self.prepare_volume_for_raytracing(v)
        self.rti.create_global_element_tree()
        self.rti.create_global_surface_tree()
        self.rti.init()
        bfe = self.model.boundary_face_element
        if bfe is not None and self.model.tets is not None and len(bfe):
            bfe = np.asarray(bfe, dtype=np.int32)
            self.rti.set_boundary_face_elements(np.arange(len(bfe), dtype=np.int32), bfe)

    def _trees(self, volumes):
        """Surface tree of each ray's volume (NumPy, or a torch tensor on the
        volumes' device)."""
        lut = np.full(max(self.volume_to_surface_tree) + 1, TREE_NONE, dtype=np.int32)
        for v, t in self.volume_to_surface_tree.items():
            lut[v] = t
        if _is_torch(volumes):
            import torch
            vt = volumes.reshape(-1).long()
            if len(vt) and (int(vt.min()) < 0 or int(vt.max()) >= len(lut)):
                raise KeyError("volume without a surface tree")
            out = torch.from_numpy(lut).to(volumes.device)[vt]
        else:
            v = np.asarray(volumes).reshape(-1)
            if len(v) and (v.min() < 0 or v.max() >= len(lut)):
                raise KeyError("volume without a surface tree")
            out = lut[v]
        if len(out) and int((out == TREE_NONE).sum()) > 0:
            raise KeyError("volume without a surface tree")
        return out

    def ray_fire(self, volume, origins, dirs, dist_limit=None, orientation=EXITING, exclude=None,
                 precision=MIXED):
        """xdg.cpp:237-247 (volume may be one id or one per ray)."""
        if np.ndim(volume) == 0:
            return self.rti.ray_fire(self.volume_to_surface_tree[int(volume)], origins, dirs,
                                     dist_limit, orientation, exclude, precision)
        return self.rti.ray_fire(0, origins, dirs, dist_limit, orientation, exclude, precision,
                                 ray_trees=self._trees(volume))

    def point_in_volume(self, volume, points, dirs=None, exclude=None, precision=MIXED):
        """xdg.cpp:104-111."""
        if np.ndim(volume) == 0:
            return self.rti.point_in_volume(self.volume_to_surface_tree[int(volume)], points, dirs,
                                            exclude, precision)
        return self.rti.point_in_volume(0, points, dirs, exclude, precision,
                                        ray_trees=self._trees(volume))

    def find_volume(self, points, dirs, precision=MIXED):
        """xdg.cpp:113-128: first non-implicit-complement volume whose
        point_in_volume is true, else the implicit complement.  Volumes are
        tried in ascending id order, all of them in one fused launch."""
        if not self._volume_map_set:
            vols = sorted(self.volume_to_surface_tree)
            self.rti.set_volume_map(vols, [self.volume_to_surface_tree[v] for v in vols],
                                    self.model.implicit_complement)
            self._volume_map_set = True
        return self.rti.find_volume(points, dirs, precision)

    def find_volume_per_volume(self, points, dirs, precision=MIXED):
        """find_volume as one point_in_volume launch per volume on the points
        not yet placed (the unfused form, for comparison)."""
        p = _host(points, np.float64, (-1, 3))
        d = _host(dirs, np.float64, (-1, 3))
        ipc = self.model.implicit_complement
        out = np.full(len(p), ipc, dtype=np.int32)
        todo = np.arange(len(p))
        for v in sorted(self.volume_to_surface_tree):
            if v == ipc or len(todo) == 0:
                continue
            inside = self.point_in_volume(v, p[todo], d[todo], precision=precision).astype(bool)
            out[todo[inside]] = v
            todo = todo[~inside]
        return out

    def find_element(self, points, volume=None, precision=MIXED):
        """xdg.cpp:130-140 (global tree when volume is None)."""
        tree = None if volume is None else self.volume_to_point_location_tree[int(volume)]
        return self.rti.find_element(tree, points, precision)

    def closest(self, volume, points, precision=MIXED):
        """xdg.cpp:249-254."""
        return self.rti.closest(self.volume_to_surface_tree[int(volume)], points, precision)

    def occluded(self, volume, origins, dirs, precision=MIXED):
        """xdg.cpp:263-270."""
        return self.rti.occluded(self.volume_to_surface_tree[int(volume)], origins, dirs, precision)

    def next_element(self, elem_index, r, u, precision=MIXED):
        return self.rti.next_element(elem_index, r, u, precision)

    def segments(self, volume, starts, ends, max_segs=1024, precision=MIXED):
        """XDG::segments(volume, start, end) (xdg.cpp:200-227) for n tracks.

        Returns a list of (element ids, lengths) per track."""
        s = _host(starts, np.float64, (-1, 3))
        e = _host(ends, np.float64, (-1, 3))
        n = len(s)
        tree = self.volume_to_point_location_tree[int(volume)]
        u = _normalize_rows(e - s)
        start_copy = s.copy()
        eid, eidx = self.rti.find_element(tree, s, precision)
        eidx = eidx.copy()
        miss = np.nonzero(eidx < 0)[0]
        valid = np.ones(n, dtype=bool)
        if len(miss):
            t, surf, _ = self.ray_fire(volume, s[miss], u[miss], None, ENTERING,
                                       precision=precision)
            hit = surf != ID_NONE
            valid[miss[~hit]] = False
            m = miss[hit]
            th = t[hit]
            nudged = s[m] + u[m] * (th + TINY_BIT)[:, None]
            _, idx2 = self.rti.find_element(tree, nudged, precision)
            valid[m[idx2 < 0]] = False
            eidx[m] = idx2
            start_copy[m] = s[m] + u[m] * th[:, None]
        # walk_elements(start, end) overload (mesh_manager_interface.cpp:138-147)
        w = e - start_copy
        dist = np.sqrt(w[:, 0] * w[:, 0] + w[:, 1] * w[:, 1] + w[:, 2] * w[:, 2])
        uw = _normalize_rows(w)
        idx = np.nonzero(valid)[0]
        out = [(np.zeros(0, dtype=np.int32), np.zeros(0)) for _ in range(n)]
        if len(idx):
            se, sl, sc, st = self.rti.walk_elements(eidx[idx], start_copy[idx], uw[idx], dist[idx],
                                                    max_segs, precision)
            for k, i in enumerate(idx):
                out[i] = (se[k, :sc[k]].copy(), sl[k, :sc[k]].copy())
        return out


    def segments_global(self, starts, ends, precision=MIXED, max_rounds=10_000, max_segs=4096):
        """XDG::segments(start, end) (xdg.cpp:142-198) for n tracks: walks the
        tet mesh from element to element and, where the track leaves the mesh,
        fires a ray in the implicit complement to the next boundary face and
        re-enters through the element behind it
        (MeshManager::get_boundary_face_element).  One device call
        (xdgcu_segments_global) runs every round of every track.  Returns
        (elements, lengths, offsets): the segments of track i are
        [offsets[i], offsets[i+1]); device arrays for CUDA tensor inputs."""
        ipc_tree = self.volume_to_surface_tree[self.model.implicit_complement]
        gtree = self.rti.global_element_tree
        n = len(starts)
        cap = max(1024, 64 * n)
        args = (ipc_tree, gtree, starts, ends)
        se, sl, off, st = self.rti.segments_global(*args, cap, max_segs, max_rounds, precision)
        total = int(off[-1])
        if total > cap:
            se, sl, off, st = self.rti.segments_global(*args, total, max_segs, max_rounds,
                                                       precision)
        return se[:total], sl[:total], off

    def walk_particles(self, elem_index, pos, dirs, rng, mfp=1.0, max_events=1_000_000,
                       precision=MIXED, tally=False, max_reentries=64):
        """The walk_elements tool loop (tools/walk_elements.h:60-96) for
        particles starting in tets ``elem_index`` (tet indices) at ``pos``
        along ``dirs``, with per-particle random streams ``rng``.

        Every in-mesh event of every particle runs in device launches of
        xdgcu_transport_elements; a particle that leaves the mesh looks for
        re-entry as the tool does -- ray_fire in the implicit complement
        (EXITING, excluding the faces this search hit), move to the hit,
        find_element(r + u*TINY_BIT) -- and, when it finds an element, goes
        back to the device loop.  Returns a dict of NumPy arrays: elem (final
        tet, -1 outside), pos, dir, rng, distance, events, status; and
        tally (track length per tet) when asked for."""
        import torch
        dev = torch.device("cuda", self.rti.device)
        n = len(elem_index)
        e = torch.as_tensor(np.ascontiguousarray(elem_index, dtype=np.int32), device=dev)
        r = torch.as_tensor(_host(pos, np.float64, (-1, 3)), device=dev).contiguous()
        u = torch.as_tensor(_host(dirs, np.float64, (-1, 3)), device=dev).contiguous()
        s = torch.as_tensor(np.ascontiguousarray(rng, dtype=np.uint64).view(np.int64),
                            device=dev).contiguous()
        d = torch.zeros(n, dtype=torch.float64, device=dev)
        ev = torch.zeros(n, dtype=torch.int32, device=dev)
        ty = torch.zeros(len(self.model.tets.conn), dtype=torch.float64, device=dev) if tally \
            else None
        ipc_tree = self.volume_to_surface_tree[self.model.implicit_complement]
        gtree = self.rti.global_element_tree
        final = np.zeros(n, dtype=np.int32)
        ended = np.asarray(elem_index) < 0  # outside the mesh with no re-entry left
        for _ in range(max_reentries + 1):
            st = self.rti.transport_elements(e, r, u, s, mfp, max_events, d, ev, ty, precision)
            torch.cuda.synchronize(dev)
            final = st.cpu().numpy()
            # particles that left the mesh in this launch
            out = np.nonzero((e.cpu().numpy() < 0) & (final == 0) & ~ended)[0]
            if len(out) == 0:
                break
            idx = torch.as_tensor(out, device=dev)
            rr, uu, dd = r[idx].cpu().numpy(), u[idx].cpu().numpy(), d[idx].cpu().numpy()
            ee = np.full(len(out), -1, dtype=np.int32)
            excl = [[] for _ in range(len(out))]
            pend = np.arange(len(out))
            while len(pend):
                t, surf, face = self.rti.ray_fire(ipc_tree, rr[pend], uu[pend], None, EXITING,
                                                  [excl[k] for k in pend], precision)
                hit = surf != ID_NONE
                pend = pend[hit]
                if len(pend) == 0:
                    break
                th = t[hit]
                rr[pend] = rr[pend] + uu[pend] * th[:, None]   # r += u * ray_hit.first
                dd[pend] = dd[pend] + th
                for k, f in zip(pend, face[hit]):
                    excl[k].append(int(f))
                _, eidx = self.rti.find_element(gtree, rr[pend] + uu[pend] * TINY_BIT, precision)
                ee[pend] = eidx
                pend = pend[(eidx < 0) & np.array([len(excl[k]) < 64 for k in pend], dtype=bool)]
            r[idx] = torch.as_tensor(rr, device=dev)
            d[idx] = torch.as_tensor(dd, device=dev)
            e[idx] = torch.as_tensor(ee, device=dev)
            ended[out[ee < 0]] = True
            if (ee < 0).all():
                break
        res = dict(elem=e.cpu().numpy(), pos=r.cpu().numpy(), dir=u.cpu().numpy(),
                   rng=s.cpu().numpy().view(np.uint64), distance=d.cpu().numpy(),
                   events=ev.cpu().numpy(), status=final)
        if tally:
            res["tally"] = ty.cpu().numpy()
        return res

    def simulate_particles(self, volumes, pos, dirs, rng, mfp=1.0, max_events=1_000_000,
                           ipc_graveyard=False, precision=MIXED, history_cap=16, tally=False):
        """The particle_sim tool loop (tools/particle_sim.h:128-141) for
        particles in ``volumes`` (one volume id per particle) at ``pos`` along
        ``dirs`` with per-particle streams ``rng``, every event on the device
        (xdgcu_transport_surfaces).  Boundary conditions come from
        CudaRayTracer.set_surface_boundary.  Returns a dict of NumPy arrays:
        volume (ID_NONE once a particle left through the graveyard or had no
        next volume), pos, dir, rng, distance, events, status and, when asked
        for, tally (path length per volume id, the tool's cell_tracks)."""
        n = len(pos)
        tree = self._trees(np.asarray(volumes)).astype(np.int32)
        r = _host(pos, np.float64, (-1, 3)).copy()
        u = _host(dirs, np.float64, (-1, 3)).copy()
        s = np.ascontiguousarray(rng, dtype=np.uint64).copy()
        hist = np.zeros((n, history_cap), dtype=np.int32)
        hc = np.zeros(n, dtype=np.int32)
        d = np.zeros(n)
        ev = np.zeros(n, dtype=np.int32)
        ty = np.zeros(self.rti.num_registered_surface_trees() + 1) if tally else None
        grave = self.volume_to_surface_tree[self.model.implicit_complement] if ipc_graveyard else 0
        st = self.rti.transport_surfaces(tree, r, u, s, mfp, max_events, hist, hc, d, ev, ty,
                                         grave, precision)
        vol_of = {t: v for v, t in self.volume_to_surface_tree.items()}
        res = dict(volume=np.array([vol_of.get(int(t), ID_NONE) for t in tree], dtype=np.int32),
                   tree=tree, pos=r, dir=u, rng=s, distance=d, events=ev, status=st)
        if tally:
            res["tally"] = {v: ty[t] for v, t in self.volume_to_surface_tree.items()}
        return res

    def check_overlaps(self, check_edges=False, precision=MIXED, max_batch=4_000_000):
        """The overlap_check tool (tools/overlap.cpp:62-191) with every
        point_in_volume / ray_fire of a stage in one batch.

        Vertex check: every vertex of every face of every surface, moved
        1e-9 along dir = normalize(0.1, 0.1, 0.1) and then 2e-9 back along
        -dir, is tested in every volume (the implicit complement included)
        with that direction; a point inside more than one volume is an
        overlap.  Edge check (check_edges): a ray along each face edge, as
        long as the edge, is fired in every volume that is not a parent of
        the edge's surface; the first of those volumes (in volume order) with
        a hit reports {forward volume of the hit surface, forward volume of
        the edge's surface}.  Returns {frozenset(volume ids): location}; of
        the locations that found a set the first one (vertex order, then
        edge order) is kept, where the reference keeps whichever its threads
        wrote last."""
        import torch
        dev = torch.device("cuda", self.rti.device)
        vols = list(self.model.volumes)
        trees = np.array([self.volume_to_surface_tree[v] for v in vols], dtype=np.int32)
        # the arithmetic below runs elementwise on the device, one IEEE
        # operation per step as in the reference's Vec3da expressions
        verts = torch.from_numpy(
            np.concatenate([s.tri_xyz().reshape(-1, 3) for s in self.model.surfaces])).to(dev)
        d = torch.from_numpy(_normalize_rows(np.array([[0.1, 0.1, 0.1]]))[0]).to(dev)
        bump = 1e-9
        loc1 = verts + d * bump                    # loc += dir * bump
        d2 = -d                                    # dir *= -1
        loc2 = loc1 + (d2 * 2.0) * bump            # loc += dir * 2.0 * bump
        found = {}
        n = len(verts)
        step = max(1, max_batch // max(1, 2 * len(vols)))
        for k0 in range(0, n, step):
            k1 = min(n, k0 + step)
            pts = torch.empty((2 * (k1 - k0), 3), dtype=torch.float64, device=dev)
            pts[0::2] = loc1[k0:k1]
            pts[1::2] = loc2[k0:k1]
            dirs = torch.empty_like(pts)
            dirs[0::2] = d
            dirs[1::2] = d2
            inside = self.rti.point_in_volumes(pts, trees, dirs, precision)
            multi = torch.nonzero(inside.sum(1) > 1).flatten()
            if multi.numel() == 0:
                continue
            rows = inside[multi].cpu().numpy()
            locs = pts[multi].cpu().numpy()
            for j in range(len(rows)):
                key = frozenset(vols[m] for m in np.nonzero(rows[j])[0])
                found.setdefault(key, locs[j].copy())
        if not check_edges:
            return found
        parents = {s.surface_id: (s.forward_volume, s.reverse_volume) for s in self.model.surfaces}
        for s in self.model.surfaces:
            pf, pr = parents[s.surface_id]
            check = [v for v in vols if v != pf and v != pr]
            if not check:
                continue
            tri = torch.from_numpy(s.tri_xyz().reshape(-1, 3, 3)).to(dev)
            v1 = tri.reshape(-1, 3)
            v2 = tri[:, [1, 2, 0], :].reshape(-1, 3)
            dv = v2 - v1
            ln = torch.sqrt(dv[:, 0] * dv[:, 0] + dv[:, 1] * dv[:, 1] + dv[:, 2] * dv[:, 2])
            dv = dv / ln[:, None]                   # dir /= edgeLength
            ne, nv = len(v1), len(check)
            ctrees = torch.tensor([self.volume_to_surface_tree[v] for v in check],
                                  dtype=torch.int32, device=dev)
            estep = max(1, max_batch // nv)
            for e0 in range(0, ne, estep):
                e1 = min(ne, e0 + estep)
                m = e1 - e0
                o = torch.repeat_interleave(v1[e0:e1], nv, dim=0)
                dd = torch.repeat_interleave(dv[e0:e1], nv, dim=0)
                dl = torch.repeat_interleave(ln[e0:e1], nv)
                rt = ctrees.repeat(m)
                t, surf, face = self.rti.ray_fire(0, o, dd, dl, EXITING, None, precision,
                                                  ray_trees=rt)
                hit = (surf != ID_NONE).reshape(m, nv)
                edges = torch.nonzero(hit.any(1)).flatten()
                if edges.numel() == 0:
                    continue
                first = torch.argmax(hit[edges].to(torch.int32), dim=1)  # first volume with a hit
                r = (edges * nv + first).cpu().numpy()
                sh_all, o_h = surf[r].cpu().numpy(), o[r].cpu().numpy()
                d_h, t_h = dd[r].cpu().numpy(), t[r].cpu().numpy()
                for j in range(len(r)):
                    org, dirv, th = o_h[j], d_h[j], t_h[j]
                    loc = np.array([org[0] + th * dirv[0], org[1] + th * dirv[1],
                                    org[2] + th * dirv[2]])
                    found.setdefault(frozenset({parents[int(sh_all[j])][0], pf}), loc)
        return found


def _normalize_rows(v):
    """Vec3da::normalize (vec3da.h:61-66), row-wise."""
    min_rcp = float(np.float32(np.float64(np.finfo(np.float32).tiny) * 1e5))
    ln = np.sqrt(v[:, 0] * v[:, 0] + v[:, 1] * v[:, 1] + v[:, 2] * v[:, 2])
    ln = np.where(ln < min_rcp, min_rcp, ln)
    return v / ln[:, None]
