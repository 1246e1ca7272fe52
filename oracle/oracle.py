"""ctypes wrapper of the CPU oracle (oracle/xdg_oracle.c) and of the
reference harness (oracle/ref_harness.cpp -> oracle/_ref/libxdg_ref.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
cpu_baseline leg of bench.py, never by the product package.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libxdg_oracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libxdg_ref.so")

INFTY = np.finfo(np.float64).max
ANY, EXITING, ENTERING = -1, 0, 1
OK, WALK_LIMIT, NO_EXIT_FACE = 0, 4, 5

_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int32)
_U8 = ctypes.POINTER(ctypes.c_uint8)
_VP = ctypes.c_void_p
_i64 = ctypes.c_int64
_i32 = ctypes.c_int32
_int = ctypes.c_int
_dbl = ctypes.c_double

_lib = None
_ref = None


def build(force: bool = False) -> None:
    """Compile the oracle with its Makefile (and the reference harness when the
    reference tree is present)."""
    if force or not os.path.exists(LIB_PATH):
        subprocess.run(["make", "-s", "-C", HERE], check=True)


REF_ENV = "XDG_REFERENCE_DIR"   # the reference source tree, when it is present


REF_DIR_NOTE = os.path.join(HERE, "_ref", "reference_dir")


def reference_dir():
    """The reference source tree: $XDG_REFERENCE_DIR, else the tree the last
    build_ref() compiled from (recorded in oracle/_ref), else None."""
    d = os.environ.get(REF_ENV)
    if not d and os.path.exists(REF_DIR_NOTE):
        with open(REF_DIR_NOTE) as f:
            d = f.read().strip()
    return d if d and os.path.isdir(d) else None


def build_ref(ref_root: str | None = None) -> bool:
    """Compile the reference harness from the tree `ref_root` (default
    $XDG_REFERENCE_DIR); False when no tree is given or it is absent."""
    ref_root = ref_root or reference_dir()
    if not ref_root or not os.path.isdir(ref_root):
        return False
    subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={ref_root}"], check=True)
    if not os.path.exists(REF_PATH):
        return False
    with open(REF_DIR_NOTE, "w") as f:
        f.write(os.path.abspath(ref_root))
    return True


def _p(a, t):
    return None if a is None else a.ctypes.data_as(t)


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        L.xo_plucker_edge_test.restype = _dbl
        L.xo_plucker_edge_test.argtypes = [_D, _D, _D, _D]
        L.xo_plucker_ray_tri.restype = _int
        L.xo_plucker_ray_tri.argtypes = [_D, _D, _D, _dbl, _dbl, _int, _int, _D]
        L.xo_tet_contains.restype = _int
        L.xo_tet_contains.argtypes = [_D, _D]
        L.xo_closest_region.restype = _int
        L.xo_closest_region.argtypes = [_D, _D]
        L.xo_closest_on_tri.argtypes = [_D, _D, _D]
        L.xo_normalize.argtypes = [_D]
        L.xo_face_normal.argtypes = [_D, _D]
        L.xo_tree_create_tris.restype = _VP
        L.xo_tree_create_tris.argtypes = [_i64, _D, _I, _I, _U8, _dbl, _int]
        L.xo_tree_create_tets.restype = _VP
        L.xo_tree_create_tets.argtypes = [_i64, _D, _I, _int]
        L.xo_tree_destroy.argtypes = [_VP]
        L.xo_ray_fire.argtypes = [_VP, _i64, _D, _D, _D, _int, _I, _I, _D, _I, _I, _int]
        L.xo_point_in_volume.argtypes = [_VP, _i64, _D, _D, _I, _I, _I, _int]
        L.xo_occluded.argtypes = [_VP, _i64, _D, _D, _I, _D, _int]
        L.xo_closest.argtypes = [_VP, _i64, _D, _D, _I, _int]
        L.xo_find_element.argtypes = [_VP, _i64, _D, _I, _I, _int]
        L.xo_tetmesh_create.restype = _VP
        L.xo_tetmesh_create.argtypes = [_i64, _D, _i64, _I, _I, _I]
        L.xo_tetmesh_destroy.argtypes = [_VP]
        L.xo_next_element.restype = _int
        L.xo_next_element.argtypes = [_VP, _i32, _D, _D, _I, _D]
        L.xo_walk_elements.argtypes = [_VP, _i64, _I, _D, _D, _D, _i32, _I, _D, _I, _I, _int]
        _U64 = ctypes.POINTER(ctypes.c_uint64)
        L.xo_uniform.restype = _dbl
        L.xo_uniform.argtypes = [_U64]
        L.xo_series_log.restype = _dbl
        L.xo_series_log.argtypes = [_dbl]
        L.xo_sample_collision.restype = _dbl
        L.xo_sample_collision.argtypes = [_U64, _dbl]
        L.xo_sample_direction.argtypes = [_U64, _D]
        L.xo_transport_elements.argtypes = [_VP, _i64, _I, _D, _D, _U64, _dbl, _i32, _D, _I, _D,
                                            _I, _int]
        L.xo_transport_surfaces.argtypes = [_VP, _i32, _I, _I, _I, _i32, _D, _i32, _i64, _I, _D,
                                            _D, _U64, _dbl, _i32, _i32, _D, _I, _D, _I, _int]
        L.xo_walk_particles.argtypes = [_VP, _VP, _VP, _i64, _I, _D, _D, _U64, _dbl, _i32, _D,
                                        _I, _I, _int]
        _lib = L
    return _lib


def ref_lib():
    """The reference's own code (None when oracle/_ref was not built here)."""
    global _ref
    if _ref is None:
        if not os.path.exists(REF_PATH):
            return None
        R = ctypes.CDLL(REF_PATH)
        R.ref_plucker_edge_test.restype = _dbl
        R.ref_plucker_edge_test.argtypes = [_D, _D, _D, _D]
        R.ref_plucker_ray_tri.restype = _int
        R.ref_plucker_ray_tri.argtypes = [_D, _D, _D, _dbl, _dbl, _int, _int, _D]
        R.ref_closest_on_tri.argtypes = [_D, _D, _D]
        R.ref_closest_region.restype = _int
        R.ref_closest_region.argtypes = [_D, _D]
        R.ref_normalize.argtypes = [_D]
        R.ref_mesh_create.restype = _VP
        R.ref_mesh_create.argtypes = [_i64, _D, _i64, _I, _I, _I]
        R.ref_mesh_destroy.argtypes = [_VP]
        R.ref_next_element.restype = _int
        R.ref_next_element.argtypes = [_VP, _i32, _D, _D, _I, _D]
        R.ref_walk_elements.restype = _i32
        R.ref_walk_elements.argtypes = [_VP, _i32, _D, _D, _dbl, _i32, _I, _D]
        R.ref_walk_elements_to.restype = _i32
        R.ref_walk_elements_to.argtypes = [_VP, _i32, _D, _D, _i32, _I, _D]
        _ref = R
    return _ref


def _f64(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a if shape is None else a.reshape(shape)


def _i32a(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def n_threads_default():
    return os.cpu_count() or 1


# --------------------------------------------------------------------------
# scalar kernels
# --------------------------------------------------------------------------

def plucker(v9, o, d, t_max=INFTY, t_min=0.0, use_orientation=False, orientation=0, use_ref=False):
    L = ref_lib() if use_ref else lib()
    fn = L.ref_plucker_ray_tri if use_ref else L.xo_plucker_ray_tri
    v9, o, d = _f64(v9), _f64(o), _f64(d)
    t = np.zeros(1)
    hit = fn(_p(v9, _D), _p(o, _D), _p(d, _D), t_max, t_min, int(use_orientation), orientation,
             _p(t, _D))
    return bool(hit), float(t[0])


def tet_contains(p, v12):
    p, v12 = _f64(p), _f64(v12)
    return bool(lib().xo_tet_contains(_p(p, _D), _p(v12, _D)))


def closest_on_tri(v9, p, use_ref=False):
    L = ref_lib() if use_ref else lib()
    fn = L.ref_closest_on_tri if use_ref else L.xo_closest_on_tri
    v9, p = _f64(v9), _f64(p)
    out = np.zeros(3)
    fn(_p(v9, _D), _p(p, _D), _p(out, _D))
    return out


def closest_region(v9, p, use_ref=False):
    L = ref_lib() if use_ref else lib()
    fn = L.ref_closest_region if use_ref else L.xo_closest_region
    v9, p = _f64(v9), _f64(p)
    return int(fn(_p(v9, _D), _p(p, _D)))


def normalize(v, use_ref=False):
    L = ref_lib() if use_ref else lib()
    fn = L.ref_normalize if use_ref else L.xo_normalize
    v = _f64(v).copy()
    fn(_p(v, _D))
    return v


def face_normal(v9):
    v9 = _f64(v9)
    n = np.zeros(3)
    lib().xo_face_normal(_p(v9, _D), _p(n, _D))
    return n


# --------------------------------------------------------------------------
# trees
# --------------------------------------------------------------------------

def _csr(excl, n):
    if excl is None:
        return None, None
    off = np.zeros(n + 1, dtype=np.int32)
    off[1:] = np.cumsum([len(e) for e in excl])
    ids = np.ascontiguousarray(np.concatenate([np.asarray(e, dtype=np.int32) for e in excl])
                               if off[-1] else np.zeros(1, dtype=np.int32), dtype=np.int32)
    return off, ids


class TriTree:
    """Oracle surface tree (see xo_tree_create_tris)."""

    def __init__(self, tri_xyz, face_ids, surf_ids, flip, bump, use_bvh=True):
        self._keep = (_f64(tri_xyz), _i32a(face_ids), _i32a(surf_ids),
                      np.ascontiguousarray(flip, dtype=np.uint8))
        x, f, s, fl = self._keep
        self.n = len(f)
        self.h = lib().xo_tree_create_tris(self.n, _p(x, _D), _p(f, _I), _p(s, _I), _p(fl, _U8),
                                           float(bump), int(use_bvh))

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.xo_tree_destroy(self.h)
            self.h = None

    def ray_fire(self, org, dirs, dist_limit=None, orientation=EXITING, excl=None, threads=None):
        org, dirs = _f64(org, (-1, 3)), _f64(dirs, (-1, 3))
        n = len(org)
        dl = None if dist_limit is None else _f64(np.broadcast_to(dist_limit, (n,)))
        off, ids = _csr(excl, n)
        t = np.zeros(n)
        s = np.zeros(n, dtype=np.int32)
        f = np.zeros(n, dtype=np.int32)
        lib().xo_ray_fire(self.h, n, _p(org, _D), _p(dirs, _D), _p(dl, _D), orientation,
                          _p(off, _I), _p(ids, _I), _p(t, _D), _p(s, _I), _p(f, _I),
                          threads or n_threads_default())
        return t, s, f

    def point_in_volume(self, pts, dirs=None, excl=None, threads=None):
        pts = _f64(pts, (-1, 3))
        n = len(pts)
        d = None if dirs is None else _f64(dirs, (-1, 3))
        off, ids = _csr(excl, n)
        out = np.zeros(n, dtype=np.int32)
        lib().xo_point_in_volume(self.h, n, _p(pts, _D), _p(d, _D), _p(off, _I), _p(ids, _I),
                                 _p(out, _I), threads or n_threads_default())
        return out

    def occluded(self, org, dirs, threads=None):
        org, dirs = _f64(org, (-1, 3)), _f64(dirs, (-1, 3))
        n = len(org)
        occ = np.zeros(n, dtype=np.int32)
        dist = np.zeros(n)
        lib().xo_occluded(self.h, n, _p(org, _D), _p(dirs, _D), _p(occ, _I), _p(dist, _D),
                          threads or n_threads_default())
        return occ, dist

    def closest(self, pts, threads=None):
        pts = _f64(pts, (-1, 3))
        n = len(pts)
        d = np.zeros(n)
        f = np.zeros(n, dtype=np.int32)
        lib().xo_closest(self.h, n, _p(pts, _D), _p(d, _D), _p(f, _I),
                         threads or n_threads_default())
        return d, f


class TetTree:
    """Oracle element tree (see xo_tree_create_tets)."""

    def __init__(self, tet_xyz, elem_ids, use_bvh=True):
        self._keep = (_f64(tet_xyz), _i32a(elem_ids))
        x, ids = self._keep
        self.n = len(ids)
        self.h = lib().xo_tree_create_tets(self.n, _p(x, _D), _p(ids, _I), int(use_bvh))

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.xo_tree_destroy(self.h)
            self.h = None

    def find_element(self, pts, threads=None):
        pts = _f64(pts, (-1, 3))
        n = len(pts)
        eid = np.zeros(n, dtype=np.int32)
        eidx = np.zeros(n, dtype=np.int32)
        lib().xo_find_element(self.h, n, _p(pts, _D), _p(eid, _I), _p(eidx, _I),
                              threads or n_threads_default())
        return eid, eidx


class TetWalker:
    """Oracle tet walk over a whole tet mesh (xo_tetmesh_*)."""

    def __init__(self, vertices, conn, adj, face_table):
        self._keep = (_f64(vertices, (-1, 3)), _i32a(conn), _i32a(adj), _i32a(face_table))
        v, c, a, ft = self._keep
        self.h = lib().xo_tetmesh_create(len(v), _p(v, _D), len(c), _p(c, _I), _p(a, _I),
                                         _p(ft, _I))

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.xo_tetmesh_destroy(self.h)
            self.h = None

    def next_element(self, elem, r, u):
        r, u = _f64(r), _f64(u)
        nxt = np.zeros(1, dtype=np.int32)
        dist = np.zeros(1)
        st = lib().xo_next_element(self.h, int(elem), _p(r, _D), _p(u, _D), _p(nxt, _I),
                                   _p(dist, _D))
        return int(nxt[0]), float(dist[0]), int(st)

    def walk(self, start_elem, start, u, distance, max_segs=256, threads=None):
        se = _i32a(np.atleast_1d(start_elem))
        n = len(se)
        start, u = _f64(start, (-1, 3)), _f64(u, (-1, 3))
        dist = _f64(np.broadcast_to(distance, (n,)))
        el = np.zeros((n, max_segs), dtype=np.int32)
        ln = np.zeros((n, max_segs))
        cnt = np.zeros(n, dtype=np.int32)
        st = np.zeros(n, dtype=np.int32)
        lib().xo_walk_elements(self.h, n, _p(se, _I), _p(start, _D), _p(u, _D), _p(dist, _D),
                               max_segs, _p(el, _I), _p(ln, _D), _p(cnt, _I), _p(st, _I),
                               threads or n_threads_default())
        return el, ln, cnt, st


    def transport(self, elem, pos, dirs, rng, mfp, max_events, distance=None, events=None,
                  n_tets=None, threads=1):
        """xo_transport_elements on copies of the state; returns (elem, pos,
        dir, rng, distance, events, status, tally)."""
        U64 = ctypes.POINTER(ctypes.c_uint64)
        e = _i32a(elem).copy()
        n = len(e)
        r, u = _f64(pos, (-1, 3)).copy(), _f64(dirs, (-1, 3)).copy()
        s = np.ascontiguousarray(rng, dtype=np.uint64).copy()
        d = np.zeros(n) if distance is None else _f64(distance).copy()
        ev = np.zeros(n, dtype=np.int32) if events is None else _i32a(events).copy()
        st = np.zeros(n, dtype=np.int32)
        tally = np.zeros(int(n_tets if n_tets is not None else self._keep[1].shape[0]))
        lib().xo_transport_elements(self.h, n, _p(e, _I), _p(r, _D), _p(u, _D), _p(s, U64),
                                    float(mfp), int(max_events), _p(d, _D), _p(ev, _I),
                                    _p(tally, _D), _p(st, _I), int(threads))
        return e, r, u, s, d, ev, st, tally

    def walk_particles(self, ipc_tree, elem_tree, elem, pos, dirs, rng, mfp, max_events,
                       threads=None):
        """xo_walk_particles (the whole walk_elements tool loop); returns
        (elem, pos, dir, rng, distance, events, status)."""
        U64 = ctypes.POINTER(ctypes.c_uint64)
        e = _i32a(elem).copy()
        n = len(e)
        r, u = _f64(pos, (-1, 3)).copy(), _f64(dirs, (-1, 3)).copy()
        s = np.ascontiguousarray(rng, dtype=np.uint64).copy()
        d = np.zeros(n)
        ev = np.zeros(n, dtype=np.int32)
        st = np.zeros(n, dtype=np.int32)
        lib().xo_walk_particles(self.h, ipc_tree.h, elem_tree.h, n, _p(e, _I), _p(r, _D),
                                _p(u, _D), _p(s, U64), float(mfp), int(max_events), _p(d, _D),
                                _p(ev, _I), _p(st, _I), threads or n_threads_default())
        return e, r, u, s, d, ev, st


class SurfaceTransport:
    """The particle_sim tool loop over oracle volume trees
    (xo_transport_surfaces).  ``tree_of_volume`` maps each volume to the
    engine's surface tree id, so particle states use the same tree ids;
    ``bc`` maps surface ids to 0 transmission / 1 vacuum / 2 reflecting."""

    def __init__(self, model, tree_of_volume, bc=None):
        bc = bc or {}
        self.n_trees = max(tree_of_volume.values())
        self.trees = [None] * self.n_trees
        for v, t in tree_of_volume.items():
            self.trees[t - 1] = volume_tree(model, v)
        self._ptrs = (ctypes.c_void_p * self.n_trees)(
            *[t.h if t is not None else None for t in self.trees])
        ns = max(s.surface_id for s in model.surfaces) + 1
        self.fwd = np.full(ns, -1, dtype=np.int32)
        self.rev = np.full(ns, -1, dtype=np.int32)
        self.bc = np.zeros(ns, dtype=np.int32)
        nf = max(int(s.face_ids.max()) for s in model.surfaces) + 1
        self.face_xyz = np.zeros((nf, 9))
        for srf in model.surfaces:
            self.fwd[srf.surface_id] = tree_of_volume.get(srf.forward_volume, -1)
            self.rev[srf.surface_id] = tree_of_volume.get(srf.reverse_volume, -1)
            self.bc[srf.surface_id] = bc.get(srf.surface_id, 0)
            self.face_xyz[srf.face_ids] = srf.tri_xyz()

    def run(self, tree, pos, dirs, rng, mfp, max_events, graveyard_tree=0, threads=None):
        """Returns (tree, pos, dir, rng, distance, events, status, tally)."""
        U64 = ctypes.POINTER(ctypes.c_uint64)
        t = _i32a(tree).copy()
        n = len(t)
        r, u = _f64(pos, (-1, 3)).copy(), _f64(dirs, (-1, 3)).copy()
        s = np.ascontiguousarray(rng, dtype=np.uint64).copy()
        d = np.zeros(n)
        ev = np.zeros(n, dtype=np.int32)
        st = np.zeros(n, dtype=np.int32)
        tally = np.zeros(self.n_trees + 1)
        lib().xo_transport_surfaces(
            ctypes.cast(self._ptrs, _VP), self.n_trees, _p(self.fwd, _I), _p(self.rev, _I),
            _p(self.bc, _I), len(self.fwd), _p(self.face_xyz, _D), len(self.face_xyz), n,
            _p(t, _I), _p(r, _D), _p(u, _D), _p(s, U64), float(mfp), int(max_events),
            int(graveyard_tree), _p(d, _D), _p(ev, _I), _p(tally, _D), _p(st, _I),
            threads or n_threads_default())
        return t, r, u, s, d, ev, st, tally


def series_log(x):
    return lib().xo_series_log(float(x))


def sample_streams(states, draws):
    """`draws` uniforms from each stream (for tests of the generator)."""
    U64 = ctypes.POINTER(ctypes.c_uint64)
    st = np.ascontiguousarray(states, dtype=np.uint64).copy()
    out = np.zeros((len(st), draws))
    one = np.zeros(1, dtype=np.uint64)
    for i in range(len(st)):
        one[0] = st[i]
        for k in range(draws):
            out[i, k] = lib().xo_uniform(_p(one, U64))
    return out


class RefWalker:
    """The reference's own MeshManager::walk_elements over a harness mesh."""

    def __init__(self, vertices, conn, adj, face_table):
        R = ref_lib()
        if R is None:
            raise RuntimeError("oracle/_ref was not built (reference tree absent)")
        self._keep = (_f64(vertices, (-1, 3)), _i32a(conn), _i32a(adj), _i32a(face_table))
        v, c, a, ft = self._keep
        self.h = R.ref_mesh_create(len(v), _p(v, _D), len(c), _p(c, _I), _p(a, _I), _p(ft, _I))

    def __del__(self):
        if getattr(self, "h", None) and _ref is not None:
            _ref.ref_mesh_destroy(self.h)
            self.h = None

    def next_element(self, elem, r, u):
        r, u = _f64(r), _f64(u)
        nxt = np.zeros(1, dtype=np.int32)
        dist = np.zeros(1)
        _ref.ref_next_element(self.h, int(elem), _p(r, _D), _p(u, _D), _p(nxt, _I), _p(dist, _D))
        return int(nxt[0]), float(dist[0])

    def walk(self, elem, start, u, distance, max_segs=4096):
        start, u = _f64(start), _f64(u)
        el = np.zeros(max_segs, dtype=np.int32)
        ln = np.zeros(max_segs)
        k = _ref.ref_walk_elements(self.h, int(elem), _p(start, _D), _p(u, _D), float(distance),
                                   max_segs, _p(el, _I), _p(ln, _D))
        return el[:min(k, max_segs)], ln[:min(k, max_segs)]

    def walk_to(self, elem, start, end, max_segs=4096):
        start, end = _f64(start), _f64(end)
        el = np.zeros(max_segs, dtype=np.int32)
        ln = np.zeros(max_segs)
        k = _ref.ref_walk_elements_to(self.h, int(elem), _p(start, _D), _p(end, _D), max_segs,
                                      _p(el, _I), _p(ln, _D))
        return el[:min(k, max_segs)], ln[:min(k, max_segs)]


# --------------------------------------------------------------------------
# model-level helpers (trees per volume, as EmbreeRayTracer builds them)
# --------------------------------------------------------------------------

def volume_bump(model, vol):
    """ray_tracing_interface.cpp:20-24: max(volume_bbox.dilation(), 1e-3)."""
    lo = np.full(3, np.inf)
    hi = np.full(3, -np.inf)
    for s, _ in model.volume_surfaces(vol):
        x = s.vertices[s.triangles.reshape(-1)]
        lo = np.minimum(lo, x.min(0))
        hi = np.maximum(hi, x.max(0))
    w = hi - lo
    chord = np.sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2])
    return max(chord * 1e-6, 1e-3)


def surface_bumps(model):
    """Per-surface bump = max over its parent volumes (embree/ray_tracer.cpp:76-89)."""
    vb = {v: volume_bump(model, v) for v in model.volumes if model.volume_surfaces(v)}
    out = {}
    for s in model.surfaces:
        b = [vb[v] for v in (s.forward_volume, s.reverse_volume) if v in vb]
        out[s.surface_id] = max(b) if b else 1e-3
    return out


def volume_tree(model, vol, use_bvh=True, bumps=None):
    """Oracle TriTree holding the surfaces of ``vol`` with its sense flips."""
    bumps = bumps or surface_bumps(model)
    xs, fs, ss, fl = [], [], [], []
    bump = 0.0
    for s, sense in model.volume_surfaces(vol):
        xs.append(s.tri_xyz())
        fs.append(s.face_ids)
        ss.append(np.full(len(s.face_ids), s.surface_id, dtype=np.int32))
        fl.append(np.full(len(s.face_ids), 1 if sense == 1 else 0, dtype=np.uint8))
        bump = max(bump, bumps[s.surface_id])
    return TriTree(np.concatenate(xs), np.concatenate(fs), np.concatenate(ss),
                   np.concatenate(fl), bump, use_bvh)


# --------------------------------------------------------------------------
# XDG::segments(start, end) (xdg.cpp:142-198), one track at a time
# --------------------------------------------------------------------------

TINY_BIT = 1e-10  # constants.h:32


class GlobalTracker:
    """The global track loop of xdg.cpp:142-198 over oracle trees: find the
    element at r in the global element tree (ignoring the element just left),
    else fire an EXITING ray in the implicit complement from r + u*TINY_BIT,
    step to the hit plus TINY_BIT and re-enter through
    get_boundary_face_element of the hit face; walk; repeat while distance
    remains."""

    def __init__(self, model):
        tm = model.tets
        self.model = model
        self.elem_ids = np.asarray(tm.elem_ids, dtype=np.int32)
        self.tets = TetTree(tm.tet_xyz(), tm.elem_ids)
        self.walker = TetWalker(tm.vertices, tm.conn, tm.adj, tm.face_table)
        self.ipc = volume_tree(model, model.implicit_complement)
        self.bfe = model.boundary_face_element

    def segments(self, start, end, max_segs=4096, max_rounds=10_000):
        r = np.array(start, dtype=np.float64)
        e = np.array(end, dtype=np.float64)
        u = e - r
        dist = float(np.sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]))
        u = u / dist
        out_e, out_l = [], []
        rounds = 0
        while dist > 0 and rounds < max_rounds:
            rounds += 1
            eid, eidx = self.tets.find_element(r[None, :], threads=1)
            cur = int(eidx[0])
            if out_e and int(eid[0]) == out_e[-1]:
                cur = -1
            if cur < 0:
                o = r + u * TINY_BIT
                t, s, f = self.ipc.ray_fire(o[None, :], u[None, :], None, EXITING, [[]], threads=1)
                if s[0] == -1 or t[0] > dist:
                    break
                hd = t[0] + TINY_BIT
                r = r + u * hd
                dist = dist - hd
                cur = int(self.bfe[f[0]]) if self.bfe is not None else -1
                if cur < 0:
                    break
            el, ln, cnt, st = self.walker.walk(np.array([cur], dtype=np.int32), r[None, :],
                                               u[None, :], np.array([dist]), max_segs, threads=1)
            k = int(cnt[0])
            ssum = 0.0
            for j in range(k):
                out_e.append(int(self.elem_ids[el[0, j]]))
                out_l.append(float(ln[0, j]))
                ssum = ssum + float(ln[0, j])
            r = r + u * ssum
            dist = dist - ssum
        return np.array(out_e, dtype=np.int32), np.array(out_l)
