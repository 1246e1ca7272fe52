"""The FP32 face filter of the mixed tet walk (`next_face` in walk.cu, vertex
copies from `k_vert32` in api.cu) skips the FP64 test of a face only when the
FP64 test (plucker.h:64-161 with orientation +1, as
mesh_manager_interface.cpp:149-200 calls it, through the oracle) rejects the
face: a face with a Plucker coordinate certified positive is an early exit
of the FP64 test.

The filter is restated here in numpy: vertices, position and direction
rounded to nearest, the six pair coordinates u . ((v_j - v_i) x (v_i - r))
in IEEE FP32 with the kernel's operation order (-fmad=false), the face's
coordinates by the pair's sign, and the threshold as written.  The FP64 test
runs with t unbounded on both sides, so only its sign test can reject.
Cases: tets of sizes 1e-4..1e2 up to 1e6 from the origin, slivers and
needles, positions inside, on faces, on edges and at vertices (offsets down
to 1e-14 of the size), and directions at random or grazing a face.
"""
import ctypes

import numpy as np
import pytest

from xdg_gb300.synth import MOCK_TET_FACES

F = np.float32
DBL_MAX = np.finfo(np.float64).max
MOAB_FACES = [(0, 1, 3), (1, 2, 3), (2, 0, 3), (0, 2, 1)]  # direct_access.h:181-183
PAIRS = [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)]


def face_early_exit(v, r, u, faces=MOAB_FACES):
    """(n, 4) bool: face f certified to be rejected by the FP64 test."""
    P = v.astype(np.float32)
    Pw = np.abs(P).max(2)
    r32, u32 = r.astype(np.float32), u.astype(np.float32)
    w = P - r32[:, None, :]
    W = np.abs(w).max((1, 2))
    Av = Pw.max(1)
    D = np.abs(u32).max(1)
    A = Av + np.abs(r32).max(1)
    thr = ((((((F(5.9604645e-08) * F(1.000001)) * D) * W) * ((F(97) * W + F(13) * Av) + F(13) * A))
            * F(1.0001)) + F(4.5e-15))
    pe = {}
    for i, j in PAIRS:
        e = P[:, j] - P[:, i]
        wi = w[:, i]
        cx = e[:, 1] * wi[:, 2] - e[:, 2] * wi[:, 1]
        cy = e[:, 2] * wi[:, 0] - e[:, 0] * wi[:, 2]
        cz = e[:, 0] * wi[:, 1] - e[:, 1] * wi[:, 0]
        pe[(i, j)] = (u32[:, 0] * cx + u32[:, 1] * cy) + u32[:, 2] * cz
    coord = lambda a, b: pe[(a, b)] if a < b else -pe[(b, a)]  # noqa: E731
    out = np.zeros((len(v), 4), dtype=bool)
    for f, (l0, l1, l2) in enumerate(faces):
        out[:, f] = (coord(l0, l1) > thr) | (coord(l1, l2) > thr) | (coord(l2, l0) > thr)
    return out


def _unit(rng, n):
    x = rng.normal(size=(n, 3))
    return x / np.linalg.norm(x, axis=1)[:, None]


def _cases(rng, n):
    scale = 10.0 ** rng.choice([0.0, 2.0, 4.0, 6.0], n)
    size = 10.0 ** rng.uniform(-4, 2, n)
    c = rng.uniform(-1, 1, (n, 3)) * scale[:, None]
    v = c[:, None, :] + rng.normal(size=(n, 4, 3)) * size[:, None, None]
    kind = rng.integers(0, 3, n)
    s = kind == 1
    w3 = rng.dirichlet([1, 1, 1], s.sum())
    base = (w3[:, :, None] * v[s, :3]).sum(1)
    nrm = np.cross(v[s, 1] - v[s, 0], v[s, 2] - v[s, 0])
    nrm /= np.linalg.norm(nrm, axis=1)[:, None]
    v[s, 3] = base + (10.0 ** rng.uniform(-9, -2, s.sum()) * size[s] * rng.choice([-1, 1], s.sum()))[:, None] * nrm
    nd = kind == 2
    d = rng.normal(size=(nd.sum(), 3))
    for k in (1, 2, 3):
        v[nd, k] = (v[nd, 0] + rng.uniform(0.2, 1, nd.sum())[:, None] * d * size[nd, None] * k
                    + (10.0 ** rng.uniform(-6, -2, nd.sum()) * size[nd])[:, None] * rng.normal(size=(nd.sum(), 3)))
    T = v[:, 1:] - v[:, :1]
    neg = np.linalg.det(T) < 0
    v[neg, 1], v[neg, 2] = v[neg, 2].copy(), v[neg, 1].copy()
    # positions: inside, on a face, on an edge, at a vertex, nudged
    pk = rng.integers(0, 4, n)
    b = rng.dirichlet([1, 1, 1, 1], n)
    drop = rng.integers(0, 4, n)
    idx = np.arange(n)
    bf = b.copy()
    bf[idx, drop] = 0
    bf /= bf.sum(1)[:, None]
    be = np.zeros((n, 4))
    a = rng.random(n)
    be[idx, drop] = a
    be[idx, (drop + 1) % 4] = 1 - a
    bv = np.zeros((n, 4))
    bv[idx, drop] = 1
    bary = np.where((pk == 0)[:, None], b, np.where((pk == 1)[:, None], bf, np.where((pk == 2)[:, None], be, bv)))
    r = (bary[:, :, None] * v).sum(1) + (10.0 ** rng.uniform(-14, -2, n) * size)[:, None] * _unit(rng, n)
    u = _unit(rng, n)
    # grazing a face: mostly in the plane of face `drop`'s opposite vertices
    gr = rng.random(n) < 0.3
    fv = np.stack([v[idx, (drop + k) % 4] for k in (1, 2, 3)], 1)
    fn = np.cross(fv[:, 1] - fv[:, 0], fv[:, 2] - fv[:, 0])
    fn /= np.linalg.norm(fn, axis=1)[:, None] + 1e-300
    inpl = u - (u * fn).sum(1)[:, None] * fn
    inpl /= np.linalg.norm(inpl, axis=1)[:, None] + 1e-300
    g = inpl + (10.0 ** rng.uniform(-12, -1, n))[:, None] * fn
    g /= np.linalg.norm(g, axis=1)[:, None]
    u = np.where(gr[:, None], g, u)
    return v, r, u


@pytest.mark.parametrize("faces", [MOAB_FACES, [tuple(f) for f in MOCK_TET_FACES]], ids=["moab", "mock"])
def test_certified_exit_is_fp64_rejection(oracle, faces):
    rng = np.random.default_rng(23)
    n = 40000
    v, r, u = _cases(rng, n)
    cert = face_early_exit(v, r, u, faces)
    L = oracle.lib()
    D = ctypes.POINTER(ctypes.c_double)
    t = np.zeros(1)
    bad = []
    for i, f in zip(*np.nonzero(cert)):
        fv = np.ascontiguousarray(v[i, list(faces[f])].reshape(9))
        ri, ui = np.ascontiguousarray(r[i]), np.ascontiguousarray(u[i])
        if L.xo_plucker_ray_tri(fv.ctypes.data_as(D), ri.ctypes.data_as(D), ui.ctypes.data_as(D),
                                DBL_MAX, -DBL_MAX, 1, 1, t.ctypes.data_as(D)):
            bad.append((i, f))
    assert not bad, f"certified early exit, FP64 test passes: {bad[:5]}"
    # the filter settles most faces: a ray leaves a tet through one face
    assert cert.sum() > 0.3 * cert.size
