"""The FP32 slab test of the mixed traversal (`make_boxray32` and
`node_test32` in traverse.cuh; boxes rounded outward to FP32 in bvh.cu)
never culls the box of a triangle the FP64 test hits: every primitive box is
dilated by the bump (ray_tracing_interface.cpp:20-24, at least 1e-3 for
surface trees), and rays for which 8 u (max_abs + |o|) is not below the bump
use FP64 boxes instead (`use64` in trace.cu).

Restated here in numpy: the ray's truncation toward zero and reciprocal,
the three FMAs per plane as correctly rounded FP32 FMAs (an exact FP64
product, an error-free sum and the midpoint case resolved by its sign), and
the culling distance rounded up to FP32.  For rays the oracle's FP64 test
(plucker.h:64-161, t in [0, inf)) says hit a triangle, the triangle's leaf
box (its FP64 box widened by the bump 1e-3, rounded outward) must pass with
the culling distance equal to the hit distance (the tie case: the reference
replaces on equal distance).  Cases: triangles of sizes 1e-4..1e2 up to 1e5
from the origin, rays from 1e-6..1e3 sizes away aimed at vertices, edges and
interior points, some nearly parallel to an axis or a face.
"""
import ctypes

import numpy as np

from fp32_emul import F, U, f32_dir, f32_trunc, fma32

BUMP = 1e-3


def slab_pass(lo, hi, o, d, tfar):
    """node_test32 for one box per ray."""
    dt = f32_trunc(d)
    safe = np.where(np.abs(dt) < F(1e-20), np.copysign(F(1e-20), dt), dt).astype(np.float32)
    inv = (F(1) / safe).astype(np.float32)
    ot = (f32_trunc(o) * inv).astype(np.float32)
    neg = np.signbit(inv)
    near = np.where(neg, hi, lo)
    far = np.where(neg, lo, hi)
    tn = fma32(near, inv, -ot)
    tf = fma32(far, inv, -ot)
    t0 = np.maximum(np.maximum(tn[:, 0], tn[:, 1]), np.maximum(tn[:, 2], F(0)))
    t1 = np.minimum(np.minimum(tf[:, 0], tf[:, 1]), np.minimum(tf[:, 2], tfar))
    return t0 <= t1


def _unit(rng, n):
    x = rng.normal(size=(n, 3))
    return x / np.linalg.norm(x, axis=1)[:, None]


def test_box_of_a_hit_is_never_culled(oracle):
    rng = np.random.default_rng(41)
    n = 60000
    scale = 10.0 ** rng.choice([0.0, 2.0, 3.0, 5.0], n)
    size = 10.0 ** rng.uniform(-4, 2, n)
    c = rng.uniform(-1, 1, (n, 3)) * scale[:, None]
    v = c[:, None, :] + rng.normal(size=(n, 3, 3)) * size[:, None, None]
    kind = rng.integers(0, 3, n)
    k = rng.integers(0, 3, n)
    idx = np.arange(n)
    b = rng.dirichlet([1, 1, 1], n)
    a = rng.random(n)
    edge = v[idx, k] + a[:, None] * (v[idx, (k + 1) % 3] - v[idx, k])
    aim = np.where((kind == 0)[:, None], v[idx, k],
                   np.where((kind == 1)[:, None], edge, (b[:, :, None] * v).sum(1)))
    d = _unit(rng, n)
    ax = rng.random(n) < 0.2  # nearly along an axis
    e = np.zeros((n, 3))
    e[idx, rng.integers(0, 3, n)] = rng.choice([-1.0, 1.0], n)
    e = e + (10.0 ** rng.uniform(-30, -3, n))[:, None] * _unit(rng, n)
    d = np.where(ax[:, None], e / np.linalg.norm(e, axis=1)[:, None], d)
    o = aim - (10.0 ** rng.uniform(-6, 3, n) * size)[:, None] * d

    L = oracle.lib()
    D = ctypes.POINTER(ctypes.c_double)
    t = np.zeros(1)
    hit = np.zeros(n, dtype=bool)
    th = np.zeros(n)
    for i in range(n):
        vi = np.ascontiguousarray(v[i].reshape(9))
        oi, di = np.ascontiguousarray(o[i]), np.ascontiguousarray(d[i])
        hit[i] = bool(L.xo_plucker_ray_tri(vi.ctypes.data_as(D), oi.ctypes.data_as(D), di.ctypes.data_as(D),
                                           np.finfo(np.float64).max, 0.0, 0, 0, t.ctypes.data_as(D)))
        th[i] = t[0]
    lo = f32_dir(v.min(1) - BUMP, up=False)
    hi = f32_dir(v.max(1) + BUMP, up=True)
    max_abs = np.maximum(np.abs(lo), np.abs(hi)).max(1)
    oabs = np.abs(f32_trunc(o)).max(1)
    fp32_boxes = (F(8) * U) * (max_abs + oabs) < F(BUMP)
    sel = hit & fp32_boxes
    assert sel.sum() > 20000
    tfar = f32_dir(th[sel], up=True)
    ok = slab_pass(lo[sel], hi[sel], o[sel], d[sel], tfar)
    bad = np.nonzero(~ok)[0]
    assert len(bad) == 0, f"box of an FP64 hit culled: {np.nonzero(sel)[0][bad[:5]]}"
