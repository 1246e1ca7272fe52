"""The FP32 Plucker pre-filter of the mixed traversal (`plucker_filter32` in
geom.cuh; the triangle record from `k_tri_gather` in api.cu, the ray from
`make_ray32`) skips a triangle only when the FP64 test (plucker.h:64-161
through the oracle) rejects it: a certified miss (two Plucker coordinates
certified to have opposite signs) is a miss of the FP64 sign test.

Both are restated here in numpy: the record's roundings (vertex and edges to
nearest, the edge bound upward), the ray's truncation toward zero, and the
filter in IEEE FP32 with the kernel's operation order (the kernels compile
with -fmad=false, so products and sums are separate roundings).  The FP64
test runs with t unbounded on both sides, so that only its sign test (and
the all-zero rejection) can reject.  Cases: triangles of sizes 1e-4..1e2 up
to 1e6 from the origin, needles, rays aimed at vertices, edges and interior
points with offsets down to 1e-14 of the size, grazing rays, and origins from
1e-6 to 1e3 sizes away.
"""
import ctypes

import numpy as np

from fp32_emul import F, f32_dir, f32_trunc

DBL_MAX = np.finfo(np.float64).max


def tri_records(v):
    """v (n, 3, 3) -> v0 (f32), v0abs, e1, e2 (f32), emax (f32, upward)."""
    e1 = v[:, 1] - v[:, 0]
    e2 = v[:, 2] - v[:, 0]
    emax = np.zeros(len(v))
    for c in range(3):
        emax = np.fmax(emax, np.abs(e1[:, c]))
        emax = np.fmax(emax, np.abs(e2[:, c]))
        emax = np.fmax(emax, np.abs(e2[:, c] - e1[:, c]))
    v0 = v[:, 0].astype(np.float32)
    v0abs = np.abs(v0).max(1)
    return v0, v0abs, e1.astype(np.float32), e2.astype(np.float32), f32_dir(emax * (1.0 + 9.5367431640625e-07), up=True)


def _triple(d, e, w):
    cx = e[:, 1] * w[:, 2] - e[:, 2] * w[:, 1]
    cy = e[:, 2] * w[:, 0] - e[:, 0] * w[:, 2]
    cz = e[:, 0] * w[:, 1] - e[:, 1] * w[:, 0]
    return (d[:, 0] * cx + d[:, 1] * cy) + d[:, 2] * cz


def certified_miss(v, o, d):
    v0, v0abs, e1, e2, emax = tri_records(v)
    o32, d32 = f32_trunc(o), f32_trunc(d)
    dmax = np.abs(d32).max(1)
    du = dmax * (F(5.9604645e-08) * F(1.000001))
    oabs = np.abs(o32).max(1)
    with np.errstate(over="ignore", invalid="ignore"):
        w0 = v0 - o32
        w1 = w0 + e1
        w2 = w0 + e2
        p01 = _triple(d32, e1, w0)
        p12 = _triple(d32, e2 - e1, w1)
        p20 = _triple(d32, -e2, w2)
        w0a = np.abs(w0).max(1)
        A = v0abs + oabs
        de = du * emax
        thr = ((de * ((F(74) * w0a + F(77) * emax) + F(13) * A)) * F(1.0001)) + F(4.5e-15)
        pos = (p01 > thr) | (p12 > thr) | (p20 > thr)
        neg = (p01 < -thr) | (p12 < -thr) | (p20 < -thr)
    return pos & neg


def _unit(rng, n):
    x = rng.normal(size=(n, 3))
    return x / np.linalg.norm(x, axis=1)[:, None]


def _cases(rng, n):
    scale = 10.0 ** rng.choice([0.0, 2.0, 4.0, 6.0], n)
    size = 10.0 ** rng.uniform(-4, 2, n)
    c = rng.uniform(-1, 1, (n, 3)) * scale[:, None]
    v = c[:, None, :] + rng.normal(size=(n, 3, 3)) * size[:, None, None]
    nd = rng.random(n) < 0.15
    t = rng.uniform(-0.5, 1.5, n)
    v[nd, 2] = (v[nd, 0] + t[nd, None] * (v[nd, 1] - v[nd, 0])
                + (10.0 ** rng.uniform(-12, -3, nd.sum()) * size[nd])[:, None] * rng.normal(size=(nd.sum(), 3)))
    # the aim point: a vertex, an edge point or an interior point, nudged
    kind = rng.integers(0, 3, n)
    k = rng.integers(0, 3, n)
    b = rng.dirichlet([1, 1, 1], n)
    a = rng.random(n)
    idx = np.arange(n)
    edge = v[idx, k] + a[:, None] * (v[idx, (k + 1) % 3] - v[idx, k])
    aim = np.where((kind == 0)[:, None], v[idx, k],
                   np.where((kind == 1)[:, None], edge, (b[:, :, None] * v).sum(1)))
    aim = aim + (10.0 ** rng.uniform(-14, -1, n) * size)[:, None] * _unit(rng, n)
    d = _unit(rng, n)
    # grazing: mostly in the triangle's plane
    gr = rng.random(n) < 0.25
    nrm = np.cross(v[:, 1] - v[:, 0], v[:, 2] - v[:, 0])
    nrm /= np.linalg.norm(nrm, axis=1)[:, None] + 1e-300
    inpl = d - (d * nrm).sum(1)[:, None] * nrm
    inpl /= np.linalg.norm(inpl, axis=1)[:, None] + 1e-300
    tilt = 10.0 ** rng.uniform(-12, -1, n)
    g = inpl + tilt[:, None] * nrm
    g /= np.linalg.norm(g, axis=1)[:, None]
    d = np.where(gr[:, None], g, d)
    dist = 10.0 ** rng.uniform(-6, 3, n) * size
    o = aim - dist[:, None] * d
    return v, o, d


def test_certified_miss_is_fp64_miss(oracle):
    rng = np.random.default_rng(17)
    n = 100000
    v, o, d = _cases(rng, n)
    cm = certified_miss(v, o, d)
    L = oracle.lib()
    t = np.zeros(1)
    D = ctypes.POINTER(ctypes.c_double)
    hit = np.zeros(n, dtype=bool)
    for i in np.nonzero(cm)[0]:
        vi, oi, di = (np.ascontiguousarray(x, dtype=np.float64) for x in (v[i].reshape(9), o[i], d[i]))
        hit[i] = bool(L.xo_plucker_ray_tri(vi.ctypes.data_as(D), oi.ctypes.data_as(D), di.ctypes.data_as(D),
                                           DBL_MAX, -DBL_MAX, 0, 0, t.ctypes.data_as(D)))
    bad = np.nonzero(cm & hit)[0]
    assert len(bad) == 0, f"certified miss, FP64 sign test passes: {bad[:5]}"
    assert cm.sum() > 4000


def test_filter_decides_ordinary_misses():
    """Rays from 1..10 sizes away aimed well outside triangles of sizes 0.1..10
    near the origin are certified misses."""
    rng = np.random.default_rng(4)
    n = 5000
    size = 10.0 ** rng.uniform(-1, 1, n)
    v = rng.uniform(-10, 10, (n, 1, 3)) + rng.normal(size=(n, 3, 3)) * size[:, None, None]
    cen = v.mean(1)
    rad = np.abs(v - cen[:, None]).max((1, 2)) * np.sqrt(3)
    aim = cen + (2.5 * rad)[:, None] * _unit(rng, n)
    d = _unit(rng, n)
    o = aim - (rng.uniform(1, 10, n) * size)[:, None] * d
    # aim points 2.5 radii out can still see the triangle behind or ahead
    # of them only if the line passes within a radius: drop those
    w = cen - aim
    perp = w - (w * d).sum(1)[:, None] * d
    clear = np.linalg.norm(perp, axis=1) > 1.2 * rad
    assert clear.sum() > 1000
    assert certified_miss(v[clear], o[clear], d[clear]).mean() > 0.9
