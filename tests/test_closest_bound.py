"""The FP32 lower bound that lets mixed-precision closest skip a triangle's
FP64 test (`k_closest` in queries.cu) never exceeds the FP64 point-triangle
distance (closest.cpp:54-183 through the oracle), so a triangle it skips is
one the FP64 test would not have taken: its distance is larger than the
best so far.

The planes come from the product's own `tri_cbound` (xdg_gb300/csrc/cbound.h,
the function `k_tri_cbound` runs on the device), compiled here for the host
with FP64 operations unfused as in the device build (-fmad=false).  The
kernel's FP32 evaluation is restated in numpy: IEEE FP32 products, sums and
square roots, and each `__fmaf_rn` as a correctly rounded fused operation.  Cases: random triangles of
sizes 1e-4..1e2 placed up to 1e6 from the origin, needles down to 1e-12 of
their length off a line (whose FP64 normals can be far off), and points on
the plane, near vertices and edges (down to 1e-12 of the triangle's size)
and far away.  The certificates the planes carry (face slab within
7 u max|V|, every vertex inside the edge planes) are checked in exact
rational arithmetic on a sample, the FP32 evaluation against 8 u (|p| + M),
and the bound's use for points well away from the triangle.
"""
import ctypes
import os
import subprocess
from fractions import Fraction

import numpy as np
import pytest

from fp32_emul import U, f32_dir, fma32, fma32_up


HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "xdg_gb300", "csrc")

WRAP = r"""
#include <cstdint>
#include "cbound.h"
extern "C" void cbound_all(const double* v, int64_t n, float* out) {
  for (int64_t i = 0; i < n; ++i) xdgcu::tri_cbound(v + 9 * i, out + 16 * i);
}
"""


@pytest.fixture(scope="module")
def cbound(tmp_path_factory):
    d = str(tmp_path_factory.mktemp("cbound"))
    src, so = os.path.join(d, "w.cpp"), os.path.join(d, "libcb.so")
    with open(src, "w") as f:
        f.write(WRAP)
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Werror", "-ffp-contract=off", "-fPIC",
                        "-shared", "-I", CSRC, src, "-o", so], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lib = ctypes.CDLL(so)
    lib.cbound_all.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p]

    def planes(v):
        v = np.ascontiguousarray(v, dtype=np.float64)
        out = np.zeros((len(v), 4, 4), dtype=np.float32)
        lib.cbound_all(v.ctypes.data, len(v), out.ctypes.data)
        return out

    return planes


def plane_dists32(pl, p):
    """h and the three edge distances in the kernel's FP32 operations."""
    px, py, pz = (p[:, k].astype(np.float32) for k in range(3))

    def ev(k):
        q = pl[:, k]
        return fma32(q[:, 0], px, fma32(q[:, 1], py, fma32(q[:, 2], pz, -q[:, 3])))

    return np.abs(ev(0)), ev(1), ev(2), ev(3)


def skip_value(pl, p, max_abs):
    """The value the kernel compares with the best distance rounded up:
    the triangle is skipped when it is larger."""
    h, s0, s1, s2 = plane_dists32(pl, p)
    mo = np.maximum(np.maximum(np.maximum(s0, s1), s2), np.float32(0))
    lb = np.sqrt(fma32(h, h, mo * mo))
    pabs = np.abs(p.astype(np.float32)).max(1)
    cmargin = (np.float32(48) * U) * (pabs + max_abs)
    return lb * (np.float32(1) - np.float32(8) * U) - cmargin, pabs


def _cases(rng, n):
    scale = 10.0 ** rng.choice([0.0, 3.0, 4.5, 6.0], n)
    size = 10.0 ** rng.uniform(-4, 2, n)
    c = rng.uniform(-1, 1, (n, 3)) * scale[:, None]
    v = c[:, None, :] + rng.normal(size=(n, 3, 3)) * size[:, None, None]
    # needles: the third vertex on the first edge's line, nudged off it
    nd = rng.random(n) < 0.15
    t = rng.uniform(-0.5, 1.5, n)
    nudge = 10.0 ** rng.uniform(-12, -3, n)
    v[nd, 2] = (v[nd, 0] + t[nd, None] * (v[nd, 1] - v[nd, 0])
                + nudge[nd, None] * size[nd, None] * rng.normal(size=(nd.sum(), 3)))
    # points: near a vertex, near an edge, over the face, or far away
    kind = rng.integers(0, 4, n)
    w = rng.dirichlet([1, 1, 1], n)
    face_pt = (w[:, :, None] * v).sum(1)
    k = rng.integers(0, 3, n)
    a, b = v[np.arange(n), k], v[np.arange(n), (k + 1) % 3]
    edge_pt = a + rng.random(n)[:, None] * (b - a)
    vert_pt = v[np.arange(n), k]
    base = np.where((kind == 0)[:, None], vert_pt, np.where((kind == 1)[:, None], edge_pt, face_pt))
    off = 10.0 ** rng.uniform(-12, 0, n)
    off = np.where(kind == 3, 10.0 ** rng.uniform(0.5, 3, n), off)
    p = base + (off * size)[:, None] * rng.normal(size=(n, 3))
    return v, p


def _fr(x):
    return Fraction(float(x))


def test_bound_never_exceeds_fp64_distance(oracle, cbound):
    rng = np.random.default_rng(2024)
    v, p = _cases(rng, 12000)
    pl = cbound(v)
    max_abs = np.abs(v).max((1, 2)).astype(np.float32)  # the smallest a tree's bound could be
    sv, pabs = skip_value(pl, p, max_abs)
    dd = np.empty(len(v))
    for i in range(len(v)):
        r = oracle.closest_on_tri(v[i].reshape(9), p[i])
        w = r - p[i]
        dd[i] = np.sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2])
    fin = np.isfinite(sv)
    assert fin.mean() > 0.9
    bad = np.nonzero(fin & (sv.astype(np.float64) > dd))[0]
    assert len(bad) == 0, f"bound above the distance at {bad[:5]}: {sv[bad[:3]]} vs {dd[bad[:3]]}"

    # useful: for far points the bound is within 10 % of the distance for
    # half of them (beyond a sharp vertex the largest edge distance
    # underestimates), above half of it for nine in ten
    size = np.abs(v - v.mean(1, keepdims=True)).max((1, 2))
    far = fin & (dd > 30 * size) & (dd > 1e3 * U * (pabs.astype(np.float64) + max_abs))
    assert far.sum() > 1000
    ratio = sv[far] / dd[far]
    assert np.median(ratio) >= 0.9 and np.percentile(ratio, 10) >= 0.5


def shaped_flag(v):
    """The FP32 record's flag (k_tri_gather): |e1 x e2|^2 >= 1e-6 |e1|^2
    |e2|^2 in the FP64 operations of the build."""
    e1 = v[:, 1] - v[:, 0]
    e2 = v[:, 2] - v[:, 0]
    ss = e1[:, 0] * e1[:, 0] + e1[:, 1] * e1[:, 1] + e1[:, 2] * e1[:, 2]
    tt = e2[:, 0] * e2[:, 0] + e2[:, 1] * e2[:, 1] + e2[:, 2] * e2[:, 2]
    st = e1[:, 0] * e2[:, 0] + e1[:, 1] * e2[:, 1] + e1[:, 2] * e2[:, 2]
    with np.errstate(all="ignore"):
        det = ss * tt - st * st
        return (ss * tt > 0) & (ss * tt < 1e300) & (det >= 1e-6 * (ss * tt))


def upper_value(pl, v, p, max_abs, edge_check=True, weights=None):
    """closest_upper_of (queries.cu) restated: the FP32 distance from p to
    the projection of p onto the triangle clamped into it, from the FP32
    record (v0 and the FP64 edges rounded to nearest), times 1 + 8u plus the
    margin, rounded up; given where the triangle is well shaped and p is
    inside edge plane 0 or 1 by the margin, else +inf.  Also returns the
    clamped weights."""
    F = np.float32
    h, s0, s1, s2 = plane_dists32(pl, p)
    pabs = np.abs(p.astype(F)).max(1)
    cmargin = (F(48) * U) * (pabs + max_abs)
    A = v[:, 0].astype(F)
    B = (v[:, 1] - v[:, 0]).astype(F)
    C = (v[:, 2] - v[:, 0]).astype(F)
    pf = p.astype(F)
    with np.errstate(all="ignore"):
        ok = shaped_flag(v) & (h >= 0) & (cmargin > 0)
        if edge_check:
            ok &= np.minimum(s0, s1) <= -cmargin
        w = pf - A
        dot = lambda a, b: a[:, 0] * b[:, 0] + a[:, 1] * b[:, 1] + a[:, 2] * b[:, 2]  # noqa: E731
        d11, d12, d22 = dot(B, B), dot(B, C), dot(C, C)
        w1, w2 = dot(w, B), dot(w, C)
        den = d11 * d22 - d12 * d12
        if weights is None:
            s, t = (d22 * w1 - d12 * w2) / den, (d11 * w2 - d12 * w1) / den
        else:
            s, t = weights(A, B, C, pf)
        s = np.fmax(s, F(0))
        t = np.fmax(t, F(0))
        over = ~(fma32_up(s, F(1), t) <= F(1))
        s2w = np.fmin(s / (s + t), F(1))
        t2w = f32_dir(F(1) - s2w.astype(np.float64), up=False)
        s = np.where(over, s2w, s).astype(F)
        t = np.where(over, t2w, t).astype(F)
        q = np.stack([fma32(t, C[:, k], fma32(s, B[:, k], A[:, k])) for k in range(3)], 1)
        d = pf - q
        d32 = np.sqrt(d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1] + d[:, 2] * d[:, 2])
        ub = fma32_up(d32, F(1) + F(8) * U, cmargin)
    return np.where(ok, ub, F(np.inf)).astype(F), s, t


def test_upper_bound_never_below_fp64_distance(oracle, cbound):
    """closest's FP32 upper bound (closest_upper_of), which prunes like a
    best distance while the exact tests wait, is never below the distance
    the exact FP64 test (closest.cpp:54-183, through the oracle) gives for
    the same triangle -- although that test returns a point off the
    triangle in its region six, where a bound from the geometry alone fails
    (checked below) -- its weights are a point of the triangle, and it is
    tight and given for most points over a triangle's face."""
    rng = np.random.default_rng(31)
    v, p = _cases(rng, 12000)
    # degenerate triangles too: repeated vertices, collinear, a point
    v[:40, 1] = v[:40, 0]
    v[40:80, 2] = 2 * v[40:80, 1] - v[40:80, 0]
    v[80:100, 1:] = v[80:100, :1]
    n = len(v)
    # points over the face (a third of them near an edge), and points in
    # v1's wedge beyond edges v0v1 and v1v2 (region six), near its sides
    w = rng.dirichlet([2, 2, 2], n)
    ne = rng.random(n) < 0.33
    w[ne, rng.integers(0, 3, ne.sum())] = 10.0 ** rng.uniform(-9, -2, ne.sum())
    w /= w.sum(1, keepdims=True)
    foot = (w[:, :, None] * v).sum(1)
    nrm = np.cross(v[:, 1] - v[:, 0], v[:, 2] - v[:, 0])
    with np.errstate(all="ignore"):
        nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    size = np.abs(v - v.mean(1, keepdims=True)).max((1, 2))
    over = foot + nrm * (size * 10.0 ** rng.uniform(-3, 1, n))[:, None]
    over = np.where(np.isfinite(over), over, p)
    a = rng.uniform(-1.0, 1e-6, n)           # weight of v2, at or below 0
    b = 1.0 + 10.0 ** rng.uniform(-9, 0, n)  # weights of v1 and v2 summing above 1
    six = v[:, 0] + (b - a)[:, None] * (v[:, 1] - v[:, 0]) + a[:, None] * (v[:, 2] - v[:, 0])
    six = six + nrm * (size * 10.0 ** rng.uniform(-6, 0, n))[:, None]
    six = np.where(np.isfinite(six), six, p)
    v = np.concatenate([v, v, v])
    p = np.concatenate([p, over, six])
    pl = cbound(v)
    max_abs = np.abs(v).max((1, 2)).astype(np.float32)
    ub, s, t = upper_value(pl, v, p, max_abs)
    assert ((s >= 0) & (t >= 0)).all()
    assert all(Fraction(float(x)) + Fraction(float(y)) <= 1 for x, y in zip(s, t))
    dd = np.empty(len(v))
    for i in range(len(v)):
        r = oracle.closest_on_tri(v[i].reshape(9), p[i])
        d = r - p[i]
        dd[i] = np.sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2])
    fin = np.isfinite(ub)
    bad = np.nonzero(fin & ~(ub.astype(np.float64) >= dd))[0]
    assert len(bad) == 0, f"bound below the distance at {bad[:5]}: {ub[bad[:3]]} vs {dd[bad[:3]]}"
    for k in range(3):  # degenerate triangles: no bound
        assert not fin[k * n:k * n + 100].any()
    # region six is where the exact test is off: the same geometric bound
    # without the edge condition fails there
    geo = upper_value(pl, v, p, max_abs, edge_check=False)[0]
    assert (geo[2 * n:].astype(np.float64) < dd[2 * n:]).sum() >= 5
    # given for most of the points over well-shaped faces that are large
    # against the margin, away from the edges, and within 1e-5 (|p| + M)
    half = slice(n, 2 * n)
    big = size > 1e-3 * (np.abs(p[half]).max(1) + max_abs[half])
    good = big & shaped_flag(v[half]) & np.isfinite(pl[half, 0, 3]) & ~ne
    assert good.sum() > 2000 and fin[half][good].mean() > 0.9
    slack = (ub[half][fin[half]].astype(np.float64) - dd[half][fin[half]]) / (
        np.abs(p[half][fin[half]]).max(1) + max_abs[half][fin[half]])
    assert np.median(slack) < 1e-5
    # and the exact test does leave the triangle in region six here
    sx = slice(2 * n, 3 * n)
    assert (dd[sx] > 1.01 * np.linalg.norm(p[sx] - v[sx, 1], axis=1)).sum() > 100


def box_lower_value(v, p, max_abs):
    """The box bound of closest_record_bounds (queries.cu) restated: the
    FP32 distance from p to the box of the vertices rebuilt from the FP32
    record (A, A + B, A + C), times 1 - 8u, less the margin."""
    F = np.float32
    A = v[:, 0].astype(F)
    B = (v[:, 1] - v[:, 0]).astype(F)
    C = (v[:, 2] - v[:, 0]).astype(F)
    V1, V2 = A + B, A + C
    lo = np.minimum(np.minimum(A, V1), V2)
    hi = np.maximum(np.maximum(A, V1), V2)
    pf = p.astype(F)
    with np.errstate(all="ignore"):
        e = np.maximum(np.maximum(lo - pf, pf - hi), F(0))
        d = np.sqrt(e[:, 0] * e[:, 0] + e[:, 1] * e[:, 1] + e[:, 2] * e[:, 2])
        cmargin = (F(48) * U) * (np.abs(pf).max(1) + max_abs)
        return d * (F(1) - F(8) * U) - cmargin


def test_box_lower_bound_never_exceeds_fp64_distance(oracle):
    """closest's second lower bound (the triangle's box, closest_record_bounds)
    never exceeds the exact FP64 test's distance (closest.cpp:54-183), in
    particular in region six, where that test's point is off the triangle;
    and it is tight for points far from small triangles."""
    rng = np.random.default_rng(44)
    v, p = _cases(rng, 12000)
    n = len(v)
    nrm = np.cross(v[:, 1] - v[:, 0], v[:, 2] - v[:, 0])
    with np.errstate(all="ignore"):
        nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    size = np.abs(v - v.mean(1, keepdims=True)).max((1, 2))
    a = rng.uniform(-3.0, 1e-6, n)
    b = 1.0 + 10.0 ** rng.uniform(-9, 0.5, n)
    six = v[:, 0] + (b - a)[:, None] * (v[:, 1] - v[:, 0]) + a[:, None] * (v[:, 2] - v[:, 0])
    six = six + nrm * (size * rng.uniform(-2, 2, n))[:, None]
    six = np.where(np.isfinite(six), six, p)
    v = np.concatenate([v, v])
    p = np.concatenate([p, six])
    max_abs = np.abs(v).max((1, 2)).astype(np.float32)
    lo = box_lower_value(v, p, max_abs)
    dd = np.empty(len(v))
    for i in range(len(v)):
        r = oracle.closest_on_tri(v[i].reshape(9), p[i])
        d = r - p[i]
        dd[i] = np.sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2])
    fin = np.isfinite(lo) & np.isfinite(dd)
    assert fin.mean() > 0.99
    bad = np.nonzero(fin & (lo.astype(np.float64) > dd))[0]
    assert len(bad) == 0, f"bound above the distance at {bad[:5]}: {lo[bad[:3]]} vs {dd[bad[:3]]}"
    size = np.concatenate([size, size])
    far = fin & (dd > 100 * size) & (dd > 1e3 * U * (np.abs(p).max(1) + max_abs))
    assert far.sum() > 500 and np.median(lo[far] / dd[far]) > 0.95


def test_plane_certificates_exact(cbound):
    """What the proof uses, in exact rational arithmetic on a sample: the face
    slab, the edge planes holding every vertex, near-orthonormal rows, and the
    FP32 evaluation within 8 u (|p| + M) of the exact plane distances."""
    rng = np.random.default_rng(77)
    v, p = _cases(rng, 1500)
    pl = cbound(v)
    ok = np.isfinite(pl[:, 0, 3])
    assert ok.mean() > 0.9
    u = Fraction(1, 2 ** 24)
    ev = plane_dists32(pl, p)
    max_abs = np.abs(v).max((1, 2)).astype(np.float32)
    pabs = np.abs(p.astype(np.float32)).max(1)
    for i in np.nonzero(ok)[0]:
        V = [[_fr(x) for x in v[i, k]] for k in range(3)]
        vmax = max(abs(x) for row in V for x in row)
        P = [[_fr(x) for x in pl[i, k]] for k in range(4)]
        n, d = P[0][:3], P[0][3]
        dot = lambda a, b: a[0] * b[0] + a[1] * b[1] + a[2] * b[2]  # noqa: E731
        for Vk in V:
            assert abs(dot(n, Vk) - d) <= 7 * u * vmax * (1 + Fraction(1, 10 ** 9)), i
        assert dot(n, n) <= (1 + 4 * u) ** 2
        for k in (1, 2, 3):
            m, c = P[k][:3], P[k][3]
            assert all(dot(m, Vq) <= c for Vq in V), (i, k)
            assert dot(m, m) <= (1 + 4 * u) ** 2 and abs(dot(n, m)) <= 4 * u, (i, k)
        pe = [_fr(x) for x in p[i]]
        lim = 8 * u * (_fr(pabs[i]) + _fr(max_abs[i]))
        assert abs(_fr(ev[0][i]) - abs(dot(n, pe) - d)) <= lim, i
        for k in (1, 2, 3):
            assert abs(_fr(ev[k][i]) - (dot(P[k][:3], pe) - P[k][3])) <= lim, (i, k)


def test_degenerate_triangles_never_skip(cbound):
    v = np.array([[[0, 0, 0], [1, 1, 1], [2, 2, 2]],      # collinear
                  [[1, 2, 3], [1, 2, 3], [4, 5, 6]],      # repeated vertex
                  [[5, 5, 5], [5, 5, 5], [5, 5, 5]],      # a point
                  [[0, 0, 0], [1, 0, 0], [np.nan, 1, 0]],  # NaN
                  [[0, 0, 0], [1e31, 0, 0], [0, 1, 0]]],   # beyond 1e30
                 dtype=np.float64)
    pl = cbound(v)
    assert np.isnan(pl[:, 0, 3]).all()
    p = np.array([[100.0, 0, 0], [0, 100.0, 0], [0, 0, 100.0], [3.0, 3, 3], [-5.0, 0, 0]])
    sv, _ = skip_value(pl, p, np.float32(1e30))
    assert not (sv > np.float32(0)).any()


def test_box_bound_never_exceeds_box_distance():
    """closest's FP32 box pruning (k_closest): the distance from the point
    rounded to FP32 to the box rounded outward, computed in FP32 (separate
    products and sums, a correctly rounded root), less 8 u of itself and
    4 u |p|, never exceeds the exact distance from the point to the FP64 box
    (checked as squares in rational arithmetic), so a box holding a triangle
    at the best distance is never pruned."""
    rng = np.random.default_rng(9)
    n = 4000
    scale = 10.0 ** rng.choice([0.0, 3.0, 6.0, 9.0], n)
    c = rng.uniform(-1, 1, (n, 3)) * scale[:, None]
    half = np.abs(rng.normal(size=(n, 3))) * (10.0 ** rng.uniform(-4, 2, n))[:, None]
    lo64, hi64 = c - half, c + half
    # points inside, on a face, just outside, or far out
    k = rng.integers(0, 4, n)
    off = np.where(k[:, None] == 0, 0.0,
                   (10.0 ** rng.uniform(-14, 3, n))[:, None] * np.abs(rng.normal(size=(n, 3))) * half)
    side = rng.choice([-1.0, 1.0], (n, 3))
    p = np.where(side > 0, hi64 + off, lo64 - off)
    p = np.where((k == 0)[:, None], lo64 + rng.random((n, 3)) * (hi64 - lo64), p)
    lo = f32_dir(lo64, up=False)
    hi = f32_dir(hi64, up=True)
    px = p.astype(np.float32)
    pabs = np.abs(px).max(1)
    s = np.zeros(n, dtype=np.float32)
    for ax in range(3):
        e = np.maximum(np.maximum(lo[:, ax] - px[:, ax], px[:, ax] - hi[:, ax]), np.float32(0))
        s = s + e * e
    dist = np.sqrt(s)
    lb = dist * (np.float32(1) - np.float32(8) * U) - (np.float32(4) * U) * pabs
    for i in range(n):
        if lb[i] <= 0:
            continue
        d2 = Fraction(0)
        for ax in range(3):
            q, a, b = Fraction(float(p[i, ax])), Fraction(float(lo64[i, ax])), Fraction(float(hi64[i, ax]))
            e = max(a - q, q - b, Fraction(0))
            d2 += e * e
        assert Fraction(float(lb[i])) ** 2 <= d2, i
    assert (lb > 0).sum() > 500  # (at 1e9 from the origin the 4 u |p| term dominates)

