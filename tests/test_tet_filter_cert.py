"""The FP32 containment pre-filter of find_element (`tet_filter32` in
geom.cuh, its per-tet record from `k_tet_gather` in api.cu) only answers
where the FP64 test (tetrahedron_contain.cpp:11-43 through the oracle) gives
the same answer: a certified inside is inside for the FP64 test, a certified
outside is outside, and everything else takes the FP64 test.

Both are restated here in numpy: the record in FP64 with the kernel's
operation order (the kernels compile with -fmad=false) and its FP32
roundings (to nearest, and upward for the two bounds), the filter in IEEE
FP32 with the kernel's operation order.  Cases: tets of sizes 1e-4..1e2 up
to 1e6 from the origin, regular, slivers (the fourth vertex 1e-2..1e-9 of
the size off the plane of the other three), needles and caps, with points
inside, just inside and just outside faces (barycentric margins down to
1e-14), near vertices and edges, anywhere in the tet's dilated box, and up
to 1000 tet sizes away (what an FP32 box rounded outward admits).
"""
import numpy as np

from fp32_emul import F, U, f32_dir


def tet_records(v):
    """v: (n, 4, 3) FP64 -> (n, 4, 4) FP32 records (v0, m), (M0, |v0|),
    (M1, e64), (M2, 0) as k_tet_gather writes them."""
    v0 = v[:, 0]
    T = np.empty((len(v), 3, 3))
    for r in range(3):
        for c in range(3):
            T[:, r, c] = v[:, c + 1, r] - v0[:, r]
    Tmax = np.abs(T).max((1, 2))
    lo, hi = v.min(1), v.max(1)
    t = lambda r, c: T[:, r, c]  # noqa: E731
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        det = (t(0, 0) * (t(1, 1) * t(2, 2) - t(1, 2) * t(2, 1))
               - t(0, 1) * (t(1, 0) * t(2, 2) - t(1, 2) * t(2, 0))
               + t(0, 2) * (t(1, 0) * t(2, 1) - t(1, 1) * t(2, 0)))
        M = np.empty((len(v), 3, 3))
        M[:, 0, 0] = (t(1, 1) * t(2, 2) - t(1, 2) * t(2, 1)) / det
        M[:, 0, 1] = (t(0, 2) * t(2, 1) - t(0, 1) * t(2, 2)) / det
        M[:, 0, 2] = (t(0, 1) * t(1, 2) - t(0, 2) * t(1, 1)) / det
        M[:, 1, 0] = (t(1, 2) * t(2, 0) - t(1, 0) * t(2, 2)) / det
        M[:, 1, 1] = (t(0, 0) * t(2, 2) - t(0, 2) * t(2, 0)) / det
        M[:, 1, 2] = (t(0, 2) * t(1, 0) - t(0, 0) * t(1, 2)) / det
        M[:, 2, 0] = (t(1, 0) * t(2, 1) - t(1, 1) * t(2, 0)) / det
        M[:, 2, 1] = (t(0, 1) * t(2, 0) - t(0, 0) * t(2, 1)) / det
        M[:, 2, 2] = (t(0, 0) * t(1, 1) - t(0, 1) * t(1, 0)) / det
        m = np.zeros(len(v))
        for r in range(3):
            m = np.fmax(m, np.abs(M[:, r, 0]) + np.abs(M[:, r, 1]) + np.abs(M[:, r, 2]))
        rmax = np.zeros(len(v))
        for r in range(3):
            rmax = np.fmax(rmax, np.fmax(np.abs(hi[:, r] - v0[:, r]), np.abs(v0[:, r] - lo[:, r])))
        w = np.sqrt((hi[:, 0] - lo[:, 0]) * (hi[:, 0] - lo[:, 0]) + (hi[:, 1] - lo[:, 1]) * (hi[:, 1] - lo[:, 1])
                    + (hi[:, 2] - lo[:, 2]) * (hi[:, 2] - lo[:, 2]))
        rmax = rmax + 2.0 * w * 1e-6 + 1e-300
        krel = Tmax * Tmax * Tmax / np.abs(det)
        eps = np.finfo(np.float64).eps
        e64 = 3.0 * eps * rmax * (18.0 * krel / Tmax + 47.0 * krel * m) + 3.0 * eps * (1.0 + 3.0 * m * rmax)
        e64 = e64 * 2.0
        ok = (det > 0) & np.isfinite(det) & (m < 1e20) & (krel < 1e6) & np.isfinite(e64)
        rec = np.zeros((len(v), 4, 4), dtype=np.float32)
        rec[:, 0, :3] = v0.astype(np.float32)
        rec[:, 0, 3] = np.where(ok, f32_dir(np.where(ok, m * (1.0 + 1e-6), 0.0), up=True), np.inf)
        rec[:, 1, :3] = M[:, 0].astype(np.float32)
        rec[:, 1, 3] = np.abs(rec[:, 0, :3]).max(1)
        rec[:, 2, :3] = M[:, 1].astype(np.float32)
        rec[:, 2, 3] = np.where(ok, f32_dir(np.where(ok, e64, 0.0), up=True), np.inf)
        rec[:, 3, :3] = M[:, 2].astype(np.float32)
    return rec, lo - (w * 1e-6)[:, None], hi + (w * 1e-6)[:, None]


def tet_filter32(rec, p):
    """1 certified inside, -1 certified outside, 0 undecided (FP32)."""
    px = p.astype(np.float32)
    pabs = np.abs(px).max(1)
    f0, f1, f2, f3 = rec[:, 0], rec[:, 1], rec[:, 2], rec[:, 3]
    m = f0[:, 3]
    with np.errstate(invalid="ignore", over="ignore"):
        r = px - f0[:, :3]
        R = np.abs(r).max(1)
        dot = lambda f: (f[:, 0] * r[:, 0] + f[:, 1] * r[:, 1]) + f[:, 2] * r[:, 2]  # noqa: E731
        l1, l2, l3 = dot(f1), dot(f2), dot(f3)
        l0 = F(1) - ((l1 + l2) + l3)
        sl = (np.abs(l1) + np.abs(l2)) + np.abs(l3)
        E = ((U * ((F(16) * m) * ((R + pabs) + f1[:, 3]) + F(4) * (F(1) + sl))) * F(1.0001)
             + f2[:, 3]) + F(4.5e-15)
        lmin = np.minimum(np.minimum(l0, l1), np.minimum(l2, l3))
        lmax = np.maximum(np.maximum(l0, l1), np.maximum(l2, l3))
        out = np.zeros(len(p), dtype=np.int32)
        out[(lmin < -E) | (lmax > F(1) + E)] = -1
        inside = (lmin >= E) & (lmax <= F(1) - E)
        out[inside & (out == 0)] = 1
    out[~(m < np.inf)] = 0
    return out


def _tets(rng, n):
    scale = 10.0 ** rng.choice([0.0, 2.0, 4.0, 6.0], n)
    size = 10.0 ** rng.uniform(-4, 2, n)
    c = rng.uniform(-1, 1, (n, 3)) * scale[:, None]
    v = c[:, None, :] + rng.normal(size=(n, 4, 3)) * size[:, None, None]
    kind = rng.integers(0, 4, n)
    # slivers: the fourth vertex close to the plane of the first three
    s = kind == 1
    w = rng.dirichlet([1, 1, 1], s.sum())
    base = (w[:, :, None] * v[s, :3]).sum(1)
    nrm = np.cross(v[s, 1] - v[s, 0], v[s, 2] - v[s, 0])
    nrm /= np.linalg.norm(nrm, axis=1)[:, None]
    h = 10.0 ** rng.uniform(-9, -2, s.sum()) * size[s]
    v[s, 3] = base + (h * rng.choice([-1, 1], s.sum()))[:, None] * nrm
    # needles: three vertices close to a line
    nd = kind == 2
    d = rng.normal(size=(nd.sum(), 3))
    for k in (1, 2, 3):
        v[nd, k] = (v[nd, 0] + rng.uniform(0.2, 1, nd.sum())[:, None] * d * size[nd, None] * k
                    + (10.0 ** rng.uniform(-6, -2, nd.sum()) * size[nd])[:, None] * rng.normal(size=(nd.sum(), 3)))
    # positive orientation, as the mesh stores it
    T = v[:, 1:] - v[:, :1]
    neg = np.linalg.det(T) < 0
    v[neg, 1], v[neg, 2] = v[neg, 2].copy(), v[neg, 1].copy()
    return v


def _points(rng, v, lo, hi):
    n = len(v)
    kind = rng.integers(0, 5, n)
    b = rng.dirichlet([1, 1, 1, 1], n)
    # near a face: one barycentric coordinate at +-1e-k
    f = rng.integers(0, 4, n)
    mar = rng.choice([-1, 1], n) * 10.0 ** rng.uniform(-14, -2, n)
    near = b.copy()
    near[np.arange(n), f] = mar
    near /= near.sum(1)[:, None]
    # near a vertex or an edge
    vert = np.zeros((n, 4))
    vert[np.arange(n), f] = 1.0
    vert += 10.0 ** rng.uniform(-14, -3, n)[:, None] * rng.normal(size=(n, 4))
    edge = np.zeros((n, 4))
    g = (f + 1) % 4
    a = rng.random(n)
    edge[np.arange(n), f] = a
    edge[np.arange(n), g] = 1 - a
    edge += 10.0 ** rng.uniform(-14, -3, n)[:, None] * rng.normal(size=(n, 4))
    bary = np.where((kind == 0)[:, None], b, np.where((kind == 1)[:, None], near,
                    np.where((kind == 2)[:, None], vert, edge)))
    p = (bary[:, :, None] * v).sum(1)
    box = lo + rng.random((n, 3)) * (hi - lo)
    p = np.where((kind == 4)[:, None], box, p)
    # up to 1000 tet sizes away: a tiny tet far from the origin has an FP32
    # box (rounded outward) far wider than itself, and the filter sees every
    # point inside that box
    far = rng.random(n) < 0.15
    size = np.abs(v - v.mean(1, keepdims=True)).max((1, 2))
    return np.where(far[:, None], v.mean(1) + (10.0 ** rng.uniform(0, 3, n) * size)[:, None]
                    * rng.uniform(-1, 1, (n, 3)), p)


def test_filter_agrees_with_fp64_test(oracle):
    rng = np.random.default_rng(31)
    n = 20000
    v = _tets(rng, n)
    rec, lo, hi = tet_records(v)
    p = _points(rng, v, lo, hi)
    c = tet_filter32(rec, p)
    ref = np.array([oracle.tet_contains(p[i], v[i].reshape(12)) for i in range(n)])
    wrong_in = np.nonzero((c == 1) & ~ref)[0]
    wrong_out = np.nonzero((c == -1) & ref)[0]
    assert len(wrong_in) == 0, f"certified inside, FP64 outside: {wrong_in[:5]}"
    assert len(wrong_out) == 0, f"certified outside, FP64 inside: {wrong_out[:5]}"
    assert (c == 1).sum() > 1000 and (c == -1).sum() > 1000


def test_filter_decides_ordinary_cases():
    """On tets of sizes 0.1..10 within 10 of the origin, points well inside
    are certified inside and points a tet size away certified outside."""
    rng = np.random.default_rng(8)
    n = 5000
    size = 10.0 ** rng.uniform(-1, 1, n)
    v = rng.uniform(-10, 10, (n, 1, 3)) + rng.normal(size=(n, 4, 3)) * size[:, None, None]
    T = v[:, 1:] - v[:, :1]
    neg = np.linalg.det(T) < 0
    v[neg, 1], v[neg, 2] = v[neg, 2].copy(), v[neg, 1].copy()
    rec, _, _ = tet_records(v)
    b = 0.05 + 0.8 * rng.dirichlet([2, 2, 2, 2], n)
    b /= b.sum(1)[:, None]
    inside = tet_filter32(rec, (b[:, :, None] * v).sum(1))
    assert (inside == 1).mean() > 0.9
    far = v.mean(1) + 3 * size[:, None] * synth_dirs(rng, n)
    assert (tet_filter32(rec, far) == -1).mean() > 0.9


def synth_dirs(rng, n):
    d = rng.normal(size=(n, 3))
    return d / np.linalg.norm(d, axis=1)[:, None]
