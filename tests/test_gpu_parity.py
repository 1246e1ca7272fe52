"""Parity of the CUDA engine with the CPU oracle on seeded synthetic models.

Integer results (surface / face / element ids, inside flags, segment counts
and sequences) must match exactly; distances must match bit for bit (both
paths evaluate the reference's FP64 formulas in the same order), which is
stricter than the 1e-12 relative tolerance the benchmark configurations ask
for.  The sizes are scaled-down versions of the benchmark configurations so
the oracle finishes in seconds.
"""
import numpy as np
import pytest

from xdg_gb300 import synth
from xdg_gb300.engine import ANY, ENTERING, EXITING, FP64, MIXED, XDG, CudaRayTracer

pytestmark = pytest.mark.gpu

PRECISIONS = [FP64, MIXED]


def assert_same(a, b, what):
    a = np.asarray(a)
    b = np.asarray(b)
    bad = np.nonzero(a != b)[0] if a.ndim == 1 else np.nonzero((a != b).any(axis=1))[0]
    assert len(bad) == 0, f"{what}: {len(bad)} mismatches, first at {bad[:5]}: {a[bad[:3]]} vs {b[bad[:3]]}"


@pytest.fixture(scope="module")
def sphere_box():
    m = synth.single_sphere_in_box(level=4, radius=10.0, half_width=20.0)
    x = XDG(m)
    x.prepare_raytracer()
    return m, x


@pytest.mark.parametrize("prec", PRECISIONS)
def test_ray_fire_sphere(cuda, oracle, sphere_box, prec):
    """ray_fire in the sphere volume: lcg rays from a ball of radius 9.9."""
    m, x = sphere_box
    o, d = synth.lcg_ball_rays(20000, 9.9, seed=12345)
    t, s, f = x.ray_fire(1, o, d, precision=prec)
    ot, os_, of = oracle.volume_tree(m, 1).ray_fire(o, d)
    assert_same(s, os_, "surface")
    assert_same(f, of, "face")
    assert_same(t, ot, "t")
    assert (s == 1).all()


@pytest.mark.parametrize("prec", PRECISIONS)
def test_ray_fire_orientations_and_limits(cuda, oracle, sphere_box, prec):
    m, x = sphere_box
    rng = np.random.default_rng(5)
    o = rng.uniform(-25, 25, (20000, 3))
    d = synth.isotropic_dirs(rng, 20000)
    dl = rng.uniform(0, 40, 20000)
    ot2 = oracle.volume_tree(m, 2)
    for orient in (EXITING, ENTERING, ANY):
        t, s, f = x.ray_fire(2, o, d, dl, orient, precision=prec)
        ot, os_, of = ot2.ray_fire(o, d, dl, orient)
        assert_same(s, os_, f"surface orient={orient}")
        assert_same(f, of, f"face orient={orient}")
        assert_same(t, ot, f"t orient={orient}")


@pytest.mark.parametrize("prec", PRECISIONS)
def test_exclusions(cuda, oracle, sphere_box, prec):
    """Re-firing with the hit face excluded (the reference's surface-crossing loop)."""
    m, x = sphere_box
    o, d = synth.lcg_ball_rays(5000, 9.9, seed=99)
    t, s, f = x.ray_fire(1, o, d, precision=prec)
    excl = [[int(ff)] for ff in f]
    p = o + d * t[:, None]
    t2, s2, f2 = x.ray_fire(1, p, d, exclude=excl, precision=prec)
    ot, os_, of = oracle.volume_tree(m, 1).ray_fire(p, d, excl=excl)
    assert_same(s2, os_, "surface")
    assert_same(f2, of, "face")
    assert_same(t2, ot, "t")


@pytest.mark.parametrize("prec", PRECISIONS)
def test_piv_occluded_closest_sphere(cuda, oracle, sphere_box, prec):
    m, x = sphere_box
    rng = np.random.default_rng(8)
    p = rng.uniform(-22, 22, (20000, 3))
    d = synth.isotropic_dirs(rng, 20000)
    for vol in (1, 2, 3):
        ot = oracle.volume_tree(m, vol)
        assert_same(x.point_in_volume(vol, p, precision=prec), ot.point_in_volume(p), f"piv default dir vol {vol}")
        assert_same(x.point_in_volume(vol, p, d, precision=prec), ot.point_in_volume(p, d), f"piv vol {vol}")
        occ, dist = x.occluded(vol, p, d, prec)
        oocc, odist = ot.occluded(p, d)
        assert_same(occ, oocc, "occluded")
        assert_same(dist, odist, "occluded distance")
        cd, cf = x.closest(vol, p[:4000], prec)
        ocd, ocf = ot.closest(p[:4000])
        assert_same(cf, ocf, "closest face")
        assert_same(cd, ocd, "closest distance")


@pytest.mark.parametrize("prec", PRECISIONS)
def test_nested_spheres_per_ray_trees(cuda, oracle, prec):
    """Scaled-down nested-sphere configuration: find_volume, then ray_fire in
    the found volume with one tree per ray, and point_in_volume."""
    m = synth.nested_spheres(n=8, level=3, jitter=1e-3, seed=7)
    x = XDG(m)
    x.prepare_raytracer()
    rng = np.random.default_rng(2)
    n = 20000
    p = rng.uniform(-9, 9, (n, 3))
    d = synth.isotropic_dirs(rng, n)
    vols = x.find_volume(p, d, precision=prec)
    # oracle find_volume, ascending volume order
    ovol = np.full(n, m.implicit_complement, dtype=np.int32)
    todo = np.arange(n)
    trees = {v: oracle.volume_tree(m, v) for v in m.volumes}
    for v in sorted(m.volumes):
        if v == m.implicit_complement:
            continue
        ins = trees[v].point_in_volume(p[todo], d[todo]).astype(bool)
        ovol[todo[ins]] = v
        todo = todo[~ins]
    assert_same(vols, ovol, "find_volume")
    t, s, f = x.ray_fire(vols, p, d, precision=prec)
    for v in m.volumes:
        sel = np.nonzero(vols == v)[0]
        if len(sel) == 0:
            continue
        ot, os_, of = trees[v].ray_fire(p[sel], d[sel])
        assert_same(s[sel], os_, f"surface vol {v}")
        assert_same(t[sel], ot, f"t vol {v}")


@pytest.mark.parametrize("prec", PRECISIONS)
def test_watertight_stress(cuda, oracle, prec):
    """Scaled-down degenerate-hit configuration: rays from inside aimed at
    vertices, edge midpoints and centroids with 1e-12..1e-6 jitter.  Every ray
    must hit (closed surface), and agree with the oracle."""
    v, tri = synth.icosphere(4, 5.0)
    s = synth.Surface(1, v, tri, np.arange(len(tri), dtype=np.int32), 1, 2)
    m = synth.Model(surfaces=[s], volumes=[1, 2], implicit_complement=2)
    x = XDG(m)
    x.prepare_raytracer()
    rng = np.random.default_rng(17)
    n = 30000
    o = synth.lcg_ball_rays(n, 4.9, seed=4)[0]
    kind = rng.uniform(0, 1, n)
    ti = rng.integers(0, len(tri), n)
    corners = v[tri[ti]]
    target = corners.mean(1)
    vi = kind < 0.4
    target[vi] = corners[vi, rng.integers(0, 3, vi.sum())]
    ei = (kind >= 0.4) & (kind < 0.8)
    a = rng.integers(0, 3, ei.sum())
    target[ei] = 0.5 * (corners[ei, a] + corners[ei, (a + 1) % 3])
    jit = 10.0 ** rng.uniform(-12, -6, n)
    target += synth.isotropic_dirs(rng, n) * jit[:, None]
    d = synth.normalize_rows(target - o)
    t, s_, f = x.ray_fire(1, o, d, precision=prec)
    assert (s_ == 1).all(), f"{(s_ != 1).sum()} lost hits"
    ot, os_, of = oracle.volume_tree(m, 1).ray_fire(o, d)
    assert_same(f, of, "face")
    assert_same(t, ot, "t")


@pytest.fixture(scope="module")
def tet_model():
    tm = synth.tet_cube(n=8, size=10.0, jitter=0.2, seed=11)
    return tm


@pytest.mark.parametrize("prec", PRECISIONS)
@pytest.mark.parametrize("settings", [{}, {"walk_edge_table": 0},
                                      {"walk_queue": 0}, {"walk_queue": 0, "walk_edge_table": 0}])
def test_find_element_and_walk_tet_cube(cuda, oracle, tet_model, prec, settings):
    """Scaled-down tet-walk configuration: find_element then the face-adjacency
    walk; element sequences and lengths bit-identical to the oracle, with the
    mixed walk's FP64 edge coordinates from the mesh's edge table or from the
    vertices, through the per-warp FP64 queue or per lane."""
    tm = tet_model
    rti = CudaRayTracer()
    rti.set_tet_mesh(tm)
    assert rti.get_tuning("walk_edges") > len(tm.conn)
    for k, v in settings.items():
        rti.set_tuning(k, v)
    m = synth.Model(volumes=[1], tets=tm, elements={1: np.arange(len(tm.conn), dtype=np.int32)})
    et = rti.create_element_tree(m, 1)
    rng = np.random.default_rng(23)
    n = 4000
    start = rng.uniform(0, 10, (n, 3))
    u = synth.isotropic_dirs(rng, n)
    length = np.minimum(rng.exponential(5.0, n), _exit_distance(start, u, 0.0, 10.0))
    eid, eidx = rti.find_element(et, start, prec)
    oid, oidx = oracle.TetTree(tm.tet_xyz(), tm.elem_ids).find_element(start)
    assert_same(eid, oid, "find_element id")
    assert_same(eidx, oidx, "find_element index")
    ok = eidx >= 0
    se, sl, sc, st = rti.walk_elements(eidx[ok], start[ok], u[ok], length[ok], 512, prec)
    w = oracle.TetWalker(tm.vertices, tm.conn, tm.adj, tm.face_table)
    oe, ol, oc, ost = w.walk(oidx[ok], start[ok], u[ok], length[ok], 512)
    assert_same(sc, oc, "segment counts")
    assert_same(st, ost, "status")
    for k in range(len(sc)):
        c = sc[k]
        assert np.array_equal(se[k, :c], tm.elem_ids[oe[k, :c]]), f"track {k} elements"
        assert np.array_equal(sl[k, :c], ol[k, :c]), f"track {k} lengths"


@pytest.mark.parametrize("prec", PRECISIONS)
def test_walk_degenerate_tracks(cuda, oracle, prec):
    """Tracks through the vertices and along the edges and faces of an
    unjittered tet cube (every coordinate a multiple of the cell size):
    along grid lines, across cell diagonals, starting on vertices and faces.
    Zero Plucker coordinates, ties between faces and zero-length segments are
    the rule here; elements, lengths and statuses must equal the oracle's,
    with the mixed walk's edge coordinates from the edge table and from the
    vertices."""
    tm = synth.tet_cube(n=6, size=6.0, jitter=0.0, seed=1)
    rng = np.random.default_rng(41)
    starts, dirs = [], []
    g = np.arange(0, 7, dtype=np.float64)
    axes = np.eye(3)
    for _ in range(300):
        p = rng.choice(g, 3)
        p = np.clip(p, 0.0, 6.0)
        kind = rng.integers(0, 4)
        if kind == 0:
            u = axes[rng.integers(0, 3)] * rng.choice([-1.0, 1.0])
        elif kind == 1:
            u = rng.choice([-1.0, 0.0, 1.0], 3)
            if not u.any():
                u = axes[0]
        elif kind == 2:
            p = p + rng.choice([0.0, 0.5], 3)
            u = rng.choice([-1.0, 1.0, 2.0], 3)
        else:
            p = p + rng.uniform(0, 1, 3) * (rng.random(3) < 0.5)
            u = rng.normal(size=3)
        starts.append(np.clip(p, 0.0, 6.0))
        dirs.append(u / np.linalg.norm(u))
    start = np.array(starts)
    u = np.array(dirs)
    rti = CudaRayTracer()
    rti.set_tet_mesh(tm)
    m = synth.Model(volumes=[1], tets=tm, elements={1: np.arange(len(tm.conn), dtype=np.int32)})
    et = rti.create_element_tree(m, 1)
    eid, eidx = rti.find_element(et, start, prec)
    oid, oidx = oracle.TetTree(tm.tet_xyz(), tm.elem_ids).find_element(start)
    assert_same(eidx, oidx, "find_element index")
    ok = eidx >= 0
    assert ok.sum() > 250
    length = np.full(len(start), 20.0)
    w = oracle.TetWalker(tm.vertices, tm.conn, tm.adj, tm.face_table)
    oe, ol, oc, ost = w.walk(oidx[ok], start[ok], u[ok], length[ok], 512)
    for edges in (1, 0):
        rti.set_tuning("walk_edge_table", edges)
        for queue in (0, 1):
            rti.set_tuning("walk_queue", queue)
            se, sl, sc, st = rti.walk_elements(eidx[ok], start[ok], u[ok], length[ok], 512, prec)
            assert_same(sc, oc, f"segment counts (edges {edges}, queue {queue})")
            assert_same(st, ost, f"status (edges {edges}, queue {queue})")
            for k in range(len(sc)):
                c = sc[k]
                assert np.array_equal(se[k, :c], tm.elem_ids[oe[k, :c]]), f"track {k} elements"
                assert np.array_equal(sl[k, :c], ol[k, :c]), f"track {k} lengths"


def _exit_distance(p, u, lo, hi):
    with np.errstate(divide="ignore", invalid="ignore"):
        t1 = (lo - p) / u
        t2 = (hi - p) / u
    tmax = np.where(u > 0, t2, np.where(u < 0, t1, np.inf))
    return tmax.min(axis=1)


def test_host_and_device_paths_agree(cuda, sphere_box):
    """The same query through host (NumPy) and device (torch) pointers."""
    torch = cuda
    m, x = sphere_box
    o, d = synth.lcg_ball_rays(4096, 9.9, seed=1)
    t, s, f = x.ray_fire(1, o, d)
    to = torch.from_numpy(o).cuda()
    td = torch.from_numpy(d).cuda()
    t2, s2, f2 = x.rti.ray_fire(x.volume_to_surface_tree[1], to, td)
    torch.cuda.synchronize()
    assert np.array_equal(t, t2.cpu().numpy())
    assert np.array_equal(s, s2.cpu().numpy())


def test_invalid_inputs(cuda, sphere_box):
    """NaN rays and bad tree ids are reported per ray, not as faults."""
    from xdg_gb300._lib import RAY_INVALID, EngineError
    m, x = sphere_box
    o = np.array([[0, 0, 0], [np.nan, 0, 0], [0, 0, 0]], dtype=np.float64)
    d = np.array([[1, 0, 0], [1, 0, 0], [0, 0, 0]], dtype=np.float64)
    t, s, f, st = x.rti.ray_fire(x.volume_to_surface_tree[1], o, d, status=True)
    assert st[1] == RAY_INVALID and s[1] == -1
    assert st[0] == 0 and s[0] == 1
    assert s[2] == -1  # zero direction: every Plucker coordinate is zero -> no hit
    with pytest.raises(EngineError):
        x.rti.ray_fire(999, o, d)
    t, s, f, st = x.rti.ray_fire(0, o, d, ray_trees=np.array([1, 1, 77], dtype=np.int32),
                                 status=True)
    assert st[2] == RAY_INVALID


@pytest.mark.parametrize("prec", PRECISIONS)
def test_walk_against_reference_vectors(cuda, prec):
    """The engine's walk against the segments the reference's own
    MeshManager::walk_elements produced (tests/golden/make_golden.py)."""
    import os
    from conftest import ROOT
    g = np.load(os.path.join(ROOT, "tests", "golden", "reference_vectors.npz"))
    tm = synth.TetMesh(vertices=g["tw_xyz"], conn=g["tw_conn"], adj=g["tw_adj"],
                       face_table=g["tw_faces"], elem_ids=np.arange(len(g["tw_conn"]), dtype=np.int32))
    rti = CudaRayTracer()
    rti.set_tet_mesh(tm)
    se, sl, sc, st = rti.walk_elements(g["tw_start"], g["tw_s"], g["tw_u"], g["tw_len"], 128, prec)
    assert np.array_equal(sc, g["tw_count"])
    assert (st == 0).all()
    for k in range(len(sc)):
        c = sc[k]
        assert np.array_equal(se[k, :c], g["tw_elem"][k, :c])
        assert np.array_equal(sl[k, :c], g["tw_seglen"][k, :c])


@pytest.mark.parametrize("prec", PRECISIONS)
def test_packed_walk_matches_strided(cuda, tet_model, prec):
    """xdgcu_walk_elements_packed: same segments as the strided walk, packed by
    the scanned offsets; tracks that do not fit are flagged, not written."""
    torch = cuda
    from xdg_gb300._lib import RAY_OUTPUT_FULL
    tm = tet_model
    rti = CudaRayTracer()
    rti.set_tet_mesh(tm)
    m = synth.Model(volumes=[1], tets=tm, elements={1: np.arange(len(tm.conn), dtype=np.int32)})
    et = rti.create_element_tree(m, 1)
    rng = np.random.default_rng(31)
    n = 5000
    start = rng.uniform(0, 10, (n, 3))
    u = synth.isotropic_dirs(rng, n)
    length = np.minimum(rng.exponential(5.0, n), _exit_distance(start, u, 0.0, 10.0))
    _, idx = rti.find_element(et, start, prec)
    se, sl, sc, st = rti.walk_elements(idx, start, u, length, 512, prec)
    total = int(sc.sum())
    # host pointers
    pe, pl, off, pst = rti.walk_elements_packed(idx, start, u, length, total, 512, prec)
    assert off[0] == 0 and off[-1] == total and np.array_equal(np.diff(off), sc)
    assert np.array_equal(pst, st)
    for k in range(n):
        assert np.array_equal(pe[off[k]:off[k + 1]], se[k, :sc[k]])
        assert np.array_equal(pl[off[k]:off[k + 1]], sl[k, :sc[k]])
    # device pointers, same result
    dev = torch.device("cuda")
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)  # noqa: E731
    de, dl, doff, dst = rti.walk_elements_packed(T(idx), T(start), T(u), T(length), total, 512, prec)
    torch.cuda.synchronize()
    assert np.array_equal(doff.cpu().numpy(), off)
    assert np.array_equal(de.cpu().numpy()[:total], pe[:total])
    assert np.array_equal(dl.cpu().numpy()[:total], pl[:total])
    # too small: offsets still complete, overflowing tracks flagged and unwritten
    cap = total // 2
    pe2, pl2, off2, pst2 = rti.walk_elements_packed(idx, start, u, length, cap, 512, prec)
    assert np.array_equal(off2, off)
    full = off[1:] > cap
    assert (pst2[full & (sc > 0)] == RAY_OUTPUT_FULL).all()
    fit = ~full
    for k in np.nonzero(fit)[0][:200]:
        assert np.array_equal(pe2[off[k]:off[k + 1]], se[k, :sc[k]])
    # empty batch
    e0, l0, off0, s0 = rti.walk_elements_packed(idx[:0], start[:0], u[:0], length[:0], 0, 512, prec)
    assert len(off0) == 1 and off0[0] == 0


@pytest.mark.parametrize("prec", PRECISIONS)
def test_packed_walk_rounds(cuda, tet_model, prec):
    """The packed walk walked once in resumed rounds (packed_walk_passes 1,
    rounds capped at 1, 3 and 8 segments per track or automatically) and
    walked twice (2: count, then emit) gives the strided walk's segments,
    offsets and statuses, with tracks stopped at max_segs among them."""
    from xdg_gb300._lib import RAY_WALK_LIMIT
    tm = tet_model
    rti = CudaRayTracer()
    rti.set_tet_mesh(tm)
    m = synth.Model(volumes=[1], tets=tm, elements={1: np.arange(len(tm.conn), dtype=np.int32)})
    et = rti.create_element_tree(m, 1)
    rng = np.random.default_rng(41)
    n = 3000
    start = rng.uniform(0, 10, (n, 3))
    u = synth.isotropic_dirs(rng, n)
    length = np.minimum(rng.exponential(8.0, n), _exit_distance(start, u, 0.0, 10.0))
    _, idx = rti.find_element(et, start, prec)
    try:
        for max_segs in (512, 12):
            se, sl, sc, st = rti.walk_elements(idx, start, u, length, max_segs, prec)
            keep = np.arange(max_segs)[None, :] < sc[:, None]
            total = int(sc.sum())
            if max_segs == 12:
                assert (st == RAY_WALK_LIMIT).sum() > 100
            for passes, cap in ((1, 0), (1, 1), (1, 3), (1, 8), (2, 0)):
                rti.set_tuning("packed_walk_passes", passes)
                rti.set_tuning("segments_walk_cap", cap)
                pe, pl, off, pst = rti.walk_elements_packed(idx, start, u, length, total, max_segs,
                                                            prec)
                what = f"max_segs={max_segs} passes={passes} cap={cap}"
                assert off[0] == 0 and np.array_equal(np.diff(off), sc), what
                assert np.array_equal(pst, st), what
                assert np.array_equal(pe[:total], se[keep]), what
                assert np.array_equal(pl[:total], sl[keep]), what
        with pytest.raises(Exception):
            rti.set_tuning("packed_walk_passes", 3)
    finally:
        rti.set_tuning("packed_walk_passes", 1)
        rti.set_tuning("segments_walk_cap", 0)


@pytest.mark.parametrize("shift", [0.0, 3.0e4])
def test_closest_ties_and_offset_mesh(cuda, oracle, shift):
    """closest in mixed precision (an FP32 bound that skips the FP64 test of
    triangles proven farther than the best so far) gives the FP64 answer bit
    for bit and the oracle's: lattice points with exact ties between the two
    triangles of a box face and between faces, points within 1e-9 of a
    jittered sphere, points at and near the sphere's centre (nearly
    equidistant from all its triangles), and the same model moved far from
    the origin.  Also with the step budget after which a warp finishes a
    point's search at 1 and 16 steps (nearly every point searched by a warp)
    and off, and with the points in Morton order and in the caller's."""
    c = np.array([shift, -0.5 * shift, 0.25 * shift])
    m = synth.Model()
    v, f = synth.icosphere(4, 3.0, center=tuple(c), jitter=1e-3, seed=21)
    m.surfaces.append(synth.Surface(1, v, f, np.arange(len(f), dtype=np.int32), 1, 2))
    bv, bf = synth.box_surface(c - 8.0, c + 8.0)
    m.surfaces.append(synth.Surface(2, bv, bf, np.arange(len(f), len(f) + len(bf), dtype=np.int32), 2, 3))
    m.volumes = [1, 2, 3]
    m.implicit_complement = 3
    x = XDG(m)
    x.prepare_raytracer()
    g = np.arange(-10.0, 10.5, 0.5)
    lat = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    rng = np.random.default_rng(4)
    dirs = synth.isotropic_dirs(rng, 3000)
    r = np.linalg.norm(v - c, axis=1).mean()
    near = c + dirs * (r + rng.choice([-1e-9, 0.0, 1e-9], 3000))[:, None]
    centre = c + rng.uniform(-0.05, 0.05, (200, 3))
    p = np.concatenate([lat + c, near, c + rng.uniform(-12, 12, (3000, 3)), centre, c[None, :]])
    budget = x.rti.get_tuning("closest_step_budget")
    assert budget > 0
    for vol in (1, 2, 3):
        ocd, ocf = oracle.volume_tree(m, vol).closest(p)
        res = {prec: x.closest(vol, p, prec) for prec in PRECISIONS}
        x.rti.set_tuning("closest_bound", 0)
        try:
            res["mixed, no bound"] = x.closest(vol, p, MIXED)
        finally:
            x.rti.set_tuning("closest_bound", 1)
        try:
            for b in (1, 16, 0):
                x.rti.set_tuning("closest_step_budget", b)
                for prec in PRECISIONS:
                    res[f"{prec}, budget {b}"] = x.closest(vol, p, prec)
        finally:
            x.rti.set_tuning("closest_step_budget", budget)
        # the points in Morton order (every batch) and in the caller's order,
        # and in Morton order with nearly every point finished by a warp
        sort_min = x.rti.get_tuning("closest_sort_min")
        try:
            for smin in (1, 0):
                x.rti.set_tuning("closest_sort_min", smin)
                for prec in PRECISIONS:
                    res[f"{prec}, sort_min {smin}"] = x.closest(vol, p, prec)
            x.rti.set_tuning("closest_sort_min", 1)
            x.rti.set_tuning("closest_step_budget", 1)
            for prec in PRECISIONS:
                res[f"{prec}, sort_min 1, budget 1"] = x.closest(vol, p, prec)
        finally:
            x.rti.set_tuning("closest_sort_min", sort_min)
            x.rti.set_tuning("closest_step_budget", budget)
        for prec, (cd, cf) in res.items():
            assert_same(cf, ocf, f"closest face vol {vol} prec {prec}")
            assert_same(cd, ocd, f"closest distance vol {vol} prec {prec}")


def test_closest_triangle_soup_region_six(cuda, oracle):
    """closest over a soup of random, needle, obtuse and degenerate triangles,
    with points placed where the reference's closest-point routine leaves the
    triangle (its region six, beyond edges v0v1 and v1v2 near v1), near
    vertices and edges, and at random: the mixed path (FP32 lower and upper
    bounds that defer and skip exact tests) equals FP64 and the oracle bit
    for bit, so no bound ever prunes the reference's answer."""
    rng = np.random.default_rng(66)
    nt = 600
    c = rng.uniform(-5, 5, (nt, 3))
    size = 10.0 ** rng.uniform(-1, 0.5, nt)
    v = c[:, None, :] + rng.normal(size=(nt, 3, 3)) * size[:, None, None]
    kind = rng.integers(0, 10, nt)
    t = rng.uniform(0.2, 0.8, nt)
    nudge = 10.0 ** rng.uniform(-7, -2, nt)
    needle = kind < 2     # third vertex just off the first edge's line
    v[needle, 2] = (v[needle, 0] + t[needle, None] * (v[needle, 1] - v[needle, 0])
                    + (nudge * size)[needle, None] * rng.normal(size=(needle.sum(), 3)))
    obtuse = kind == 2    # v1 near the middle of v0v2, pushed out a little
    v[obtuse, 1] = (0.5 * (v[obtuse, 0] + v[obtuse, 2])
                    + 0.05 * size[obtuse, None] * rng.normal(size=(obtuse.sum(), 3)))
    degen = kind == 3     # a repeated vertex
    v[degen, 2] = v[degen, 1]
    m = synth.Model()
    verts = v.reshape(-1, 3)
    faces = np.arange(3 * nt, dtype=np.int32).reshape(nt, 3)
    m.surfaces.append(synth.Surface(1, verts, faces, np.arange(nt, dtype=np.int32), 1, 2))
    m.volumes = [1, 2]
    m.implicit_complement = 2
    x = XDG(m)
    x.prepare_raytracer()
    nrm = np.cross(v[:, 1] - v[:, 0], v[:, 2] - v[:, 0])
    with np.errstate(all="ignore"):
        nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    nrm = np.where(np.isfinite(nrm), nrm, 0.0)
    a = rng.uniform(-2.0, 0.0, nt)
    b = 1.0 + 10.0 ** rng.uniform(-6, 0.3, nt)
    six = (v[:, 0] + (b - a)[:, None] * (v[:, 1] - v[:, 0]) + a[:, None] * (v[:, 2] - v[:, 0])
           + nrm * (size * rng.uniform(-1, 1, nt))[:, None])
    k = rng.integers(0, 3, nt)
    ends = v[np.arange(nt), k], v[np.arange(nt), (k + 1) % 3]
    edge = ends[0] + rng.random(nt)[:, None] * (ends[1] - ends[0])
    off = (size * 10.0 ** rng.uniform(-9, -1, nt))[:, None] * rng.normal(size=(nt, 3))
    p = np.concatenate([six, v[:, 1] + off, edge + off, rng.uniform(-8, 8, (1500, 3))])
    ocd, ocf = oracle.volume_tree(m, 1).closest(p)
    assert (ocf >= 0).all()
    sort_min = x.rti.get_tuning("closest_sort_min")
    try:
        for smin in (1, 0):  # Morton order, and the caller's
            x.rti.set_tuning("closest_sort_min", smin)
            for prec in PRECISIONS:
                cd, cf = x.closest(1, p, prec)
                assert_same(cf, ocf, f"closest face prec {prec} sort_min {smin}")
                assert_same(cd, ocd, f"closest distance prec {prec} sort_min {smin}")
    finally:
        x.rti.set_tuning("closest_sort_min", sort_min)


def test_closest_far_points(cuda, oracle, sphere_box):
    """Points 1e15..1e25 away: beyond about 1e19 a box distance squared
    overflows FP32, and the mixed path then tests every triangle in FP64
    instead of pruning; results equal FP64's and the oracle's."""
    m, x = sphere_box
    rng = np.random.default_rng(12)
    n = 600
    p = synth.isotropic_dirs(rng, n) * (10.0 ** rng.uniform(15, 25, n))[:, None]
    for vol in (2, 3):
        ocd, ocf = oracle.volume_tree(m, vol).closest(p)
        assert (ocf >= 0).all()
        for prec in PRECISIONS:
            cd, cf = x.closest(vol, p, prec)
            assert_same(cf, ocf, f"closest face vol {vol} prec {prec}")
            assert_same(cd, ocd, f"closest distance vol {vol} prec {prec}")
