"""The reference's MeshMock tests, run on the CUDA engine in both precisions.

Each test mirrors a Catch2 test of the reference (file:line in the
docstring) and additionally checks every value against the CPU oracle bit
for bit.
"""
import numpy as np
import pytest

from xdg_gb300 import synth
from xdg_gb300.engine import ENTERING, EXITING, FP64, ID_NONE, INFTY, MIXED, XDG, CudaRayTracer

pytestmark = pytest.mark.gpu

PRECISIONS = [FP64, MIXED]


def mock_tracer(volumetric=False):
    m = synth.mock_cube(volumetric_elements=volumetric)
    rti = CudaRayTracer()
    vt, et = rti.register_volume(m, m.volumes[0])
    return m, rti, vt, et


@pytest.mark.parametrize("prec", PRECISIONS)
def test_ray_fire_mock(cuda, oracle, prec):
    """tests/test_ray_fire.cpp:19-111"""
    m, rti, vt, et = mock_tracer(False)
    assert vt != ID_NONE and et == ID_NONE
    ot = oracle.volume_tree(m, 0)

    def fire(o, d, dl=None, orient=EXITING, excl=None):
        t, s, f = rti.ray_fire(vt, [o], [d], dl, orient, excl, prec)
        t2, s2, f2 = ot.ray_fire([o], [d], dl, orient, excl)
        assert t[0] == t2[0] and s[0] == s2[0] and f[0] == f2[0]
        return t[0], s[0], f[0]

    for d, exp in [((1, 0, 0), 5.0), ((-1, 0, 0), 2.0), ((0, 1, 0), 6.0), ((0, -1, 0), 3.0),
                   ((0, 0, 1), 7.0), ((0, 0, -1), 4.0)]:
        assert abs(fire((0, 0, 0), d)[0] - exp) < 1e-6
    assert abs(fire((-10, 0, 0), (1, 0, 0))[0] - 15.0) < 1e-6
    assert abs(fire((10, 0, 0), (-1, 0, 0))[0] - 12.0) < 1e-6
    assert abs(fire((-10, 0, 0), (1, 0, 0), orient=ENTERING)[0] - 8.0) < 1e-6
    assert abs(fire((10, 0, 0), (-1, 0, 0), orient=ENTERING)[0] - 5.0) < 1e-6
    assert fire((0, 0, 0), (1, 0, 0), dl=4.5)[1] == ID_NONE
    t, s, f = fire((0, 0, 0), (1, 0, 0), dl=5.1)
    assert s != ID_NONE and abs(t - 5.0) < 1e-6
    excl = []
    t, s, f = fire((0, 0, 0), (1, 0, 0), excl=[excl])
    assert abs(t - 5.0) < 1e-6
    excl.append(int(f))  # the reference appends the hit face (embree/ray_tracer.cpp:324)
    assert len(excl) == 1
    t, s, f = fire((0, 0, 0), (1, 0, 0), excl=[excl])
    assert s == ID_NONE and t == INFTY


@pytest.mark.parametrize("prec", PRECISIONS)
def test_point_in_volume_mock(cuda, oracle, prec):
    """tests/test_point_in_volume.cpp:17-79"""
    m, rti, vt, _ = mock_tracer(False)
    ot = oracle.volume_tree(m, 0)
    pts = [(0, 0, 0), (0, 0, 1000), (4.0 - 1e-6, 0, 0), (5.001, 0, 0)]
    r = rti.point_in_volume(vt, pts, precision=prec)
    assert list(r) == [1, 0, 1, 0]
    assert list(r) == list(ot.point_in_volume(pts))
    pts = [(5.0, 0, 0), (5.1, 0, 0), (5.1, 0, 0)]
    dirs = [(1, 0, 0), (1, 0, 0), (-1, 0, 0)]
    r = rti.point_in_volume(vt, pts, dirs, precision=prec)
    assert list(r) == [1, 0, 0]
    assert list(r) == list(ot.point_in_volume(pts, dirs))


@pytest.mark.parametrize("prec", PRECISIONS)
def test_occluded_mock(cuda, oracle, prec):
    """tests/test_occluded.cpp:12-31"""
    m = synth.mock_cube(True)
    xdg = XDG(m)
    xdg.prepare_raytracer()
    occ, dist = xdg.occluded(0, [(-100, 0, 0), (-100, 0, 0)], [(1, 0, 0), (-1, 0, 0)], prec)
    assert list(occ) == [1, 0]
    assert dist[0] == -INFTY and dist[1] == INFTY


@pytest.mark.parametrize("prec", PRECISIONS)
def test_find_element_mock(cuda, oracle, prec):
    """tests/test_find_element.cpp:12-41"""
    m = synth.mock_cube(True)
    rti = CudaRayTracer()
    vt, et = rti.register_volume(m, 0)
    assert rti.num_registered_trees() == 2
    eid, eidx = rti.find_element(et, [(0, 0, 0), (10, 10, 10)], prec)
    assert eid[0] != ID_NONE and eid[1] == ID_NONE
    tt = oracle.TetTree(m.tets.tet_xyz(), m.tets.elem_ids)
    rng = np.random.default_rng(3)
    pts = rng.uniform([-3, -4, -5], [6, 7, 8], (2000, 3))
    eid, _ = rti.find_element(et, pts, prec)
    oid, _ = tt.find_element(pts)
    assert np.array_equal(eid, oid)


def test_bvh_tree_counts(cuda):
    """tests/test_bvh.cpp:12-47 and the tree counts of test_tracks.cpp:35, 62"""
    m = synth.mock_cube(True)
    rti = CudaRayTracer()
    rti.register_volume(m, 0)
    assert rti.num_registered_trees() == 2
    assert rti.num_registered_surface_trees() == 1
    assert rti.num_registered_element_trees() == 1
    x = XDG(synth.mock_cube(True))
    x.prepare_raytracer()
    assert x.rti.num_registered_trees() == 4
    x = XDG(synth.mock_cube(True, implicit_complement=True))
    x.prepare_raytracer()
    assert x.rti.num_registered_trees() == 6


@pytest.mark.parametrize("prec", PRECISIONS)
def test_closest_mock(cuda, oracle, prec):
    """tests/test_closest.cpp:18-59"""
    m = synth.mock_cube(True)
    xdg = XDG(m)
    xdg.prepare_raytracer()
    d, f = xdg.closest(0, [(0, 0, 0), (4, 0, 0), (10, 0, 0)], prec)
    assert np.allclose(d, [2.0, 1.0, 5.0], atol=1e-6)
    rng = np.random.default_rng(11)
    c = 0.5 * (synth.MOCK_BOX_LO + synth.MOCK_BOX_HI)
    p = np.tile(c, (1000, 1))
    p[:, 0] = rng.uniform(-10, 10, 1000)
    d, f = xdg.closest(0, p, prec)
    exp = np.where(p[:, 0] < c[0], np.abs(p[:, 0] - synth.MOCK_BOX_LO[0]),
                   np.abs(p[:, 0] - synth.MOCK_BOX_HI[0]))
    assert np.allclose(d, exp, atol=1e-6)
    od, of = oracle.volume_tree(m, 0).closest(p)
    assert np.array_equal(d, od) and np.array_equal(f, of)


def test_normal_mock(cuda, oracle):
    """tests/test_normal.cpp:15-43: surface_normal = face_normal(closest face)"""
    m = synth.mock_cube(True)
    xdg = XDG(m)
    xdg.prepare_raytracer()
    d, f = xdg.closest(0, [(4.0, 0, 0)])
    assert abs(d[0] - 1.0) < 1e-6
    face = int(f[0])
    v = m.tets.vertices[np.concatenate([s.triangles for s in m.surfaces])[face]].reshape(9)
    n = oracle.face_normal(v)
    assert np.allclose(n, [1.0, 0.0, 0.0])


@pytest.mark.parametrize("prec", PRECISIONS)
def test_walk_to_corner(cuda, oracle, prec):
    """tests/test_tally_segments.cpp:15-72: next_element chain to the corner"""
    m = synth.mock_cube(True)
    xdg = XDG(m)
    xdg.prepare_raytracer()
    assert xdg.rti.num_registered_trees() == 4
    r = np.array([-1.0, -2.0, -3.0])
    ur = synth.MOCK_BOX_HI
    u = oracle.normalize(ur - r)
    w = ur - r
    distance = np.sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2])
    eid, eidx = xdg.find_element([r], precision=prec)
    assert eid[0] != ID_NONE
    walker = oracle.TetWalker(m.tets.vertices, m.tets.conn, m.tets.adj, m.tets.face_table)
    elem = int(eidx[0])
    it = 0
    nxt = ID_NONE
    while elem != ID_NONE and it < 100:
        nx, ex, st = xdg.next_element([elem], [r], [u], prec)
        onx, oex, _ = walker.next_element(elem, r, u)
        assert int(nx[0]) == onx and ex[0] == oex
        nxt, exd = int(nx[0]), float(ex[0])
        assert exd < distance
        r = r + u * exd
        elem = nxt
        distance -= exd
        it += 1
    assert it < 100 and nxt == ID_NONE
    assert np.allclose(r, ur, rtol=1e-4)


@pytest.mark.parametrize("prec", PRECISIONS)
def test_tracks_mock(cuda, oracle, prec):
    """tests/test_tracks.cpp:25-123"""
    m = synth.mock_cube(True)
    xdg = XDG(m)
    xdg.prepare_raytracer()
    segs = xdg.segments(0, [(0, 0, 0)], [(1, 1, 1)], precision=prec)
    assert abs(segs[0][1].sum() - np.sqrt(3.0)) <= 1e-5 * np.sqrt(3.0)
    # random internal tracks: the chord length is recovered
    rng = np.random.default_rng(42)
    n = 1000
    s = rng.uniform(synth.MOCK_BOX_LO, synth.MOCK_BOX_HI, (n, 3))
    e = rng.uniform(synth.MOCK_BOX_LO, synth.MOCK_BOX_HI, (n, 3))
    segs = xdg.segments(0, s, e, precision=prec)
    chord = np.linalg.norm(s - e, axis=1)
    for k in range(n):
        assert len(segs[k][0]) > 0
        assert abs(segs[k][1].sum() - chord[k]) <= 1e-5 * chord[k]
    # intersecting track from outside (needs the implicit complement)
    m2 = synth.mock_cube(True, implicit_complement=True)
    x2 = XDG(m2)
    x2.prepare_raytracer()
    assert x2.rti.num_registered_trees() == 6
    c = 0.5 * (synth.MOCK_BOX_LO + synth.MOCK_BOX_HI)
    start = c.copy()
    start[0] -= 10
    segs = x2.segments(0, [start], [c], precision=prec)
    exp = c[0] - synth.MOCK_BOX_LO[0]
    assert abs(segs[0][1].sum() - exp) <= 1e-5 * exp


@pytest.mark.parametrize("prec", PRECISIONS)
def test_degenerate_lattice_rays(cuda, oracle, prec):
    """Origins on an integer lattice covering faces, edges and corners of the
    mock box, the 26 lattice directions with +0/-0 components, unnormalised
    and normalised: every query agrees with the oracle bit for bit."""
    m = synth.mock_cube(False)
    rti = CudaRayTracer()
    vt, _ = rti.register_volume(m, 0)
    ot = oracle.volume_tree(m, 0)
    g = np.arange(-3.0, 7.0)
    O = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    dirs = np.array([(i, j, k) for i in (-1.0, 0.0, 1.0) for j in (-1.0, 0.0, 1.0)
                     for k in (-1.0, 0.0, 1.0) if (i, j, k) != (0.0, 0.0, 0.0)])
    negz = np.where(dirs == 0.0, -0.0, dirs)  # the same directions with -0.0 components
    D = np.concatenate([dirs, negz, synth.normalize_rows(dirs), 2.5 * dirs])
    oo = np.repeat(O, len(D), axis=0)
    dd = np.tile(D, (len(O), 1))
    oo = np.where(oo == 0.0, np.where(np.arange(len(oo))[:, None] % 2 == 0, -0.0, 0.0), oo)
    for orient in (EXITING, ENTERING, -1):
        t, s, f = rti.ray_fire(vt, oo, dd, None, orient, precision=prec)
        t2, s2, f2 = ot.ray_fire(oo, dd, None, orient)
        assert np.array_equal(s, s2) and np.array_equal(f, f2) and np.array_equal(t, t2), orient
    assert np.array_equal(rti.point_in_volume(vt, oo, dd, precision=prec), ot.point_in_volume(oo, dd))
    occ, dist = rti.occluded(vt, oo, dd, prec)
    oocc, odist = ot.occluded(oo, dd)
    assert np.array_equal(occ, oocc) and np.array_equal(dist, odist)
