"""CPU: the oracle against the reference.

* tests/golden/reference_vectors.npz was produced by the reference's own
  compiled code (tests/golden/make_golden.py); the oracle must reproduce it
  bit for bit.
* Where the reference tree is present, the oracle is also compared live with
  the reference's code on fresh random inputs.
* The known-answer tests of the reference's Catch2 suite that need no mesh
  library (MeshMock and the unit tests) are replayed against the oracle.
"""
import os

import numpy as np
import pytest

from conftest import ROOT
from xdg_gb300 import synth

GOLD = os.path.join(ROOT, "tests", "golden", "reference_vectors.npz")


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


def test_plucker_matches_reference_vectors(oracle, gold):
    n = len(gold["pl_hit"])
    for i in range(n):
        h, t = oracle.plucker(gold["pl_v"][i], gold["pl_o"][i], gold["pl_d"][i], gold["pl_tmax"][i],
                              0.0, bool(gold["pl_use_or"][i]), int(gold["pl_orient"][i]))
        assert h == bool(gold["pl_hit"][i]), i
        if h:
            assert t == gold["pl_t"][i], (i, t, gold["pl_t"][i])


def test_closest_matches_reference_vectors(oracle, gold):
    for i in range(len(gold["cl_region"])):
        assert oracle.closest_region(gold["cl_v"][i], gold["cl_p"][i]) == gold["cl_region"][i]
        assert np.array_equal(oracle.closest_on_tri(gold["cl_v"][i], gold["cl_p"][i]), gold["cl_out"][i])


def test_normalize_matches_reference_vectors(oracle, gold):
    for v, w in zip(gold["nv_in"], gold["nv_out"]):
        assert np.array_equal(oracle.normalize(v), w)


def test_walk_matches_reference_vectors(oracle, gold):
    w = oracle.TetWalker(gold["tw_xyz"], gold["tw_conn"], gold["tw_adj"], gold["tw_faces"])
    el, ln, cnt, st = w.walk(gold["tw_start"], gold["tw_s"], gold["tw_u"], gold["tw_len"], 128)
    assert np.array_equal(cnt, gold["tw_count"])
    assert (st == 0).all()
    for i in range(len(cnt)):
        c = cnt[i]
        assert np.array_equal(el[i, :c], gold["tw_elem"][i, :c])
        assert np.array_equal(ln[i, :c], gold["tw_seglen"][i, :c])


def test_mock_walk_to_corner(oracle, gold):
    """tests/test_tally_segments.cpp:15-72 on the oracle, against the chain the
    reference's own next_element produced."""
    m = synth.mock_cube(True)
    w = oracle.TetWalker(m.tets.vertices, m.tets.conn, m.tets.adj, m.tets.face_table)
    tt = oracle.TetTree(m.tets.tet_xyz(), m.tets.elem_ids)
    r = np.array([-1.0, -2.0, -3.0])
    ur = synth.MOCK_BOX_HI
    u = oracle.normalize(ur - r)
    assert np.array_equal(u, gold["mock_chain_u"])
    w_ = ur - r
    distance = np.sqrt(w_[0] * w_[0] + w_[1] * w_[1] + w_[2] * w_[2])
    elem = int(tt.find_element([r])[1][0])
    assert elem != -1
    chain_e, chain_d = [], []
    while elem != -1 and len(chain_e) < 100:
        nx, ex, _ = w.next_element(elem, r, u)
        assert ex < distance
        chain_e.append(nx)
        chain_d.append(ex)
        r = r + u * ex
        distance -= ex
        elem = nx
    assert chain_e == list(gold["mock_chain_next"])
    assert chain_d == list(gold["mock_chain_dist"])
    assert np.allclose(r, ur, rtol=1e-4)


def test_mock_ray_queries(oracle):
    """test_ray_fire.cpp:19-111, test_point_in_volume.cpp:17-79,
    test_occluded.cpp:12-31, test_closest.cpp:18-59 on the oracle."""
    m = synth.mock_cube(True)
    t = oracle.volume_tree(m, 0)
    o = np.zeros((6, 3))
    d = np.array([[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1.0]])
    tt, s, f = t.ray_fire(o, d)
    assert np.allclose(tt, [5, 2, 6, 3, 7, 4], atol=1e-6)
    tt, s, f = t.ray_fire([[-10, 0, 0], [10, 0, 0]], [[1, 0, 0], [-1, 0, 0]])
    assert np.allclose(tt, [15, 12], atol=1e-6)
    tt, s, f = t.ray_fire([[-10, 0, 0], [10, 0, 0]], [[1, 0, 0], [-1, 0, 0]],
                          orientation=oracle.ENTERING)
    assert np.allclose(tt, [8, 5], atol=1e-6)
    tt, s, f = t.ray_fire([[0, 0, 0]] * 2, [[1, 0, 0]] * 2, dist_limit=np.array([4.5, 5.1]))
    assert s[0] == -1 and s[1] != -1 and abs(tt[1] - 5.0) < 1e-6
    tt, s, f = t.ray_fire([[0, 0, 0]], [[1, 0, 0]])
    tt2, s2, f2 = t.ray_fire([[0, 0, 0]], [[1, 0, 0]], excl=[[int(f[0])]])
    assert s2[0] == -1
    assert list(t.point_in_volume([[0, 0, 0], [0, 0, 1000], [4 - 1e-6, 0, 0], [5.001, 0, 0]])) == [1, 0, 1, 0]
    assert list(t.point_in_volume([[5, 0, 0], [5.1, 0, 0], [5.1, 0, 0]],
                                  [[1, 0, 0], [1, 0, 0], [-1, 0, 0]])) == [1, 0, 0]
    occ, dist = t.occluded([[-100, 0, 0]] * 2, [[1, 0, 0], [-1, 0, 0]])
    assert list(occ) == [1, 0]
    cd, cf = t.closest([[0, 0, 0], [4, 0, 0], [10, 0, 0]])
    assert np.allclose(cd, [2, 1, 5], atol=1e-6)


def test_tet_containment_kats(oracle):
    """tests/test_tet_containment.cpp:14-94 and test_tet_intersection.cpp:14-34."""
    A = np.array([0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0, 1.0])
    B = np.array([1, 1, 1, 2, 1, 1, 1, 2, 1, 1, 1, 2.0])
    inside = [(0.1, 0.1, 0.1), (0, 0, 0.5), (0.3, 0.3, 0.1), (0.3, 0.1, 0.3), (0.1, 0.3, 0.3),
              (0.3, 0.3, 0.3)]
    outside = [(2, 2, 2), (-0.5, -0.5, 0), (0.3, 0.3, -0.1), (0.3, -0.1, 0.3), (-0.1, 0.3, 0.3),
               (0.4, 0.4, 0.4)]
    for p in inside:
        assert oracle.tet_contains(p, A), p
    for p in outside:
        assert not oracle.tet_contains(p, A), p
    for p in [(1.2, 1.2, 1.2), (1, 1, 1.5), (1.3, 1.3, 1.1)]:
        assert oracle.tet_contains(p, B), p
    for p in [(0, 0, 0), (1.3, 1.3, 0.9), (0.1, 0.1, 0.1)]:
        assert not oracle.tet_contains(p, B), p
    assert not oracle.tet_contains((1.2, 1.2, 1.2), A)


def test_tet_containment_is_barycentric(oracle):
    """The adjugate/determinant solve agrees with a linear solve away from faces."""
    rng = np.random.default_rng(3)
    for _ in range(300):
        v = rng.normal(0, 1, (4, 3))
        if abs(np.linalg.det(v[1:] - v[0])) < 1e-2:
            continue
        p = rng.normal(0, 1, 3)
        lam = np.linalg.solve((v[1:] - v[0]).T, p - v[0])
        bary = np.concatenate([[1 - lam.sum()], lam])
        if np.min(np.abs(bary)) < 1e-9 or np.min(np.abs(bary - 1)) < 1e-9:
            continue
        exp = bool((bary >= 0).all() and (bary <= 1).all())
        assert oracle.tet_contains(p, v.reshape(12)) == exp


def test_closest_region_kats(oracle):
    """tests/test_closest.cpp:61-184"""
    tri = np.array([-1.0, -1.0, 0.0, 2.0, 1.0, 0.0, -2.0, 3.0, 0.0])
    cases = [((0, 0, 0), 0), ((3, 3, 0), 1), ((-2.5, 3.5, 0), 2), ((-2.5, -1.5, 0), 3),
             ((-2, -2, 0), 4), ((1, -0.5, 0), 5), ((10, 0, 0), 6)]
    for p, r in cases:
        assert oracle.closest_region(tri, p) == r
    v = tri.reshape(3, 3)
    for k in range(3):
        assert np.array_equal(oracle.closest_on_tri(tri, v[k]), v[k])
        mid = (v[k] + v[(k + 1) % 3]) / 2.0
        assert np.allclose(oracle.closest_on_tri(tri, mid), mid, atol=1e-6)


@pytest.mark.parametrize("seed", [1, 2])
def test_plucker_live_against_reference(oracle, ref_lib, seed):
    rng = np.random.default_rng(seed)
    for _ in range(4000):
        v = rng.normal(0, 3, 9)
        if rng.uniform() < 0.5:  # aim at a vertex or edge
            k = rng.integers(0, 3)
            tgt = v.reshape(3, 3)[k] * (1 - rng.uniform() * 1e-12)
        else:
            tgt = rng.normal(0, 3, 3)
        o = rng.normal(0, 4, 3)
        d = tgt - o
        d /= np.linalg.norm(d)
        use_or = rng.uniform() < 0.3
        a = oracle.plucker(v, o, d, oracle.INFTY, 0.0, use_or, 1)
        b = oracle.plucker(v, o, d, oracle.INFTY, 0.0, use_or, 1, use_ref=True)
        assert a == b


def test_walk_live_against_reference(oracle, ref_lib):
    tm = synth.tet_cube(n=5, size=5.0, jitter=0.2, seed=9)
    rw = oracle.RefWalker(tm.vertices, tm.conn, tm.adj, tm.face_table)
    w = oracle.TetWalker(tm.vertices, tm.conn, tm.adj, tm.face_table)
    tt = oracle.TetTree(tm.tet_xyz(), tm.elem_ids)
    rng = np.random.default_rng(4)
    n = 400
    s = rng.uniform(0.01, 4.99, (n, 3))
    u = synth.isotropic_dirs(rng, n)
    ln = rng.uniform(0, 8, n)
    _, start = tt.find_element(s)
    el, sl, cnt, st = w.walk(start, s, u, ln, 256)
    for i in range(n):
        e, l2 = rw.walk(int(start[i]), s[i], u[i], float(ln[i]), 256)
        assert np.array_equal(el[i, :cnt[i]], e) and np.array_equal(sl[i, :cnt[i]], l2)
    # the (start, end) overload normalises u exactly like the oracle's normalize
    e0 = s[0] + np.array([1.5, -0.7, 0.3])
    e, l2 = rw.walk_to(int(start[0]), s[0], e0)
    uu = oracle.normalize(e0 - s[0])
    wv = e0 - s[0]
    dist = np.sqrt(wv[0] * wv[0] + wv[1] * wv[1] + wv[2] * wv[2])
    el, sl, cnt, st = w.walk(start[:1], s[:1], uu[None], dist, 256)
    assert np.array_equal(el[0, :cnt[0]], e) and np.array_equal(sl[0, :cnt[0]], l2)


def test_bvh_equals_brute_force(oracle):
    m = synth.single_sphere_in_box(level=3)
    a = oracle.volume_tree(m, 1, use_bvh=True)
    b = oracle.volume_tree(m, 1, use_bvh=False)
    o, d = synth.lcg_ball_rays(3000, 9.9, seed=3)
    for x, y in zip(a.ray_fire(o, d), b.ray_fire(o, d)):
        assert np.array_equal(x, y)
    rng = np.random.default_rng(1)
    p = rng.uniform(-25, 25, (2000, 3))
    assert np.array_equal(a.point_in_volume(p), b.point_in_volume(p))
    for x, y in zip(a.closest(p), b.closest(p)):
        assert np.array_equal(x, y)
    tm = synth.tet_cube(n=4, size=4.0)
    ta = oracle.TetTree(tm.tet_xyz(), tm.elem_ids, use_bvh=True)
    tb = oracle.TetTree(tm.tet_xyz(), tm.elem_ids, use_bvh=False)
    q = rng.uniform(-0.5, 4.5, (3000, 3))
    for x, y in zip(ta.find_element(q), tb.find_element(q)):
        assert np.array_equal(x, y)


def test_synthetic_tet_cube_is_valid():
    tm = synth.tet_cube(n=6, size=3.0, jitter=0.2, seed=2)
    v = tm.vertices[tm.conn]
    det = np.einsum("ij,ij->i", np.cross(v[:, 1] - v[:, 0], v[:, 2] - v[:, 0]), v[:, 3] - v[:, 0])
    assert (det > 0).all()
    # adjacency is symmetric and every interior face is shared by exactly two tets
    for t in range(len(tm.conn)):
        for f in range(4):
            nb = tm.adj[t, f]
            if nb >= 0:
                assert t in tm.adj[nb]
    assert np.isclose(np.abs(det).sum() / 6.0, 27.0)
