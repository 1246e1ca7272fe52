"""The oracle's particle loops (CPU): random sampling and the walk_elements
tool loop (tools/walk_elements.h:60-96).

The engine and the oracle give every particle its own SplitMix64 stream and
evaluate the collision-distance logarithm with the same series, so particle
histories can be compared bit for bit.  These tests pin the sampling
functions against the mathematics (log accuracy, uniformity, isotropy) and
the loops against properties that hold for any random stream: without
collisions a particle walks a straight chord through the mesh, exactly the
walk_elements track; track length is conserved in the per-tet tally; a
particle leaving a convex mesh never re-enters.
"""
import math

import numpy as np
import pytest

from xdg_gb300 import synth


def test_series_log_accuracy(oracle):
    rng = np.random.default_rng(1)
    xs = list(np.exp(rng.uniform(math.log(2.0 ** -53), 0.0, 5000)))
    xs += [1.0, 1.0 - 2.0 ** -53, 0.5, 0.25, 2.0 ** -53, math.sqrt(0.5), math.sqrt(2.0) / 2.0,
           0.7071067811865476, 0.7071067811865475, 3.0, 1e10, 123.456]
    worst = 0.0
    for x in xs:
        ref = math.log(x)
        got = oracle.series_log(x)
        if ref == 0.0:
            assert got == 0.0
            continue
        worst = max(worst, abs(got - ref) / abs(ref))
    assert worst < 4.5e-16, worst


def test_uniform_and_direction_sampling(oracle):
    states = np.array([12345, 2 ** 63 + 7, 99], dtype=np.uint64)
    u = oracle.sample_streams(states, 4000)
    assert u.min() >= 0.0 and u.max() < 1.0
    assert abs(u.mean() - 0.5) < 0.01
    # distinct streams differ
    assert not np.array_equal(u[0], u[1])
    import ctypes
    L = oracle.lib()
    s = np.array([42], dtype=np.uint64)
    d = np.zeros(3)
    dirs = np.zeros((4000, 3))
    for k in range(4000):
        L.xo_sample_direction(s.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
                              d.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        dirs[k] = d
    norms = np.sqrt((dirs ** 2).sum(1))
    assert np.abs(norms - 1.0).max() < 4e-16
    assert np.abs(dirs.mean(0)).max() < 0.05          # isotropic: zero mean
    assert np.abs((dirs ** 2).mean(0) - 1 / 3).max() < 0.03


@pytest.fixture(scope="module")
def cube_model():
    tm = synth.tet_cube(n=8, size=10.0, jitter=0.2, seed=11)
    return synth.model_from_tets(tm, np.ones(len(tm.conn), dtype=np.int32))


def _sources(oracle, model, n, seed):
    tm = model.tets
    rng = np.random.default_rng(seed)
    lo, hi = tm.vertices.min(0), tm.vertices.max(0)
    p = rng.uniform(lo + 0.3, hi - 0.3, (n, 3))
    tree = oracle.TetTree(tm.tet_xyz(), tm.elem_ids)
    _, idx = tree.find_element(p)
    keep = idx >= 0
    return idx[keep], p[keep], synth.isotropic_dirs(rng, int(keep.sum()))


def test_no_collision_transport_is_the_straight_walk(oracle, cube_model):
    tm = cube_model.tets
    elem, p, u = _sources(oracle, cube_model, 300, 5)
    w = oracle.TetWalker(tm.vertices, tm.conn, tm.adj, tm.face_table)
    rng = np.arange(1, len(elem) + 1, dtype=np.uint64) * np.uint64(7919)
    e, r, d, s, dist, ev, st, tally = w.transport(elem, p, u, rng, 1e300, 10_000)
    el, ln, cnt, wst = w.walk(elem, p, u, 1e300, max_segs=2048)
    assert (st == 0).all() and (wst == 0).all() and (e == -1).all()
    assert np.array_equal(ev, cnt)
    for i in range(len(elem)):
        acc = 0.0
        rr = p[i].copy()
        for k in range(cnt[i]):
            acc += ln[i, k]
            rr = rr + ln[i, k] * u[i]
        assert dist[i] == acc
        assert np.array_equal(r[i], rr)
    assert np.array_equal(d, u)  # no collision: direction unchanged
    assert abs(tally.sum() - dist.sum()) <= 1e-12 * dist.sum()


def test_transport_with_collisions(oracle, cube_model):
    tm = cube_model.tets
    elem, p, u = _sources(oracle, cube_model, 300, 6)
    w = oracle.TetWalker(tm.vertices, tm.conn, tm.adj, tm.face_table)
    rng = np.arange(1, len(elem) + 1, dtype=np.uint64) * np.uint64(104729)
    e, r, d, s, dist, ev, st, tally = w.transport(elem, p, u, rng, 1.0, 100_000)
    assert (st == 0).all() and (e == -1).all()
    assert ev.min() >= 1 and ev.mean() > 20          # many collisions in a 10-wide box
    assert abs(tally.sum() - dist.sum()) <= 1e-12 * dist.sum()
    # every particle ends on the cube's boundary
    lo, hi = tm.vertices.min(0), tm.vertices.max(0)
    edge = np.minimum(np.abs(r - lo), np.abs(r - hi)).min(1)
    assert edge.max() < 0.25                      # the jittered boundary stays within the cells
    # a bounded run stops with EVENT_LIMIT and resumes to the same end state
    e1, r1, d1, s1, dist1, ev1, st1, _ = w.transport(elem, p, u, rng, 1.0, 10)
    assert (st1[(ev1 == 10) & (e1 >= 0)] == 7).all() and (st1[e1 < 0] == 0).all()
    e2, r2, d2, s2, dist2, ev2, st2, _ = w.transport(e1, r1, d1, s1, 1.0, 100_000, dist1, ev1)
    assert np.array_equal(ev2, ev) and np.array_equal(dist2, dist) and np.array_equal(r2, r)


def test_walk_particles_convex_equals_transport(oracle, cube_model):
    tm = cube_model.tets
    elem, p, u = _sources(oracle, cube_model, 200, 7)
    w = oracle.TetWalker(tm.vertices, tm.conn, tm.adj, tm.face_table)
    ipc = oracle.volume_tree(cube_model, cube_model.implicit_complement)
    et = oracle.TetTree(tm.tet_xyz(), tm.elem_ids)
    rng = np.arange(1, len(elem) + 1, dtype=np.uint64) * np.uint64(31337)
    a = w.transport(elem, p, u, rng, 2.0, 100_000)
    b = w.walk_particles(ipc, et, elem, p, u, rng, 2.0, 100_000)
    for k, name in enumerate(["elem", "pos", "dir", "rng", "distance", "events", "status"]):
        assert np.array_equal(a[k], b[k]), name


def test_walk_particles_reenters_across_gaps(oracle):
    m = synth.tet_blocks([((0.0, 0.0, 0.0), 4, 4.0), ((6.0, 0.0, 0.0), 4, 4.0),
                          ((0.0, 6.0, 0.0), 4, 4.0)], jitter=0.2, seed=3)
    tm = m.tets
    w = oracle.TetWalker(tm.vertices, tm.conn, tm.adj, tm.face_table)
    ipc = oracle.volume_tree(m, m.implicit_complement)
    et = oracle.TetTree(tm.tet_xyz(), tm.elem_ids)
    rng0 = np.random.default_rng(9)
    n = 400
    p = rng0.uniform(0.2, 3.8, (n, 3))
    _, elem = et.find_element(p)
    u = synth.isotropic_dirs(rng0, n)
    u[: n // 2] = np.array([1.0, 0.0, 0.0])           # half aimed at the second block
    rng = np.arange(1, n + 1, dtype=np.uint64) * np.uint64(65537)
    a = w.transport(elem, p, u, rng, 50.0, 100_000)
    b = w.walk_particles(ipc, et, elem, p, u, rng, 50.0, 100_000)
    assert (b[6] == 0).all()
    # particles that crossed a gap travel farther than their first exit
    crossed = b[4] > a[4]
    assert crossed.sum() > n // 10
    # a particle that crossed continued its own random stream
    assert not np.array_equal(a[3][crossed], b[3][crossed])


# --------------------------------------------------------------------------
# particle_sim surface-tracking loop (tools/particle_sim.h:128-141)
# --------------------------------------------------------------------------

def _sphere_sources(n, seed):
    rng = np.random.default_rng(seed)
    p = rng.uniform(-6.0, 6.0, (n, 3))          # inside the radius-10 sphere
    return p, synth.isotropic_dirs(rng, n)


@pytest.mark.parametrize("case", ["vacuum", "graveyard", "reflecting"])
def test_surface_loop_boundaries(oracle, case):
    m = synth.single_sphere_in_box(level=3, radius=10.0, half_width=20.0)
    trees = {1: 1, 2: 2, 3: 3}
    bc = {2: 1} if case == "vacuum" else ({2: 2} if case == "reflecting" else {})
    sim = oracle.SurfaceTransport(m, trees, bc)
    n = 200
    p, u = _sphere_sources(n, 4)
    rng = np.arange(1, n + 1, dtype=np.uint64) * np.uint64(2654435761)
    max_ev = 400 if case == "reflecting" else 1_000_000
    t, r, d, s, dist, ev, st, tally = sim.run(np.ones(n, dtype=np.int32), p, u, rng, 5.0, max_ev,
                                             graveyard_tree=3 if case == "graveyard" else 0)
    assert abs(tally.sum() - dist.sum()) <= 1e-12 * dist.sum()
    assert np.abs(np.sqrt((d ** 2).sum(1)) - 1.0).max() < 4e-16
    edge = np.abs(r).max(1)
    if case == "reflecting":
        assert (st == 7).all() and (ev == max_ev).all() and (t >= 1).all()
        assert edge.max() <= 20.0 + 1e-9            # never leaves the box
        assert tally[3] == 0.0
    else:
        assert (st == 0).all()
        assert np.abs(edge - 20.0).max() < 1e-9      # every particle ends on the box
        assert (t == (2 if case == "vacuum" else -1)).all()
        assert tally[1] > 0 and tally[2] > 0 and tally[3] == 0.0


def test_surface_loop_without_collisions_is_a_ray_fire_chain(oracle):
    """With a huge mean free path each event is one surface crossing: the
    particle's distance is the sum of the chain of ray_fire distances."""
    m = synth.nested_spheres(n=4, level=2, jitter=1e-3, seed=7)
    trees = {v: v for v in m.volumes}
    sim = oracle.SurfaceTransport(m, trees)
    n = 50
    rng0 = np.random.default_rng(2)
    p = rng0.uniform(-0.4, 0.4, (n, 3))
    u = synth.isotropic_dirs(rng0, n)
    rng = np.arange(1, n + 1, dtype=np.uint64)
    t, r, d, s, dist, ev, st, _ = sim.run(np.ones(n, dtype=np.int32), p, u, rng, 1e300, 1000,
                                         graveyard_tree=5)
    assert (st == 0).all() and (t == -1).all() and (ev == 4).all()
    for i in range(n):
        o, acc, excl = p[i].copy(), 0.0, []
        for k in range(1, 5):
            th, sid, fid = oracle.volume_tree(m, k).ray_fire(o[None], u[i][None], excl=[excl])
            o = o + th[0] * u[i]
            acc += th[0]
            excl = excl + [int(fid[0])]
        assert dist[i] == acc and np.array_equal(r[i], o)
