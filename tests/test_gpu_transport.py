"""Device particle loops against the oracle.

xdgcu_transport_elements runs the in-mesh part of the walk_elements tool
loop (tools/walk_elements.h:73-87) for every particle in one launch; the
engine's XDG.walk_particles adds the tool's re-entry through the implicit
complement (:88-94).  Both use per-particle random streams that the oracle
reproduces, so every particle's final tet, position, direction, stream
state, path length and event count must equal the oracle's bit for bit, in
both precisions.  The per-tet track-length tally is summed with atomics in
no fixed order: it must agree within 1e-12 relative per tet (and its total
with the total path length).
"""
import numpy as np
import pytest

from xdg_gb300 import synth
from xdg_gb300.engine import FP64, MIXED, XDG

pytestmark = pytest.mark.gpu

NAMES = ["elem", "pos", "dir", "rng", "distance", "events", "status"]


def assert_same(a, b, what):
    a = np.asarray(a)
    b = np.asarray(b)
    assert a.shape == b.shape, what
    bad = np.nonzero((a != b).reshape(len(a), -1).any(1))[0] if len(a) else []
    assert len(bad) == 0, f"{what}: {len(bad)} mismatches, first at {bad[:5]}"


@pytest.fixture(scope="module")
def cube(cuda):
    tm = synth.tet_cube(n=20, size=10.0, jitter=0.2, seed=11)
    m = synth.model_from_tets(tm, np.ones(len(tm.conn), dtype=np.int32))
    x = XDG(m)
    x.prepare_raytracer()
    rng = np.random.default_rng(21)
    n = 6000
    p = rng.uniform(0.05, 9.95, (n, 3))
    _, elem = x.find_element(p)
    u = synth.isotropic_dirs(rng, n)
    return m, x, elem.astype(np.int32), p, u


def _oracle_walker(oracle, m):
    tm = m.tets
    return oracle.TetWalker(tm.vertices, tm.conn, tm.adj, tm.face_table)


@pytest.mark.parametrize("prec", [FP64, MIXED])
@pytest.mark.parametrize("mfp", [0.5, 3.0])
def test_transport_elements_matches_oracle(cube, oracle, prec, mfp):
    import torch
    m, x, elem, p, u = cube
    seeds = x.rti.seed_streams(77, len(elem))
    w = _oracle_walker(oracle, m)
    o = w.transport(elem, p, u, seeds, mfp, 1_000_000)
    dev = torch.device("cuda", 0)
    e = torch.as_tensor(elem, device=dev)
    r = torch.as_tensor(p, device=dev).clone()
    d = torch.as_tensor(u, device=dev).clone()
    s = torch.as_tensor(seeds.view(np.int64), device=dev).clone()
    dist = torch.zeros(len(elem), dtype=torch.float64, device=dev)
    ev = torch.zeros(len(elem), dtype=torch.int32, device=dev)
    tally = torch.zeros(len(m.tets.conn), dtype=torch.float64, device=dev)
    st = x.rti.transport_elements(e, r, d, s, mfp, 1_000_000, dist, ev, tally, precision=prec)
    torch.cuda.synchronize()
    got = [e.cpu().numpy(), r.cpu().numpy(), d.cpu().numpy(), s.cpu().numpy().view(np.uint64),
           dist.cpu().numpy(), ev.cpu().numpy(), st.cpu().numpy()]
    for k, name in enumerate(NAMES):
        assert_same(got[k], o[k], name)
    assert (got[0] == -1).all() and (got[6] == 0).all()
    # events run at once or gathered across the warp: same histories
    for wait in (1, 32):
        x.rti.set_tuning("transport_event_wait", wait)
        try:
            e2, r2, d2, s2 = e.clone(), r.clone(), d.clone(), s.clone()
            e2.copy_(torch.as_tensor(elem, device=dev))
            r2.copy_(torch.as_tensor(p, device=dev))
            d2.copy_(torch.as_tensor(u, device=dev))
            s2.copy_(torch.as_tensor(seeds.view(np.int64), device=dev))
            dist2, ev2 = torch.zeros_like(dist), torch.zeros_like(ev)
            x.rti.transport_elements(e2, r2, d2, s2, mfp, 1_000_000, dist2, ev2, None,
                                     precision=prec)
            torch.cuda.synchronize()
            assert torch.equal(e2, e) and torch.equal(r2, r) and torch.equal(s2, s)
            assert torch.equal(dist2, dist) and torch.equal(ev2, ev)
        finally:
            x.rti.set_tuning("transport_event_wait", 4)
    ty = tally.cpu().numpy()
    assert np.allclose(ty, o[7], rtol=1e-12, atol=1e-300)
    assert abs(ty.sum() - got[4].sum()) <= 1e-12 * got[4].sum()


def test_transport_host_arrays_and_event_limit(cube, oracle):
    """Host arrays (staged through the C ABI) give the device results; a run
    cut at max_events and resumed ends in the same state."""
    m, x, elem, p, u = cube
    n = 2000
    seeds = x.rti.seed_streams(5, n)
    w = _oracle_walker(oracle, m)
    full = w.transport(elem[:n], p[:n], u[:n], seeds, 1.0, 1_000_000)
    e, r, d, s = elem[:n].copy(), p[:n].copy(), u[:n].copy(), seeds.copy()
    dist, ev = np.zeros(n), np.zeros(n, dtype=np.int32)
    st = x.rti.transport_elements(e, r, d, s, 1.0, 7, dist, ev, None, precision=MIXED)
    cut = (ev == 7) & (e >= 0)
    assert cut.sum() > n // 2 and (st[cut] == 7).all()
    st = x.rti.transport_elements(e, r, d, s, 1.0, 1_000_000, dist, ev, None, precision=MIXED)
    for k, (name, a) in enumerate(zip(NAMES, [e, r, d, s, dist, ev, st])):
        assert_same(a, full[k], name)


def test_transport_invalid_and_outside(cube):
    m, x, elem, p, u = cube
    e = np.array([elem[0], -1, len(m.tets.conn) + 5, elem[1]], dtype=np.int32)
    r = p[:4].copy()
    r[3, 0] = np.nan
    d = u[:4].copy()
    s = x.rti.seed_streams(1, 4)
    dist, ev = np.zeros(4), np.zeros(4, dtype=np.int32)
    st = x.rti.transport_elements(e, r, d, s, 1.0, 1000, dist, ev, None, precision=MIXED)
    assert list(st) == [0, 0, 1, 1]
    assert ev[1] == 0 and ev[2] == 0 and ev[3] == 0 and ev[0] > 0
    with pytest.raises(Exception, match="mean_free_path"):
        x.rti.transport_elements(e, r, d, s, 0.0, 1000, dist, ev, None)


@pytest.mark.parametrize("prec", [FP64, MIXED])
def test_walk_particles_reentry_matches_oracle(cuda, oracle, prec):
    """Three separate meshed blocks with implicit-complement gaps: particles
    leaving one block re-enter another through ray_fire + find_element."""
    m = synth.tet_blocks([((0.0, 0.0, 0.0), 5, 4.0), ((6.0, 0.0, 0.0), 5, 4.0),
                          ((0.0, 6.0, 0.0), 5, 4.0)], jitter=0.2, seed=3)
    x = XDG(m)
    x.prepare_raytracer()
    tm = m.tets
    rng0 = np.random.default_rng(9)
    n = 3000
    p = rng0.uniform(0.2, 3.8, (n, 3))
    _, elem = x.find_element(p)
    assert (elem >= 0).all()
    u = synth.isotropic_dirs(rng0, n)
    u[: n // 2] = np.array([1.0, 0.0, 0.0])
    seeds = x.rti.seed_streams(123, n)
    got = x.walk_particles(elem, p, u, seeds, mfp=20.0, precision=prec, tally=True)
    w = _oracle_walker(oracle, m)
    ipc = oracle.volume_tree(m, m.implicit_complement)
    et = oracle.TetTree(tm.tet_xyz(), tm.elem_ids)
    o = w.walk_particles(ipc, et, elem, p, u, seeds, 20.0, 1_000_000)
    for k, name in enumerate(NAMES):
        assert_same(got[name], o[k], name)
    first = w.transport(elem, p, u, seeds, 20.0, 1_000_000)
    assert (got["distance"] > first[4]).sum() > n // 10  # many crossed a gap
    # the tally holds the in-mesh path only: the gaps crossed are not in it
    assert 0.0 < got["tally"].sum() < got["distance"].sum()


# --------------------------------------------------------------------------
# particle_sim surface-tracking loop (tools/particle_sim.h:128-141)
# --------------------------------------------------------------------------

SNAMES = ["tree", "pos", "dir", "rng", "distance", "events", "status"]


def _same_tally(got, ref):
    """Per-tree path length, summed with atomics: within 1e-12 relative.
    The engine's array also has a slot for the global tree, never entered."""
    assert np.allclose(got[:len(ref)], ref, rtol=1e-12, atol=0)
    assert (got[len(ref):] == 0).all()


def _surface_run(x, prec, tree, p, u, seeds, mfp, max_events, grave=0, cap=16):
    n = len(tree)
    t, r, d, s = tree.copy(), p.copy(), u.copy(), seeds.copy()
    hist = np.zeros((n, cap), dtype=np.int32)
    hc = np.zeros(n, dtype=np.int32)
    dist, ev = np.zeros(n), np.zeros(n, dtype=np.int32)
    tally = np.zeros(x.rti.num_registered_surface_trees() + 1)
    st = x.rti.transport_surfaces(t, r, d, s, mfp, max_events, hist, hc, dist, ev, tally,
                                  grave, prec)
    return [t, r, d, s, dist, ev, st, tally, hist, hc]


@pytest.mark.parametrize("prec", [FP64, MIXED])
@pytest.mark.parametrize("case", ["vacuum", "graveyard", "reflecting"])
def test_transport_surfaces_sphere_in_box(cuda, oracle, prec, case):
    from xdg_gb300.engine import BC_REFLECTING, BC_VACUUM
    m = synth.single_sphere_in_box(level=3, radius=10.0, half_width=20.0)
    x = XDG(m)
    x.prepare_raytracer()
    bc = {2: BC_VACUUM} if case == "vacuum" else ({2: BC_REFLECTING} if case == "reflecting"
                                                   else {})
    if bc:
        x.rti.set_surface_boundary(bc)
    n = 3000
    rng0 = np.random.default_rng(4)
    p = rng0.uniform(-6.0, 6.0, (n, 3))
    u = synth.isotropic_dirs(rng0, n)
    seeds = x.rti.seed_streams(99, n)
    tree = np.full(n, x.volume_to_surface_tree[1], dtype=np.int32)
    grave = x.volume_to_surface_tree[3] if case == "graveyard" else 0
    max_ev = 300 if case == "reflecting" else 1_000_000
    got = _surface_run(x, prec, tree, p, u, seeds, 5.0, max_ev, grave)
    sim = oracle.SurfaceTransport(m, x.volume_to_surface_tree, bc)
    o = sim.run(tree, p, u, seeds, 5.0, max_ev, graveyard_tree=grave)
    for k, name in enumerate(SNAMES):
        assert_same(got[k], o[k], name)
    _same_tally(got[7], o[7])
    assert (got[6] == (7 if case == "reflecting" else 0)).all()


@pytest.mark.parametrize("prec", [FP64, MIXED])
def test_transport_surfaces_nested_spheres(cuda, oracle, prec):
    """Eight nested shells, transmission everywhere, the implicit complement
    as graveyard; the device path, the host-array path and a run cut at
    max_events then resumed all equal the oracle."""
    import torch
    m = synth.nested_spheres(n=8, level=3, jitter=1e-3, seed=7)
    x = XDG(m)
    x.prepare_raytracer()
    n = 4000
    rng0 = np.random.default_rng(8)
    p = rng0.uniform(-7.5, 7.5, (n, 3))
    u = synth.isotropic_dirs(rng0, n)
    vols = x.find_volume(p, u)
    keep = vols != m.implicit_complement
    p, u, vols = p[keep], u[keep], vols[keep]
    n = len(p)
    tree = x._trees(vols).astype(np.int32)
    seeds = x.rti.seed_streams(7, n)
    grave = x.volume_to_surface_tree[m.implicit_complement]
    sim = oracle.SurfaceTransport(m, x.volume_to_surface_tree)
    o = sim.run(tree, p, u, seeds, 0.7, 1_000_000, graveyard_tree=grave)
    # host arrays
    got = _surface_run(x, prec, tree, p, u, seeds, 0.7, 1_000_000, grave)
    for k, name in enumerate(SNAMES):
        assert_same(got[k], o[k], name)
    _same_tally(got[7], o[7])
    assert (got[0] == -1).all() and got[5].mean() > 10
    # events run one lane at a time or a whole warp at a time: same results
    for wait in (1, 32):
        x.rti.set_tuning("particle_event_wait", wait)
        try:
            g2 = _surface_run(x, prec, tree, p, u, seeds, 0.7, 1_000_000, grave)
        finally:
            x.rti.set_tuning("particle_event_wait", 16)
        for k, name in enumerate(SNAMES):
            assert_same(g2[k], o[k], f"{name} event_wait={wait}")
    # device tensors, cut at 5 events then resumed with the saved history
    dev = torch.device("cuda", 0)
    T = [torch.as_tensor(a, device=dev).clone() for a in
         (tree, p, u, seeds.view(np.int64), np.zeros((n, 16), np.int32), np.zeros(n, np.int32),
          np.zeros(n), np.zeros(n, np.int32))]
    st1 = x.rti.transport_surfaces(*T[:4], 0.7, 5, T[4], T[5], T[6], T[7], None, grave, prec)
    torch.cuda.synchronize()
    assert int((st1 == 7).sum()) > n // 2
    st2 = x.rti.transport_surfaces(*T[:4], 0.7, 1_000_000, T[4], T[5], T[6], T[7], None, grave,
                                   prec)
    res = [T[0].cpu().numpy(), T[1].cpu().numpy(), T[2].cpu().numpy(),
           T[3].cpu().numpy().view(np.uint64), T[6].cpu().numpy(), T[7].cpu().numpy(),
           st2.cpu().numpy()]
    for k, name in enumerate(SNAMES):
        assert_same(res[k], o[k], "resumed " + name)


def test_simulate_particles_facade(cuda):
    from xdg_gb300.engine import BC_VACUUM
    m = synth.single_sphere_in_box(level=3, radius=10.0, half_width=20.0)
    x = XDG(m)
    x.prepare_raytracer()
    x.rti.set_surface_boundary({2: BC_VACUUM})
    n = 500
    p = np.zeros((n, 3))
    u = np.tile([1.0, 0.0, 0.0], (n, 1))   # the tool's initial particle
    res = x.simulate_particles(np.ones(n, dtype=np.int32), p, u, x.rti.seed_streams(3, n),
                               mfp=1.0, tally=True)
    assert (res["status"] == 0).all() and (res["volume"] == 2).all()
    assert abs(sum(res["tally"].values()) - res["distance"].sum()) < 1e-9 * res["distance"].sum()
    with pytest.raises(Exception):
        x.rti.set_surface_boundary({77: BC_VACUUM})
