"""Launch parameters and the autotuner do not change results.

The traversal's work distribution (contiguous slices or the device work
queue), the coherent ray order, the stack depth, the occupancy variant and
the node/flush schedule decide only which lane runs which ray when; ids and
distances must stay bit-identical to the default settings and to the oracle.
The autotuners must leave the context on settings that reproduce the same
outputs, and report a positive sample time.
"""
import numpy as np
import pytest

from xdg_gb300 import synth
from xdg_gb300.engine import (FP64, MIXED, QUERY_FIND_VOLUME, QUERY_POINT_IN_VOLUME,
                              QUERY_RAY_FIRE, TUNING_KEYS, XDG)

pytestmark = pytest.mark.gpu

SETTINGS = [
    {},
    {"trace_grab": 32},
    {"trace_grab": 256, "trace_sort_min": 1},
    {"trace_sort_min": 1},
    {"trace_stack": 64, "trace_occupancy": 2},
    {"trace_stack": 32, "trace_occupancy": 4, "trace_node_iters": 1, "trace_node_iters_fp64": 4},
    {"trace_grab": 4096, "trace_node_iters": 16, "trace_flush_wait": 32, "trace_stack": 40},
    {"trace_flush_wait": 1, "trace_grab": 64},
    {"trace_edge_table": 0},
    {"trace_edge_table": 0, "trace_grab": 64, "trace_stack": 48},
]


def assert_same(a, b, what):
    a = np.asarray(a)
    b = np.asarray(b)
    bad = np.nonzero(a != b)[0]
    assert len(bad) == 0, f"{what}: {len(bad)} mismatches, first at {bad[:5]}"


@pytest.fixture(scope="module")
def nested(cuda):
    m = synth.nested_spheres(n=8, level=3, jitter=1e-3, seed=7)
    x = XDG(m)
    x.prepare_raytracer()
    rng = np.random.default_rng(17)
    n = 120_000
    p = rng.uniform(-9, 9, (n, 3))
    d = synth.isotropic_dirs(rng, n)
    vols = x.find_volume(p, d)
    return m, x, p, d, vols


def _with(rti, settings):
    old = rti.tuning()
    for k, v in settings.items():
        rti.set_tuning(k, v)
    return old


def _restore(rti, old):
    for k, v in old.items():
        rti.set_tuning(k, v)


@pytest.mark.parametrize("prec", [FP64, MIXED])
def test_settings_do_not_change_results(nested, oracle, prec):
    """ray_fire with per-ray trees, point_in_volume and find_volume under
    every setting, host arrays (chunked staging) and device tensors."""
    import torch
    m, x, p, d, vols = nested
    base_t, base_s, base_f = x.ray_fire(vols, p, d, precision=prec)
    base_in = x.point_in_volume(3, p, precision=prec)
    base_fv = x.find_volume(p, d, precision=prec)
    # the default settings agree with the oracle (ascending volume order)
    sub = slice(0, 20_000)
    for v in np.unique(vols[sub]):
        k = np.nonzero(vols[sub] == v)[0]
        ot, os_, of = oracle.volume_tree(m, int(v)).ray_fire(p[k], d[k])
        assert_same(base_t[k], ot, f"t vol {v}")
        assert_same(base_f[k], of, f"face vol {v}")
    pd, dd = torch.from_numpy(p).cuda(), torch.from_numpy(d).cuda()
    td = torch.from_numpy(x._trees(vols)).cuda()
    for st in SETTINGS[1:]:
        old = _with(x.rti, st)
        try:
            t, s, f = x.ray_fire(vols, p, d, precision=prec)
            assert_same(t, base_t, f"t {st}")
            assert_same(s, base_s, f"surface {st}")
            assert_same(f, base_f, f"face {st}")
            assert_same(x.point_in_volume(3, p, precision=prec), base_in, f"piv {st}")
            assert_same(x.find_volume(p, d, precision=prec), base_fv, f"find_volume {st}")
            t2, s2, f2, status = x.rti.ray_fire(0, pd, dd, precision=prec, ray_trees=td,
                                                status=True)
            torch.cuda.synchronize()
            assert int((status != 0).sum()) == 0
            assert_same(t2.cpu().numpy(), base_t, f"device t {st}")
            assert_same(f2.cpu().numpy(), base_f, f"device face {st}")
        finally:
            _restore(x.rti, old)


def test_small_stack_overflow_is_reported(nested):
    """A requested 16-entry stack is raised to the trees' bound, (width - 1)
    x depth: no ray overflows, every result is kept."""
    import torch
    m, x, p, d, vols = nested
    pd, dd = torch.from_numpy(p).cuda(), torch.from_numpy(d).cuda()
    td = torch.from_numpy(x._trees(vols)).cuda()
    t0, s0, f0, st0 = x.rti.ray_fire(0, pd, dd, precision=MIXED, ray_trees=td, status=True)
    old = _with(x.rti, {"trace_stack": 16})
    try:
        t1, s1, f1, st1 = x.rti.ray_fire(0, pd, dd, precision=MIXED, ray_trees=td, status=True)
    finally:
        _restore(x.rti, old)
    st1 = st1.cpu().numpy()
    assert (st1 == 0).all()
    ok = st1 == 0
    assert_same(t1.cpu().numpy()[ok], t0.cpu().numpy()[ok], "t where no overflow")
    assert_same(f1.cpu().numpy()[ok], f0.cpu().numpy()[ok], "face where no overflow")


def test_bad_settings_rejected(nested):
    _, x, _, _, _ = nested
    for k, v in [("trace_stack", 12), ("trace_stack", 50), ("trace_stack", 72),
                 ("trace_grab", 33), ("trace_grab", -32), ("trace_sort_min", -1),
                 ("closest_bound", 2), ("trace_edge_table", -1), ("bvh_sah", 2),
                 ("bvh_prim_cost", 0)]:
        with pytest.raises(Exception):
            x.rti.set_tuning(k, v)
    assert set(x.rti.tuning()) == set(TUNING_KEYS)


@pytest.mark.parametrize("prec", [FP64, MIXED])
def test_autotune_trace(nested, prec):
    import torch
    m, x, p, d, vols = nested
    pd, dd = torch.from_numpy(p).cuda(), torch.from_numpy(d).cuda()
    td = torch.from_numpy(x._trees(vols)).cuda()
    t0, s0, f0 = x.rti.ray_fire(0, pd, dd, precision=prec, ray_trees=td)
    old = x.rti.tuning()
    try:
        ms, tuned = x.rti.autotune_trace(QUERY_RAY_FIRE, 0, pd, dd, precision=prec, ray_trees=td,
                                         reps=3)
        assert ms > 0
        assert tuned["trace_occupancy"] in (2, 3, 4) and tuned["trace_stack"] in (32, 40, 48, 64)
        t1, s1, f1 = x.rti.ray_fire(0, pd, dd, precision=prec, ray_trees=td)
        torch.cuda.synchronize()
        assert torch.equal(t0, t1) and torch.equal(s0, s1) and torch.equal(f0, f1)
        ms2, _ = x.rti.autotune_trace(QUERY_POINT_IN_VOLUME, 3, pd, None, precision=prec, reps=2)
        ms3, _ = x.rti.autotune_trace(QUERY_FIND_VOLUME, 0, pd, dd, precision=prec, reps=2)
        assert ms2 > 0 and ms3 > 0
    finally:
        _restore(x.rti, old)


def test_autotune_needs_device_sample(nested):
    m, x, p, d, vols = nested
    with pytest.raises(Exception, match="device memory"):
        x.rti.autotune_trace(QUERY_RAY_FIRE, 1, p[:100], d[:100])


@pytest.mark.parametrize("prec", [FP64, MIXED])
def test_autotune_walk(cuda, prec):
    import torch
    tm = synth.tet_cube(n=16, size=10.0, jitter=0.2, seed=11)
    m = synth.model_from_tets(tm, np.ones(len(tm.conn), dtype=np.int32))
    x = XDG(m)
    x.prepare_raytracer()
    rng = np.random.default_rng(3)
    n = 20_000
    p = rng.uniform(0.01, 9.99, (n, 3))
    u = synth.isotropic_dirs(rng, n)
    dist = np.minimum(rng.exponential(5.0, n), 30.0)
    eid, eidx = x.find_element(p)
    assert (eidx >= 0).all()
    dev = [torch.from_numpy(a).cuda() for a in (eidx.astype(np.int32), p, u, dist)]
    e0, l0, c0, _ = x.rti.walk_elements(*dev, max_segs=256, precision=prec)
    old = x.rti.tuning()
    try:
        ms, tuned = x.rti.autotune_walk(*dev, max_segs=256, precision=prec, reps=3)
        assert ms > 0
        e1, l1, c1, _ = x.rti.walk_elements(*dev, max_segs=256, precision=prec)
        torch.cuda.synchronize()
        assert torch.equal(c0, c1)
        c = c0.cpu().numpy()
        mask = np.arange(256)[None, :] < c[:, None]
        assert_same(e1.cpu().numpy()[mask], e0.cpu().numpy()[mask], "elements")
        assert_same(l1.cpu().numpy()[mask], l0.cpu().numpy()[mask], "lengths")
    finally:
        _restore(x.rti, old)


@pytest.mark.parametrize("prec", [FP64, MIXED])
def test_node_width_8(cuda, oracle, prec):
    """Trees built 8-wide (two 4-wide records per node) and rebuilt 4-wide
    give the same ids and distances for every query, equal to the oracle."""
    m = synth.nested_spheres(n=8, level=3, jitter=1e-3, seed=7)
    x8 = XDG(m)
    x8.rti.set_tuning("node_width", 8)
    x8.prepare_raytracer()
    assert x8.rti.tree_info(1)["width"] == 8
    x4 = XDG(m)
    x4.prepare_raytracer()
    assert x4.rti.tree_info(1)["width"] == 4
    rng = np.random.default_rng(23)
    n = 60_000
    p = rng.uniform(-9, 9, (n, 3))
    d = synth.isotropic_dirs(rng, n)
    vols = x4.find_volume(p, d, precision=prec)
    assert_same(x8.find_volume(p, d, precision=prec), vols, "find_volume")
    r8 = x8.ray_fire(vols, p, d, precision=prec)
    r4 = x4.ray_fire(vols, p, d, precision=prec)
    for a, b, what in zip(r8, r4, ("t", "surface", "face")):
        assert_same(a, b, what)
    k = np.nonzero(vols[:5000] == 4)[0]
    ot, os_, of = oracle.volume_tree(m, 4).ray_fire(p[k], d[k])
    assert_same(r8[0][k], ot, "t vs oracle")
    assert_same(r8[2][k], of, "face vs oracle")
    assert_same(x8.point_in_volume(5, p, precision=prec), x4.point_in_volume(5, p, precision=prec),
                "piv")
    c8, c4 = x8.closest(3, p[:5000], precision=prec), x4.closest(3, p[:5000], precision=prec)
    assert_same(c8[0], c4[0], "closest distance")
    assert_same(c8[1], c4[1], "closest face")
    # with most points' searches finished by a whole warp (8 children a node)
    pc = np.concatenate([np.zeros((1, 3)), p[:2000]])
    x8.rti.set_tuning("closest_step_budget", 4)
    try:
        w8 = x8.closest(3, pc, precision=prec)
    finally:
        x8.rti.set_tuning("closest_step_budget", 1024)
    ocd, ocf = oracle.volume_tree(m, 3).closest(pc)
    assert_same(w8[0], ocd, "closest distance, warp-finished, 8-wide")
    assert_same(w8[1], ocf, "closest face, warp-finished, 8-wide")
    o8, o4 = x8.occluded(2, p, d, precision=prec), x4.occluded(2, p, d, precision=prec)
    assert_same(o8[0], o4[0], "occluded")
    # back to 4-wide by a rebuild: same results again
    x8.rti.set_tuning("node_width", 4)
    x8.rti.rebuild_trees(3)
    assert x8.rti.tree_info(1)["width"] == 4
    for a, b, what in zip(x8.ray_fire(vols, p, d, precision=prec), r4, ("t", "surface", "face")):
        assert_same(a, b, "rebuilt " + what)


@pytest.mark.parametrize("prec", [FP64, MIXED])
@pytest.mark.parametrize("width", [4, 8])
def test_sah_and_greedy_collapse(cuda, oracle, prec, width):
    """Trees whose wide nodes are chosen by the surface-area cost (bvh_sah 1,
    the default, at two primitive costs) and greedily (bvh_sah 0) give the
    same ids and distances for every query, equal to the oracle; the SAH
    trees visit fewer nodes."""
    m = synth.nested_spheres(n=8, level=4, jitter=1e-3, seed=7)
    rng = np.random.default_rng(29)
    n = 60_000
    p = rng.uniform(-9, 9, (n, 3))
    d = synth.isotropic_dirs(rng, n)
    res = {}
    nodes = {}
    for sah, cost in ((0, 300), (1, 300), (1, 1500)):
        x = XDG(m)
        x.rti.set_tuning("node_width", width)
        x.rti.set_tuning("bvh_sah", sah)
        x.rti.set_tuning("bvh_prim_cost", cost)
        x.prepare_raytracer()
        vols = x.find_volume(p, d, precision=prec)
        x.rti.set_counting(True)
        rf = x.ray_fire(vols, p, d, precision=prec)
        nodes[(sah, cost)] = x.rti.counters()["node"]
        x.rti.set_counting(False)
        res[(sah, cost)] = (vols, rf, x.point_in_volume(5, p, precision=prec),
                            x.closest(3, p[:5000], precision=prec),
                            x.occluded(2, p, d, precision=prec))
    ref = res[(0, 300)]
    for key, r in res.items():
        assert_same(r[0], ref[0], f"find_volume {key}")
        for a, b, what in zip(r[1], ref[1], ("t", "surface", "face")):
            assert_same(a, b, f"{what} {key}")
        assert_same(r[2], ref[2], f"piv {key}")
        assert_same(r[3][0], ref[3][0], f"closest distance {key}")
        assert_same(r[3][1], ref[3][1], f"closest face {key}")
        assert_same(r[4][0], ref[4][0], f"occluded {key}")
    vols = ref[0]
    k = np.nonzero(vols[:5000] == 4)[0]
    ot, os_, of = oracle.volume_tree(m, 4).ray_fire(p[k], d[k])
    assert_same(res[(1, 300)][1][0][k], ot, "t vs oracle")
    assert_same(res[(1, 300)][1][2][k], of, "face vs oracle")
    assert nodes[(1, 300)] < nodes[(0, 300)]


@pytest.mark.parametrize("prec", [FP64, MIXED])
def test_sah_element_trees(cuda, prec):
    tm = synth.tet_cube(n=12, size=10.0, jitter=0.2, seed=11)
    m = synth.model_from_tets(tm, np.ones(len(tm.conn), dtype=np.int32))
    out = []
    for sah in (0, 1):
        x = XDG(m)
        x.rti.set_tuning("bvh_sah", sah)
        x.prepare_raytracer()
        rng = np.random.default_rng(5)
        out.append(x.find_element(rng.uniform(-0.5, 10.5, (50_000, 3)), precision=prec))
    assert_same(out[0][0], out[1][0], "element id")
    assert_same(out[0][1], out[1][1], "element index")


@pytest.mark.parametrize("prec", [FP64, MIXED])
def test_node_width_8_elements(cuda, prec):
    tm = synth.tet_cube(n=12, size=10.0, jitter=0.2, seed=11)
    m = synth.model_from_tets(tm, np.ones(len(tm.conn), dtype=np.int32))
    x8 = XDG(m)
    x8.rti.set_tuning("node_width", 8)
    x8.prepare_raytracer()
    x4 = XDG(m)
    x4.prepare_raytracer()
    rng = np.random.default_rng(5)
    p = rng.uniform(-0.5, 10.5, (50_000, 3))
    a, b = x8.find_element(p, precision=prec), x4.find_element(p, precision=prec)
    assert_same(a[0], b[0], "element id")
    assert_same(a[1], b[1], "element index")
    assert (a[0] >= 0).sum() > 35_000  # (10/11)^3 of the points lie in the cube


def test_scratch_pool(nested):
    """The calls' scratch comes from the context's pool, which keeps up to
    scratch_keep_bytes of it between calls: after a closest call (its
    deferral flags and seeds are scratch) the pool holds memory; setting 0
    releases it at once; results are the same."""
    _, x, p, _, vols = nested
    rti = x.rti
    keep = rti.get_tuning("scratch_keep_bytes")
    assert keep == 8 << 30
    ref = x.closest(2, p, MIXED)
    assert rti.get_tuning("scratch_bytes_reserved") > 0
    try:
        rti.set_tuning("scratch_keep_bytes", 0)
        assert rti.get_tuning("scratch_bytes_reserved") == 0
        rti.set_tuning("scratch_bytes_high", 0)
        got = x.closest(2, p, MIXED)
        assert rti.get_tuning("scratch_bytes_high") > 0
        assert_same(got[0], ref[0], "closest distance")
        assert_same(got[1], ref[1], "closest face")
        for k, v in [("scratch_keep_bytes", -1), ("scratch_bytes_high", 5)]:
            with pytest.raises(Exception):
                rti.set_tuning(k, v)
    finally:
        rti.set_tuning("scratch_keep_bytes", keep)


def test_find_element_phased(cuda, oracle):
    """The mixed find_element one lane per point (find_element_phased 0) and
    in warp-synchronous phases (1), and both precisions, with the points in
    Morton order (find_sort_min 1) and in the caller's (0), give the oracle's
    element ids and indices, for points inside the cube, on its faces, and
    on mesh vertices (on the faces of many tets at once, where the lowest
    element id decides)."""
    tm = synth.tet_cube(n=12, size=10.0, jitter=0.2, seed=11)
    m = synth.model_from_tets(tm, np.ones(len(tm.conn), dtype=np.int32))
    x = XDG(m)
    x.prepare_raytracer()
    rng = np.random.default_rng(9)
    inner = rng.uniform(-0.5, 10.5, (30_000, 3))
    face = rng.uniform(0.0, 10.0, (30_000, 3))
    face[np.arange(len(face)), rng.integers(0, 3, len(face))] = rng.choice([0.0, 10.0], len(face))
    verts = tm.vertices[rng.integers(0, len(tm.vertices), 10_000)]
    p = np.concatenate([inner, face, verts])
    oid, oidx = oracle.TetTree(tm.tet_xyz(), tm.elem_ids).find_element(p)
    assert x.rti.get_tuning("find_element_phased") == 0
    sort_min = x.rti.get_tuning("find_sort_min")
    try:
        for phased in (0, 1):
            x.rti.set_tuning("find_element_phased", phased)
            for smin in (1, 0):  # the points in Morton order, and in the caller's
                x.rti.set_tuning("find_sort_min", smin)
                for prec in (MIXED, FP64):
                    eid, eidx = x.find_element(p, precision=prec)
                    what = f"phased={phased} sort_min={smin} {prec}"
                    assert_same(eid, oid, f"element id, {what}")
                    assert_same(eidx, oidx, f"element index, {what}")
        with pytest.raises(Exception):
            x.rti.set_tuning("find_element_phased", 2)
        with pytest.raises(Exception):
            x.rti.set_tuning("find_sort_min", -1)
    finally:
        x.rti.set_tuning("find_element_phased", 0)
        x.rti.set_tuning("find_sort_min", sort_min)
    assert (oid >= 0).sum() > 50_000


def test_autotune_width(nested):
    """The tree-shape search rebuilds the trees and keeps results unchanged."""
    import torch
    m, x, p, d, vols = nested
    pd, dd = torch.from_numpy(p).cuda(), torch.from_numpy(d).cuda()
    td = torch.from_numpy(x._trees(vols)).cuda()
    t0, s0, f0 = x.rti.ray_fire(0, pd, dd, ray_trees=td)
    old = x.rti.tuning()
    try:
        ms, tuned = x.rti.autotune_trace(QUERY_RAY_FIRE, 0, pd, dd, ray_trees=td, reps=2,
                                         tune_tree=True)
        assert tuned["node_width"] in (4, 8) and tuned["leaf_max"] in (2, 3, 4)
        assert x.rti.tree_info(1)["width"] == tuned["node_width"]
        t1, s1, f1 = x.rti.ray_fire(0, pd, dd, ray_trees=td)
        torch.cuda.synchronize()
        assert torch.equal(t0, t1) and torch.equal(s0, s1) and torch.equal(f0, f1)
    finally:
        _restore(x.rti, old)
        x.rti.rebuild_trees(3)
