"""XDG::segments(start, end) (xdg.cpp:142-198) -- tracks across several
meshed volumes and the implicit complement between them -- on the CUDA
engine, against the oracle's track loop: element sequences and lengths bit
for bit, in both precisions."""
import numpy as np
import pytest

from xdg_gb300 import synth
from xdg_gb300.engine import FP64, MIXED, XDG

pytestmark = pytest.mark.gpu

PRECISIONS = [FP64, MIXED]


def compare(oracle, m, starts, ends, prec):
    x = XDG(m)
    x.prepare_raytracer()
    el, ln, off = x.segments_global(starts, ends, precision=prec)
    g = oracle.GlobalTracker(m)
    for i in range(len(starts)):
        oe, ol = g.segments(starts[i], ends[i])
        e_i, l_i = el[off[i]:off[i + 1]], ln[off[i]:off[i + 1]]
        assert np.array_equal(e_i, oe), f"track {i}: elements {e_i[:8]} vs {oe[:8]}"
        assert np.array_equal(l_i, ol), f"track {i}: lengths"
    return el, ln, off


def single_tet_tracks(oracle, m):
    tv = m.tets.vertices[m.tets.conn[0]]
    half = 2.0 * np.linalg.norm(tv.max(0) - tv.min(0))
    s = m.surfaces[0]
    a, b = [], []
    for tri in s.triangles:
        n = oracle.face_normal(s.vertices[tri].reshape(9))
        for vert in s.vertices[tri]:
            a.append(vert - n * half)
            b.append(vert + n * half)
    c = tv.mean(0)
    for vert in tv:
        d = oracle.normalize(vert - c)
        a += [c, vert + d * half]
        b += [vert + d * half, c]
    return np.array(a), np.array(b)


@pytest.mark.parametrize("prec", PRECISIONS)
@pytest.mark.parametrize("verts", [None, [[0.1, -0.2, 0.05], [1.3, 0.1, -0.1], [0.2, 1.1, 0.3],
                                          [-0.1, 0.3, 1.4]]])
def test_single_tet_tracks(cuda, oracle, prec, verts):
    """The single-tet vertex-tangent and vertex-crossing tracks of
    tests/test_tracks.cpp:125-300."""
    m = synth.single_tet(verts)
    a, b = single_tet_tracks(oracle, m)
    compare(oracle, m, a, b, prec)


@pytest.mark.parametrize("prec", PRECISIONS)
def test_blocks_with_gaps(cuda, oracle, prec):
    """Three jittered meshed blocks with gaps; tracks start and end inside,
    outside and between the blocks."""
    m = synth.tet_blocks([((0.0, 0.0, 0.0), 6, 10.0), ((12.0, 0.0, 0.0), 5, 10.0),
                          ((0.0, 11.0, 0.5), 4, 8.0)], jitter=0.2, seed=3)
    rng = np.random.default_rng(9)
    n = 1500
    a = rng.uniform([-4, -4, -4], [26, 23, 14], (n, 3))
    b = rng.uniform([-4, -4, -4], [26, 23, 14], (n, 3))
    el, ln, off = compare(oracle, m, a, b, prec)
    # tracks from inside a block to inside a block tally at least the
    # straight-line length inside the blocks they start and end in
    assert off[-1] > n


def test_blocks_track_length_sum(cuda):
    """A track crossing every block along x tallies the length inside the blocks."""
    m = synth.tet_blocks([((0.0, 0.0, 0.0), 5, 10.0), ((12.0, 0.0, 0.0), 5, 10.0),
                          ((24.0, 0.0, 0.0), 5, 10.0)], jitter=0.0)
    x = XDG(m)
    x.prepare_raytracer()
    rng = np.random.default_rng(4)
    n = 2000
    y = rng.uniform(0.5, 9.5, (n, 2))
    a = np.column_stack([np.full(n, -3.0), y])
    b = np.column_stack([np.full(n, 40.0), y])
    el, ln, off = x.segments_global(a, b)
    tot = np.add.reduceat(ln, off[:-1])
    assert np.allclose(tot, 30.0, rtol=1e-12)


def _gapped_blocks():
    return synth.tet_blocks([((0.0, 0.0, 0.0), 6, 10.0), ((12.0, 0.0, 0.0), 5, 10.0),
                             ((0.0, 11.0, 0.5), 4, 8.0)], jitter=0.2, seed=3)


@pytest.mark.parametrize("prec", PRECISIONS)
def test_device_arrays_and_status(cuda, prec):
    """The same tracks given as CUDA tensors: the call stays on the device
    (outputs are CUDA tensors) and gives the host call's segments; every
    track ends with status OK."""
    torch = cuda
    m = _gapped_blocks()
    x = XDG(m)
    x.prepare_raytracer()
    rng = np.random.default_rng(21)
    n = 3000
    a = rng.uniform([-4, -4, -4], [26, 23, 14], (n, 3))
    b = rng.uniform([-4, -4, -4], [26, 23, 14], (n, 3))
    el, ln, off = x.segments_global(a, b, precision=prec)
    ta, tb = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
    ipc = x.volume_to_surface_tree[m.implicit_complement]
    se, sl, toff, st = x.rti.segments_global(ipc, x.rti.global_element_tree, ta, tb, int(off[-1]),
                                             precision=prec)
    assert se.is_cuda and toff.is_cuda
    torch.cuda.synchronize()
    assert np.array_equal(toff.cpu().numpy(), off)
    assert np.array_equal(se.cpu().numpy()[:off[-1]], el)
    assert np.array_equal(sl.cpu().numpy()[:off[-1]], ln)
    assert int((st != 0).sum().item()) == 0


def test_capacity_and_round_limit(cuda, oracle):
    """Too small an output: offsets are complete, the tracks that do not fit
    are not written and get XDGCU_RAY_OUTPUT_FULL, the others are exact.  One
    round only: a track that needed a re-entry stops with
    XDGCU_RAY_WALK_LIMIT, and its segments are the first of the full loop's."""
    m = _gapped_blocks()
    x = XDG(m)
    x.prepare_raytracer()
    rng = np.random.default_rng(5)
    n = 400
    a = rng.uniform([-4, -4, -4], [26, 23, 14], (n, 3))
    b = rng.uniform([-4, -4, -4], [26, 23, 14], (n, 3))
    el, ln, off = x.segments_global(a, b)
    ipc = x.volume_to_surface_tree[m.implicit_complement]
    gt = x.rti.global_element_tree
    cap = int(off[-1]) // 2
    se, sl, off2, st = x.rti.segments_global(ipc, gt, a, b, cap)
    assert np.array_equal(off2, off)
    fits = off[1:] <= cap
    full = (~fits) & (off[1:] > off[:-1])
    assert np.array_equal(st == 6, full)  # XDGCU_RAY_OUTPUT_FULL
    for i in np.nonzero(fits)[0]:
        assert np.array_equal(se[off[i]:off[i + 1]], el[off[i]:off[i + 1]])
        assert np.array_equal(sl[off[i]:off[i + 1]], ln[off[i]:off[i + 1]])
    se1, sl1, off1, st1 = x.rti.segments_global(ipc, gt, a, b, int(off[-1]), max_rounds=1)
    g = oracle.GlobalTracker(m)
    limited = 0
    for i in range(n):
        e1, l1 = se1[off1[i]:off1[i + 1]], sl1[off1[i]:off1[i + 1]]
        ef, lf = el[off[i]:off[i + 1]], ln[off[i]:off[i + 1]]
        assert np.array_equal(e1, ef[:len(e1)]) and np.array_equal(l1, lf[:len(l1)])
        if st1[i] == 4:  # XDGCU_RAY_WALK_LIMIT
            limited += 1
        else:
            assert st1[i] == 0 and len(e1) == len(ef)
        oe, ol = g.segments(a[i], b[i], max_rounds=1)
        assert np.array_equal(e1, oe) and np.array_equal(l1, ol)
    assert limited > 0


@pytest.mark.parametrize("prec", PRECISIONS)
def test_tet_cube_tracks_leaving_the_mesh(cuda, oracle, prec):
    """A jittered 8^3 tet cube (one volume, the implicit complement around it):
    tracks from inside to points outside, from outside through the cube and
    from outside past it, against the oracle's loop."""
    tm = synth.tet_cube(n=8, size=8.0, jitter=0.2, seed=2)
    m = synth.model_from_tets(tm, np.ones(len(tm.conn), dtype=np.int32))
    rng = np.random.default_rng(31)
    n = 1200
    a = np.concatenate([rng.uniform(0.2, 7.8, (n // 2, 3)), rng.uniform(-6, 14, (n // 2, 3))])
    b = rng.uniform(-6, 14, (n, 3))
    compare(oracle, m, a, b, prec)


@pytest.mark.parametrize("prec", PRECISIONS)
def test_paused_walks_resume_exactly(cuda, oracle, prec):
    """Walks capped at 1, 3 and 8 segments per round pause and resume across
    many rounds; the segments equal the uncapped loop's and the oracle's."""
    m = _gapped_blocks()
    x = XDG(m)
    x.prepare_raytracer()
    rng = np.random.default_rng(41)
    n = 600
    a = rng.uniform([-4, -4, -4], [26, 23, 14], (n, 3))
    b = rng.uniform([-4, -4, -4], [26, 23, 14], (n, 3))
    ref = x.segments_global(a, b, precision=prec)
    try:
        for cap in (1, 3, 8):
            x.rti.set_tuning("segments_walk_cap", cap)
            got = x.segments_global(a, b, precision=prec)
            for u, v, what in zip(got, ref, ("elements", "lengths", "offsets")):
                assert np.array_equal(u, v), f"cap {cap}: {what}"
    finally:
        x.rti.set_tuning("segments_walk_cap", 0)
    g = oracle.GlobalTracker(m)
    el, ln, off = ref
    for i in range(0, n, 7):
        oe, ol = g.segments(a[i], b[i])
        assert np.array_equal(el[off[i]:off[i + 1]], oe) and np.array_equal(ln[off[i]:off[i + 1]], ol)
