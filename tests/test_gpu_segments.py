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
