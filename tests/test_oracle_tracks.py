"""The oracle's global track loop (XDG::segments(start, end), xdg.cpp:142-198)
on the reference's single-tet track tests (tests/test_tracks.cpp:125-300),
restated on an in-memory tetrahedron, and on two meshed blocks with a gap."""
import numpy as np
import pytest

from xdg_gb300 import synth


def single_tet_cases():
    # an irregular tet so that no face is axis aligned
    return synth.single_tet([[0.1, -0.2, 0.05], [1.3, 0.1, -0.1], [0.2, 1.1, 0.3],
                             [-0.1, 0.3, 1.4]])


TANGENT_TETS = [None, [[1.0, 1.0, 1.0], [3.0, 1.0, 1.0], [1.0, 3.0, 1.0], [1.0, 1.0, 3.0]]]


def tangent_tracks(oracle, m):
    """Tracks through each face vertex along the face normal, skipping those
    that run along a tet edge (test_tracks.cpp:160-176)."""
    tv = m.tets.vertices[m.tets.conn[0]]
    half = 2.0 * np.linalg.norm(tv.max(0) - tv.min(0))
    s = m.surfaces[0]
    for tri in s.triangles:
        n = oracle.face_normal(s.vertices[tri].reshape(9))
        for vert in s.vertices[tri]:
            if any(np.linalg.norm(np.cross(w - vert, n)) < 1e-12
                   for w in tv if not np.array_equal(w, vert)):
                continue
            yield vert - n * half, vert + n * half


@pytest.mark.parametrize("verts", TANGENT_TETS)
def test_vertex_tangent_tracks_tally_nothing(oracle, verts):
    """test_tracks.cpp:125-198: tracks through a face vertex along the face
    normal touch the tet at that vertex only and tally nothing.  The tets
    here have exactly representable faces, like the reference's fixture: the
    walk then starts exactly at the vertex and leaves through a face at
    distance 0."""
    g = oracle.GlobalTracker(synth.single_tet(verts))
    cases = 0
    for a, b in tangent_tracks(oracle, g.model):
        el, ln = g.segments(a, b)
        assert abs(ln.sum()) <= 1e-12
        cases += 1
    assert cases > 0


def test_vertex_tangent_without_exit_face(oracle):
    """On an irregular tet the re-entry point lands a rounding error past
    the touched vertex in some of these tracks, so no face passes the exit
    test (t_min = 0, mesh_manager_interface.cpp:169-176).  The reference then
    tallies the remaining distance in the element (min(INFTY, distance),
    :120-124) and indexes the adjacency with -1 (undefined); the oracle and the
    engine tally the same and stop the track there."""
    m = single_tet_cases()
    g = oracle.GlobalTracker(m)
    tot = [g.segments(a, b)[1].sum() for a, b in tangent_tracks(oracle, m)]
    assert min(tot) <= 1e-12
    full = [t for t in tot if t > 1e-12]
    assert full and all(t > 1.0 for t in full)


def test_vertex_crossing_tracks(oracle):
    """test_tracks.cpp:200-300: centroid -> through a vertex -> outside, and
    back, tally the centroid-to-vertex distance."""
    m = single_tet_cases()
    g = oracle.GlobalTracker(m)
    tv = m.tets.vertices[m.tets.conn[0]]
    c = tv.mean(0)
    ext = np.linalg.norm(tv.max(0) - tv.min(0))
    for vert in tv:
        d = oracle.normalize(vert - c)
        out = vert + d * ext
        exp = np.linalg.norm(vert - c)
        fwd = g.segments(c, out)[1].sum()
        rev = g.segments(out, c)[1].sum()
        assert abs(fwd - exp) <= 1e-5 * exp
        assert abs(rev - exp) <= 1e-5 * exp


def test_two_blocks_with_gap(oracle):
    m = synth.tet_blocks([((0.0, 0.0, 0.0), 4, 10.0), ((12.0, 0.0, 0.0), 4, 10.0)])
    g = oracle.GlobalTracker(m)
    el, ln = g.segments([-5.0, 5.1, 4.9], [30.0, 5.2, 5.0])
    w = np.array([35.0, 0.1, 0.1])
    exp = 20.0 * np.linalg.norm(w) / 35.0
    assert abs(ln.sum() - exp) <= 1e-9 * exp
    assert (el[:len(el) // 2] < 384).any() and (el >= 384).any()
