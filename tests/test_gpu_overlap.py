"""The overlap_check tool (tools/overlap.cpp) on the device against the oracle.

xdgcu_point_in_volumes tests every point in every volume in one launch; the
engine's XDG.check_overlaps runs the tool's vertex check (every face vertex
moved 1e-9 along +/- normalize(0.1, 0.1, 0.1), point_in_volume in every
volume) and edge check (a ray along every face edge in every volume that is
not a parent of the edge's surface).  The oracle restates the same loops
one query at a time; the inside flags and the sets of overlapping volumes
must be identical.
"""
import numpy as np
import pytest

from xdg_gb300 import synth
from xdg_gb300.engine import EXITING, FP64, MIXED, XDG

pytestmark = pytest.mark.gpu


def overlapping_spheres(level=2, shift=3.0):
    """Spheres A (volume 1) and B (volume 2), radius 5, centres shift apart
    along x: they overlap; volume 3 is the implicit complement."""
    m = synth.Model()
    va, fa = synth.icosphere(level, 5.0)
    vb, fb = synth.icosphere(level, 5.0, center=(shift, 0.0, 0.0))
    m.surfaces.append(synth.Surface(1, va, fa, np.arange(len(fa), dtype=np.int32), 1, 3))
    m.surfaces.append(synth.Surface(2, vb, fb, np.arange(len(fa), len(fa) + len(fb),
                                                         dtype=np.int32), 2, 3))
    m.volumes = [1, 2, 3]
    m.implicit_complement = 3
    return m


def oracle_overlaps(oracle, m, check_edges):
    """tools/overlap.cpp:9-191, one query at a time on oracle trees."""
    vols = list(m.volumes)
    ot = {v: oracle.volume_tree(m, v) for v in vols}
    d = np.array([0.1, 0.1, 0.1])
    d = d / np.sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2])
    found = {}
    verts = np.concatenate([s.tri_xyz().reshape(-1, 3) for s in m.surfaces])
    loc1 = verts + d * 1e-9
    loc2 = loc1 + ((-d) * 2.0) * 1e-9
    pts = np.empty((2 * len(verts), 3))
    pts[0::2], pts[1::2] = loc1, loc2
    dirs = np.empty_like(pts)
    dirs[0::2], dirs[1::2] = d, -d
    inside = np.stack([ot[v].point_in_volume(pts, dirs) for v in vols], axis=1)
    for j in np.nonzero(inside.sum(1) > 1)[0]:
        found.setdefault(frozenset(vols[k] for k in np.nonzero(inside[j])[0]), pts[j])
    if check_edges:
        parents = {s.surface_id: (s.forward_volume, s.reverse_volume) for s in m.surfaces}
        for s in m.surfaces:
            pf, pr = parents[s.surface_id]
            tri = s.tri_xyz().reshape(-1, 3, 3)
            for t in tri:
                for k in range(3):
                    v1, v2 = t[k], t[(k + 1) % 3]
                    dv = v2 - v1
                    ln = np.sqrt(dv[0] * dv[0] + dv[1] * dv[1] + dv[2] * dv[2])
                    dv = dv / ln
                    for v in vols:
                        if v in (pf, pr):
                            continue
                        th, sh, fh = ot[v].ray_fire(v1[None], dv[None], np.array([ln]), EXITING)
                        if sh[0] != -1:
                            found.setdefault(frozenset({parents[int(sh[0])][0], pf}),
                                             v1 + th[0] * dv)
                            break
    return inside, found


@pytest.mark.parametrize("prec", [FP64, MIXED])
def test_overlapping_spheres(cuda, oracle, prec):
    m = overlapping_spheres()
    x = XDG(m)
    x.prepare_raytracer()
    inside_o, found_o = oracle_overlaps(oracle, m, check_edges=True)
    found = x.check_overlaps(check_edges=True, precision=prec)
    assert set(found) == set(found_o)
    assert frozenset({1, 2}) in found
    # the inside matrix itself, host arrays and device tensors
    import torch
    vols = list(m.volumes)
    trees = [x.volume_to_surface_tree[v] for v in vols]
    verts = np.concatenate([s.tri_xyz().reshape(-1, 3) for s in m.surfaces])
    d = np.array([0.1, 0.1, 0.1]) / np.sqrt(0.03)
    pts = verts + d * 1e-9
    got = x.rti.point_in_volumes(pts, trees, np.tile(d, (len(pts), 1)), precision=prec)
    assert np.array_equal(got, inside_o[0::2])
    gd = x.rti.point_in_volumes(torch.from_numpy(pts).cuda(), trees,
                                torch.from_numpy(np.tile(d, (len(pts), 1))).cuda(),
                                precision=prec)
    torch.cuda.synchronize()
    assert np.array_equal(gd.cpu().numpy(), got)


@pytest.mark.parametrize("prec", [FP64, MIXED])
def test_nested_spheres_have_no_overlaps(cuda, oracle, prec):
    m = synth.nested_spheres(n=4, level=2, jitter=1e-3, seed=7)
    x = XDG(m)
    x.prepare_raytracer()
    assert x.check_overlaps(check_edges=True, precision=prec) == {}
    assert oracle_overlaps(oracle, m, check_edges=False)[1] == {}


def test_point_in_volumes_matches_point_in_volume(cuda):
    """Each column equals a point_in_volume launch in that tree, default
    direction included."""
    m = synth.nested_spheres(n=8, level=3, jitter=1e-3, seed=7)
    x = XDG(m)
    x.prepare_raytracer()
    rng = np.random.default_rng(3)
    p = rng.uniform(-9, 9, (20_000, 3))
    trees = [x.volume_to_surface_tree[v] for v in m.volumes]
    for dirs in (None, synth.isotropic_dirs(rng, len(p))):
        got = x.rti.point_in_volumes(p, trees, dirs)
        for k, t in enumerate(trees):
            assert np.array_equal(got[:, k], x.rti.point_in_volume(t, p, dirs)), (k, dirs is None)
        # no point is in two volumes of a valid model, and each point inside
        # the outer sphere is in exactly one (a point of the implicit
        # complement whose ray escapes reports outside, as the reference does)
        assert (got.sum(1) <= 1).all()
        r = np.sqrt((p * p).sum(1))
        assert (got[r < 7.9].sum(1) == 1).all()  # the coarse polyhedron lies inside r = 8
