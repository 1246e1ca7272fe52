"""Writes tests/golden/reference_vectors.npz from the reference's own code.

The vectors are produced by oracle/_ref/libxdg_ref.so, which oracle/Makefile
compiles from the reference's sources (include/xdg/geometry/plucker.h,
src/geometry/closest.cpp, src/mesh_manager_interface.cpp, ...).  They pin the
C oracle (and through it the CUDA engine) where the reference tree is absent.

    XDG_REFERENCE_DIR=<reference tree> python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as xo  # noqa: E402
from xdg_gb300 import synth  # noqa: E402

INF = xo.INFTY


def plucker_cases(rng):
    """Random and degenerate ray/triangle configurations."""
    cases = []
    # random triangles and rays
    for _ in range(700):
        v = rng.normal(0, 3, 9)
        o = rng.normal(0, 3, 3)
        d = rng.normal(0, 1, 3)
        d /= np.linalg.norm(d)
        cases.append((v, o, d))
    # rays aimed at vertices, edge midpoints and centroids (watertightness)
    for _ in range(1000):
        v = rng.normal(0, 3, 9).reshape(3, 3)
        o = rng.normal(0, 5, 3)
        k = rng.integers(0, 3)
        target = [v[k], 0.5 * (v[k] + v[(k + 1) % 3]), v.mean(0)][rng.integers(0, 3)]
        target = target + rng.normal(0, 1, 3) * 10.0 ** rng.uniform(-16, -8)
        d = target - o
        d /= np.linalg.norm(d)
        cases.append((v.reshape(9), o, d))
    # axis-aligned unit-ish geometry (mock-cube like), coplanar rays, zero direction
    for _ in range(300):
        v = rng.integers(-3, 4, 9).astype(np.float64)
        o = rng.integers(-5, 6, 3).astype(np.float64)
        d = np.zeros(3)
        d[rng.integers(0, 3)] = rng.choice([-1.0, 1.0])
        if rng.uniform() < 0.1:
            d = rng.integers(-1, 2, 3).astype(np.float64)
        cases.append((v, o, d))
    return cases


def main():
    if not xo.build_ref():
        raise SystemExit("reference sources not found (set XDG_REFERENCE_DIR to the reference "
                         "tree); cannot generate golden vectors")
    xo.build()
    R = xo.ref_lib()
    rng = np.random.default_rng(20241203)
    out = {}

    # Plucker test, both modes, several tMax values
    cases = plucker_cases(rng)
    V = np.array([c[0] for c in cases])
    O = np.array([c[1] for c in cases])
    D = np.array([c[2] for c in cases])
    n = len(cases)
    tmax = np.where(rng.uniform(size=n) < 0.5, INF, rng.uniform(0, 20, n))
    use_or = (rng.uniform(size=n) < 0.3).astype(np.int32)
    orient = np.where(rng.uniform(size=n) < 0.5, 1, -1).astype(np.int32)
    hit = np.zeros(n, dtype=np.int32)
    t = np.zeros(n)
    for i in range(n):
        h, tt = xo.plucker(V[i], O[i], D[i], tmax[i], 0.0, bool(use_or[i]), int(orient[i]), use_ref=True)
        hit[i] = h
        t[i] = tt if h else 0.0
    out.update(pl_v=V, pl_o=O, pl_d=D, pl_tmax=tmax, pl_use_or=use_or, pl_orient=orient,
               pl_hit=hit, pl_t=t)

    # closest point on triangle and its region
    m = 800
    CV = rng.normal(0, 2, (m, 9))
    CP = rng.normal(0, 4, (m, 3))
    CV[:200] = np.array([-1.0, -1.0, 0.0, 2.0, 1.0, 0.0, -2.0, 3.0, 0.0])  # test_closest.cpp:63-67
    CP[:200, 2] = 0.0
    cp = np.array([xo.closest_on_tri(CV[i], CP[i], use_ref=True) for i in range(m)])
    cr = np.array([xo.closest_region(CV[i], CP[i], use_ref=True) for i in range(m)], dtype=np.int32)
    out.update(cl_v=CV, cl_p=CP, cl_out=cp, cl_region=cr)

    # Vec3da::normalize, including a vector below min_rcp_input
    NV = np.concatenate([rng.normal(0, 10, (300, 3)), [[1e-40, 0.0, 0.0], [3.0, 4.0, 0.0]]])
    out.update(nv_in=NV, nv_out=np.array([xo.normalize(v, use_ref=True) for v in NV]))

    # next_element / walk_elements on a small jittered tet cube (MOAB order)
    tm = synth.tet_cube(n=4, size=4.0, jitter=0.2, seed=5)
    rw = xo.RefWalker(tm.vertices, tm.conn, tm.adj, tm.face_table)
    tt = xo.TetTree(tm.tet_xyz(), tm.elem_ids)
    ntr = 200
    S = rng.uniform(0.05, 3.95, (ntr, 3))
    U = synth.isotropic_dirs(rng, ntr)
    L = rng.uniform(0.0, 6.0, ntr)
    _, start = tt.find_element(S)
    assert (start >= 0).all()
    maxs = 128
    WE = np.full((ntr, maxs), -1, dtype=np.int32)
    WL = np.zeros((ntr, maxs))
    WC = np.zeros(ntr, dtype=np.int32)
    for i in range(ntr):
        e, ln = rw.walk(int(start[i]), S[i], U[i], float(L[i]), maxs)
        WC[i] = len(e)
        WE[i, :len(e)] = e
        WL[i, :len(e)] = ln
    out.update(tw_xyz=tm.vertices, tw_conn=tm.conn, tw_adj=tm.adj, tw_faces=tm.face_table,
               tw_start=start, tw_s=S, tw_u=U, tw_len=L, tw_elem=WE, tw_seglen=WL, tw_count=WC)

    # the MeshMock walk-to-corner chain of tests/test_tally_segments.cpp:26-71
    mm = synth.mock_cube(True)
    mw = xo.RefWalker(mm.tets.vertices, mm.tets.conn, mm.tets.adj, mm.tets.face_table)
    r = np.array([-1.0, -2.0, -3.0])
    ur = synth.MOCK_BOX_HI
    u = xo.normalize(ur - r, use_ref=True)
    mt = xo.TetTree(mm.tets.tet_xyz(), mm.tets.elem_ids)
    elem = int(mt.find_element([r])[1][0])
    chain_e, chain_d = [], []
    while elem != -1 and len(chain_e) < 100:
        nx, ex = mw.next_element(elem, r, u)
        chain_e.append(nx)
        chain_d.append(ex)
        r = r + u * ex
        elem = nx
    out.update(mock_chain_next=np.array(chain_e, dtype=np.int32), mock_chain_dist=np.array(chain_d),
               mock_chain_u=u)

    path = os.path.join(HERE, "reference_vectors.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
