"""Seeded synthetic geometry and ray sources for the XDG ray-query engine.

The reference measures on MOAB/libMesh model files that are not available
here; these generators build the same kinds of inputs in memory:

* ``mock_cube``  -- the in-memory MeshMock fixture of the reference tests
  (tests/mesh_mock.h:246-319): box [-2,5]x[-3,6]x[-4,7], 6 surfaces x 2
  triangles, 12 tets around the centre vertex with its adjacency table.
* ``icosphere`` / ``torus`` -- closed, outward-oriented triangle surfaces.
* ``tet_cube``   -- an n^3 hex grid split into 6 Kuhn tets per hex, MOAB face
  ordering (moab/direct_access.h:181-183), face adjacency built by vertex
  triple matching.
* ``lcg_*``       -- the LCG / Marsaglia ray sampler of
  tools/ray_benchmark.h:18-63 (state = seed ^ i per ray), vectorised.

All coordinates are float64.  Triangles are counter-clockwise seen from the
front face, so (v1-v0) x (v2-v0) is the outward normal (plucker.h:8-21).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

# MOAB canonical tet face ordering (moab/direct_access.h:181-183)
MOAB_TET_FACES = np.array([[0, 1, 3], [1, 2, 3], [2, 0, 3], [0, 2, 1]], dtype=np.int32)
# MeshMock face ordering (tests/mesh_mock.h:108-115)
MOCK_TET_FACES = np.array([[0, 1, 2], [0, 2, 3], [0, 3, 1], [1, 3, 2]], dtype=np.int32)


@dataclass
class Surface:
    """One surface: triangles (n x 3 vertex indices into ``vertices``)."""
    surface_id: int
    vertices: np.ndarray          # (nv, 3) float64
    triangles: np.ndarray         # (nt, 3) int32
    face_ids: np.ndarray          # (nt,) int32, mesh face ids
    forward_volume: int = -1
    reverse_volume: int = -1

    def tri_xyz(self) -> np.ndarray:
        """(nt, 9) float64: the three vertices of each triangle in mesh order."""
        return np.ascontiguousarray(self.vertices[self.triangles].reshape(-1, 9))


@dataclass
class Model:
    """A set of surfaces with volume senses, optionally with a tet mesh."""
    surfaces: list = field(default_factory=list)
    volumes: list = field(default_factory=list)
    implicit_complement: int = -1
    tets: "TetMesh | None" = None
    elements: dict = field(default_factory=dict)  # volume -> tet indices
    # MeshManager::get_boundary_face_element: tet index adjacent to each
    # surface face id (-1 for a face with no element), or None
    boundary_face_element: "np.ndarray | None" = None

    def volume_elements(self, vol):
        """MeshManager::get_volume_elements: tet indices of ``vol`` (or None)."""
        return self.elements.get(vol)

    def volume_surfaces(self, vol):
        """[(surface, sense)] with sense 0 forward / 1 reverse."""
        out = []
        for s in self.surfaces:
            if s.forward_volume == vol:
                out.append((s, 0))
            if s.reverse_volume == vol:
                out.append((s, 1))
        return out


@dataclass
class TetMesh:
    vertices: np.ndarray   # (nv, 3) float64
    conn: np.ndarray       # (n, 4) int32
    adj: np.ndarray        # (n, 4) int32, -1 on the boundary, in face_table order
    face_table: np.ndarray  # (4, 3) int32
    elem_ids: np.ndarray   # (n,) int32

    def tet_xyz(self) -> np.ndarray:
        return np.ascontiguousarray(self.vertices[self.conn].reshape(-1, 12))


# --------------------------------------------------------------------------
# MeshMock
# --------------------------------------------------------------------------

def mock_cube(volumetric_elements: bool = True, implicit_complement: bool = False) -> Model:
    """The reference test fixture MeshMock (tests/mesh_mock.h:17-321).

    One volume (id 0) with six surfaces 0..5 of two triangles each (faces
    2s, 2s+1), all forward-sensed to volume 0.  With ``implicit_complement``
    a volume 1 is added holding every surface in reverse sense, as
    MeshManager::create_implicit_complement does (mesh_manager_interface.cpp:19-45).
    """
    lo = np.array([-2.0, -3.0, -4.0])
    hi = np.array([5.0, 6.0, 7.0])
    c = 0.5 * (lo + hi)
    # upper z plane, then lower z plane, then the centre (mesh_mock.h:251-263)
    verts = np.array([
        [hi[0], lo[1], hi[2]], [hi[0], hi[1], hi[2]], [lo[0], hi[1], hi[2]], [lo[0], lo[1], hi[2]],
        [hi[0], lo[1], lo[2]], [hi[0], hi[1], lo[2]], [lo[0], hi[1], lo[2]], [lo[0], lo[1], lo[2]],
        c,
    ])
    tris = np.array([
        [0, 1, 2], [0, 2, 3],   # surface 0
        [4, 6, 5], [4, 7, 6],   # surface 1
        [0, 5, 1], [0, 4, 5],   # surface 2
        [2, 6, 7], [2, 7, 3],   # surface 3
        [1, 5, 6], [1, 6, 2],   # surface 4
        [0, 7, 4], [0, 3, 7],   # surface 5
    ], dtype=np.int32)
    tets = np.array([
        [0, 1, 2, 8], [0, 2, 3, 8], [4, 6, 5, 8], [4, 7, 6, 8],
        [0, 5, 1, 8], [0, 4, 5, 8], [2, 6, 7, 8], [2, 7, 3, 8],
        [0, 7, 4, 8], [0, 3, 7, 8], [1, 5, 6, 8], [1, 6, 2, 8],
    ], dtype=np.int32)
    adj = np.array([
        [-1, 1, 4, 11], [-1, 9, 0, 7], [-1, 5, 3, 10], [-1, 2, 8, 6],
        [-1, 0, 5, 10], [-1, 4, 8, 2], [-1, 7, 11, 3], [-1, 1, 6, 9],
        [-1, 5, 9, 3], [-1, 8, 1, 7], [-1, 11, 4, 2], [-1, 0, 10, 6],
    ], dtype=np.int32)
    m = Model()
    for s in range(6):
        m.surfaces.append(Surface(
            surface_id=s, vertices=verts, triangles=tris[2 * s:2 * s + 2],
            face_ids=np.array([2 * s, 2 * s + 1], dtype=np.int32),
            forward_volume=0, reverse_volume=-1))
    m.volumes = [0]
    if implicit_complement:
        for s in m.surfaces:
            s.reverse_volume = 1
        m.volumes.append(1)
        m.implicit_complement = 1
    if volumetric_elements:
        m.tets = TetMesh(vertices=verts, conn=tets, adj=adj,
                         face_table=MOCK_TET_FACES.copy(),
                         elem_ids=np.arange(12, dtype=np.int32))
        # MeshMock::get_volume_elements ignores its argument and returns all
        # twelve tets for every volume (mesh_mock.h:77-80)
        m.elements = {v: np.arange(12, dtype=np.int32) for v in m.volumes}
    return m


MOCK_BOX_LO = np.array([-2.0, -3.0, -4.0])
MOCK_BOX_HI = np.array([5.0, 6.0, 7.0])


# --------------------------------------------------------------------------
# Closed surfaces
# --------------------------------------------------------------------------

def icosphere(level: int, radius: float = 1.0, center=(0.0, 0.0, 0.0),
              jitter: float = 0.0, seed: int = 0):
    """Icosahedron subdivided ``level`` times, projected to the sphere.

    20*4^level triangles, 10*4^level + 2 vertices, outward CCW.  ``jitter``
    scales each vertex radially by (1 + U(-jitter, jitter)).
    """
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = np.array([
        [-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0],
        [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
        [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], dtype=np.float64)
    f = np.array([
        [0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
        [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
        [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
        [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], dtype=np.int64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    for _ in range(level):
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
        e.sort(axis=1)
        key = e[:, 0] * (len(v) + 1) + e[:, 1]
        uniq, inv = np.unique(key, return_inverse=True)
        a = uniq // (len(v) + 1)
        b = uniq % (len(v) + 1)
        mid = v[a] + v[b]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        base = len(v)
        v = np.concatenate([v, mid])
        nf = len(f)
        m01 = base + inv[:nf]
        m12 = base + inv[nf:2 * nf]
        m20 = base + inv[2 * nf:]
        f = np.concatenate([
            np.stack([f[:, 0], m01, m20], 1),
            np.stack([f[:, 1], m12, m01], 1),
            np.stack([f[:, 2], m20, m12], 1),
            np.stack([m01, m12, m20], 1)])
    r = np.full(len(v), float(radius))
    if jitter:
        rng = np.random.default_rng(seed)
        r = r * (1.0 + rng.uniform(-jitter, jitter, len(v)))
    v = v * r[:, None] + np.asarray(center, dtype=np.float64)
    # make every triangle outward (CCW seen from outside)
    n = np.cross(v[f[:, 1]] - v[f[:, 0]], v[f[:, 2]] - v[f[:, 0]])
    cen = (v[f[:, 0]] + v[f[:, 1]] + v[f[:, 2]]) / 3.0 - np.asarray(center)
    flip = (n * cen).sum(1) < 0
    f[flip] = f[flip][:, [0, 2, 1]]
    return v, f.astype(np.int32)


def torus(major: float, minor: float, n_major: int, n_minor: int, center=(0.0, 0.0, 0.0)):
    """Closed torus around the z axis, 2*n_major*n_minor outward triangles."""
    i = np.arange(n_major)
    j = np.arange(n_minor)
    th = 2 * np.pi * i / n_major
    ph = 2 * np.pi * j / n_minor
    TH, PH = np.meshgrid(th, ph, indexing="ij")
    x = (major + minor * np.cos(PH)) * np.cos(TH)
    y = (major + minor * np.cos(PH)) * np.sin(TH)
    z = minor * np.sin(PH)
    v = np.stack([x, y, z], -1).reshape(-1, 3) + np.asarray(center, dtype=np.float64)
    I, J = np.meshgrid(i, j, indexing="ij")
    a = I * n_minor + J
    b = ((I + 1) % n_major) * n_minor + J
    c = ((I + 1) % n_major) * n_minor + (J + 1) % n_minor
    d = I * n_minor + (J + 1) % n_minor
    f = np.concatenate([np.stack([a, b, c], -1).reshape(-1, 3),
                        np.stack([a, c, d], -1).reshape(-1, 3)])
    # orient outward: normal away from the tube centre line
    p0, p1, p2 = v[f[:, 0]], v[f[:, 1]], v[f[:, 2]]
    n = np.cross(p1 - p0, p2 - p0)
    cen = (p0 + p1 + p2) / 3.0 - np.asarray(center)
    ring = cen.copy()
    ring[:, 2] = 0
    ring *= (major / np.maximum(np.linalg.norm(ring, axis=1, keepdims=True), 1e-300))
    flip = (n * (cen - ring)).sum(1) < 0
    f[flip] = f[flip][:, [0, 2, 1]]
    return v, f.astype(np.int32)


def box_surface(lo, hi):
    """Axis-aligned box as 12 outward triangles (8 vertices)."""
    lo = np.asarray(lo, dtype=np.float64)
    hi = np.asarray(hi, dtype=np.float64)
    v = np.array([[x, y, z] for z in (lo[2], hi[2]) for y in (lo[1], hi[1])
                  for x in (lo[0], hi[0])], dtype=np.float64)
    # vertex index = x + 2y + 4z bits
    quads = [(0, 2, 3, 1), (4, 5, 7, 6), (0, 1, 5, 4), (2, 6, 7, 3), (0, 4, 6, 2), (1, 3, 7, 5)]
    f = []
    for a, b, c, d in quads:
        f += [[a, b, c], [a, c, d]]
    f = np.array(f, dtype=np.int64)
    n = np.cross(v[f[:, 1]] - v[f[:, 0]], v[f[:, 2]] - v[f[:, 0]])
    cen = (v[f[:, 0]] + v[f[:, 1]] + v[f[:, 2]]) / 3.0 - 0.5 * (lo + hi)
    flip = (n * cen).sum(1) < 0
    f[flip] = f[flip][:, [0, 2, 1]]
    return v, f.astype(np.int32)


# --------------------------------------------------------------------------
# Models for the benchmark configurations
# --------------------------------------------------------------------------

def single_sphere_in_box(level=4, radius=10.0, half_width=20.0) -> Model:
    """Icosphere (surface 1) inside a cube boundary (surface 2).

    Volume 1: inside the sphere; volume 2: between sphere and cube;
    volume 3: the implicit complement outside the cube.
    """
    m = Model()
    v, f = icosphere(level, radius)
    m.surfaces.append(Surface(1, v, f, np.arange(len(f), dtype=np.int32), 1, 2))
    bv, bf = box_surface([-half_width] * 3, [half_width] * 3)
    m.surfaces.append(Surface(2, bv, bf, np.arange(len(f), len(f) + len(bf), dtype=np.int32), 2, 3))
    m.volumes = [1, 2, 3]
    m.implicit_complement = 3
    return m


def nested_spheres(n=8, level=6, jitter=1e-3, seed=7) -> Model:
    """n concentric icospheres of radii 1..n, each vertex radially jittered.

    Sphere k is surface k with forward volume k (inside it) and reverse volume
    k+1; volume n+1 is the implicit complement.
    """
    m = Model()
    base = 0
    for k in range(1, n + 1):
        v, f = icosphere(level, float(k), jitter=jitter, seed=seed * 1000 + k)
        ids = np.arange(base, base + len(f), dtype=np.int32)
        base += len(f)
        m.surfaces.append(Surface(k, v, f, ids, k, k + 1))
    m.volumes = list(range(1, n + 2))
    m.implicit_complement = n + 1
    return m


def tet_cube(n=50, size=10.0, jitter=0.2, seed=11, origin=(0.0, 0.0, 0.0)) -> TetMesh:
    """[0,size]^3 as n^3 hexes x 6 Kuhn tets, MOAB face order, adjacency.

    Interior vertices are jittered by U(-jitter, jitter) * cell size per axis.
    Every tet is positively oriented (det[v1-v0, v2-v0, v3-v0] > 0), so the
    MOAB faces {0,1,3},{1,2,3},{2,0,3},{0,2,1} point outward.
    """
    h = size / n
    g = np.arange(n + 1)
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    idx = lambda i, j, k: (i * (n + 1) + j) * (n + 1) + k  # noqa: E731
    verts = np.stack([X, Y, Z], -1).reshape(-1, 3).astype(np.float64) * h
    if jitter:
        rng = np.random.default_rng(seed)
        interior = ((X > 0) & (X < n) & (Y > 0) & (Y < n) & (Z > 0) & (Z < n)).reshape(-1)
        verts[interior] += rng.uniform(-jitter * h, jitter * h, (interior.sum(), 3))
    verts += np.asarray(origin, dtype=np.float64)
    I, J, K = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    I, J, K = I.reshape(-1), J.reshape(-1), K.reshape(-1)
    unit = np.eye(3, dtype=np.int64)
    tets = []
    for perm in ([0, 1, 2], [0, 2, 1], [1, 0, 2], [1, 2, 0], [2, 0, 1], [2, 1, 0]):
        p0 = np.stack([I, J, K], 1)
        p1 = p0 + unit[perm[0]]
        p2 = p1 + unit[perm[1]]
        p3 = p0 + 1
        tets.append(np.stack([idx(*p.T) for p in (p0, p1, p2, p3)], 1))
    conn = np.stack(tets, 1).reshape(-1, 4).astype(np.int64)
    # orient positively
    a, b, c, d = (verts[conn[:, i]] for i in range(4))
    det = np.einsum("ij,ij->i", np.cross(b - a, c - a), d - a)
    neg = det < 0
    conn[neg] = conn[neg][:, [0, 2, 1, 3]]
    a, b, c, d = (verts[conn[:, i]] for i in range(4))
    det = np.einsum("ij,ij->i", np.cross(b - a, c - a), d - a)
    if (det <= 0).any():
        raise ValueError("tet_cube: jitter produced inverted tets")
    conn = conn.astype(np.int32)
    adj = face_adjacency(conn, MOAB_TET_FACES)
    return TetMesh(vertices=verts, conn=conn, adj=adj, face_table=MOAB_TET_FACES.copy(),
                   elem_ids=np.arange(len(conn), dtype=np.int32))


def face_adjacency(conn: np.ndarray, face_table: np.ndarray) -> np.ndarray:
    """(n, 4) neighbour across each local face (-1 on the boundary)."""
    n = len(conn)
    faces = conn[:, face_table].reshape(-1, 3).astype(np.int64)  # (4n, 3)
    faces.sort(axis=1)
    nv = int(conn.max()) + 1
    key = (faces[:, 0] * nv + faces[:, 1]) * nv + faces[:, 2]
    order = np.argsort(key, kind="stable")
    ks = key[order]
    adj = np.full(4 * n, -1, dtype=np.int64)
    same = np.nonzero(ks[1:] == ks[:-1])[0]
    a = order[same]
    b = order[same + 1]
    adj[a] = b // 4
    adj[b] = a // 4
    return adj.reshape(n, 4).astype(np.int32)


# --------------------------------------------------------------------------
# Ray sources
# --------------------------------------------------------------------------

_M32 = np.uint64(0xFFFFFFFF)


def _rand01(state: np.ndarray) -> np.ndarray:
    """tools/ray_benchmark.h:18-22, in place on a uint64 array of uint32 states."""
    state *= np.uint64(1664525)
    state += np.uint64(1013904223)
    state &= _M32
    return state.astype(np.float64) * (1.0 / 4294967296.0)


def _unit_dir(state: np.ndarray) -> np.ndarray:
    """tools/ray_benchmark.h:24-40 (Marsaglia), vectorised rejection loop."""
    n = len(state)
    out = np.empty((n, 3))
    todo = np.arange(n)
    while len(todo):
        st = state[todo]
        x1 = _rand01(st) * 2.0 - 1.0
        x2 = _rand01(st) * 2.0 - 1.0
        state[todo] = st
        s = x1 * x1 + x2 * x2
        ok = (s > 0.0) & (s < 1.0)
        t = 2.0 * np.sqrt(1.0 - s[ok])
        out[todo[ok], 0] = x1[ok] * t
        out[todo[ok], 1] = x2[ok] * t
        out[todo[ok], 2] = 1.0 - 2.0 * s[ok]
        todo = todo[~ok]
    return out


def lcg_states(n: int, seed: int = 12345) -> np.ndarray:
    """Per-ray LCG state seed ^ i (tools/ray_benchmark.cpp:189)."""
    return (np.uint64(seed) ^ np.arange(n, dtype=np.uint64)) & _M32


def lcg_ball_rays(n: int, radius: float, seed: int = 12345, center=(0.0, 0.0, 0.0)):
    """Isotropic directions from origins uniform in a ball of ``radius``.

    Follows the ray_benchmark sampler (tools/ray_benchmark.h:42-63) but draws
    a second, independent direction for the origin offset, so the directions
    are isotropic with respect to the origins (the tool reuses the ray
    direction as the offset direction, which makes every ray point radially
    outward).
    """
    st = lcg_states(n, seed)
    d = _unit_dir(st)
    off = _unit_dir(st)
    r = radius * np.cbrt(_rand01(st))
    o = np.asarray(center, dtype=np.float64) + off * r[:, None]
    return np.ascontiguousarray(o), np.ascontiguousarray(d)


def lcg_benchmark_rays(n: int, origin, source_radius: float, seed: int = 12345):
    """Exactly tools/ray_benchmark.h:42-63 (offset along the ray direction)."""
    st = lcg_states(n, seed)
    d = _unit_dir(st)
    o = np.tile(np.asarray(origin, dtype=np.float64), (n, 1))
    if source_radius > 0.0:
        r = source_radius * np.cbrt(_rand01(st))
        o = o + d * r[:, None]
    return np.ascontiguousarray(o), np.ascontiguousarray(d)


def isotropic_dirs(rng: np.random.Generator, n: int) -> np.ndarray:
    """Unit vectors uniform on the sphere (float64)."""
    z = rng.uniform(-1.0, 1.0, n)
    phi = rng.uniform(0.0, 2.0 * np.pi, n)
    s = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    return np.ascontiguousarray(np.stack([s * np.cos(phi), s * np.sin(phi), z], 1))


def normalize_rows(v: np.ndarray) -> np.ndarray:
    """Row-wise Vec3da::normalize (vec3da.h:61-66) with the min_rcp_input clamp."""
    min_rcp = float(np.float32(np.finfo(np.float32).tiny * 1e5))
    ln = np.sqrt(v[:, 0] * v[:, 0] + v[:, 1] * v[:, 1] + v[:, 2] * v[:, 2])
    ln = np.where(ln < min_rcp, min_rcp, ln)
    return np.ascontiguousarray(v / ln[:, None])


# --------------------------------------------------------------------------
# Degenerate-hit rays (watertightness stress) and many-surface models
# --------------------------------------------------------------------------

def watertight_rays(vertices: np.ndarray, triangles: np.ndarray, n: int, radius: float,
                    seed: int = 4):
    """Rays from origins uniform in a ball of ``radius`` aimed at triangle
    features: 40 % at a random vertex, 40 % at a random edge midpoint, 20 % at
    a centroid, each target moved by an isotropic jitter of length
    10^U(-12, -6).  Returns (origins, unit directions, kind) with kind 0 =
    vertex, 1 = edge, 2 = centroid."""
    rng = np.random.default_rng(seed)
    o = lcg_ball_rays(n, radius, seed=seed)[0]
    u = rng.uniform(0.0, 1.0, n)
    ti = rng.integers(0, len(triangles), n)
    corners = vertices[triangles[ti]]
    target = corners.mean(1)
    kind = np.full(n, 2, dtype=np.int8)
    vi = u < 0.4
    kind[vi] = 0
    target[vi] = corners[vi, rng.integers(0, 3, vi.sum())]
    ei = (u >= 0.4) & (u < 0.8)
    kind[ei] = 1
    a = rng.integers(0, 3, ei.sum())
    target[ei] = 0.5 * (corners[ei, a] + corners[ei, (a + 1) % 3])
    jit = 10.0 ** rng.uniform(-12.0, -6.0, n)
    target += isotropic_dirs(rng, n) * jit[:, None]
    return np.ascontiguousarray(o), normalize_rows(target - o), kind


@dataclass
class Shape:
    """Analytic description of a closed surface, for interior sampling."""
    kind: str                 # "sphere" or "torus"
    center: np.ndarray
    inner: float              # sphere: inscribed radius; torus: inscribed tube radius
    major: float = 0.0        # torus centre-line radius


def _sphere_inscribed(v: np.ndarray, f: np.ndarray, center: np.ndarray) -> float:
    p0, p1, p2 = v[f[:, 0]], v[f[:, 1]], v[f[:, 2]]
    n = np.cross(p1 - p0, p2 - p0)
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    return float(np.abs(((p0 - center) * n).sum(1)).min())


def many_surfaces(n: int = 256, seed: int = 5, tri_range=(1e3, 5e5), spacing: float = 4.0):
    """``n`` closed surfaces on a grid, alternating icosphere / torus, each the
    forward boundary of its own volume (surface k+1 bounds volume k+1); volume
    n+1 is the implicit complement around all of them.

    Triangle counts are 10^U(log10 lo, log10 hi): spheres take the nearest
    subdivision level (20*4^L triangles), tori an n_major x n_minor grid with
    R/r ~ U[2, 5].  Returns (model, shapes) with one ``Shape`` per surface.
    """
    rng = np.random.default_rng(seed)
    g = int(np.ceil(n ** (1.0 / 3.0) - 1e-9))
    m = Model()
    shapes = []
    base = 0
    lo, hi = np.log10(tri_range[0]), np.log10(tri_range[1])
    for k in range(n):
        cell = np.array([k % g, (k // g) % g, k // (g * g)], dtype=np.float64)
        c = spacing * (cell + 0.5)
        target = 10.0 ** rng.uniform(lo, hi)
        if k % 2 == 0:
            level = int(np.clip(np.round(np.log(target / 20.0) / np.log(4.0)), 1, 7))
            v, f = icosphere(level, 0.4 * spacing, c)
            shapes.append(Shape("sphere", c, _sphere_inscribed(v, f, c)))
        else:
            a = rng.uniform(2.0, 5.0)
            minor = 0.45 * spacing / (a + 1.0)
            major = a * minor
            n_minor = max(6, int(round(np.sqrt(target / (2.0 * a)))))
            n_major = max(12, int(round(a * n_minor)))
            v, f = torus(major, minor, n_major, n_minor, c)
            sag = ((major + minor) * (1.0 - np.cos(np.pi / n_major))
                   + minor * (1.0 - np.cos(np.pi / n_minor)))
            shapes.append(Shape("torus", c, minor - 1.5 * sag, major))
        ids = np.arange(base, base + len(f), dtype=np.int32)
        base += len(f)
        m.surfaces.append(Surface(k + 1, v, f, ids, k + 1, n + 1))
    m.volumes = list(range(1, n + 2))
    m.implicit_complement = n + 1
    return m, shapes


def interior_points(shape: Shape, count: int, rng: np.random.Generator, margin: float = 0.98):
    """``count`` points uniform inside the shape's inscribed solid, shrunk by
    ``margin`` (so they are strictly inside the triangulated surface)."""
    if shape.kind == "sphere":
        r = margin * shape.inner * np.cbrt(rng.uniform(0.0, 1.0, count))
        return shape.center + isotropic_dirs(rng, count) * r[:, None]
    tube = margin * shape.inner
    out = np.empty((0, 3))
    while len(out) < count:
        k = 2 * (count - len(out)) + 16
        s = tube * np.sqrt(rng.uniform(0.0, 1.0, k))
        ph = rng.uniform(0.0, 2.0 * np.pi, k)
        th = rng.uniform(0.0, 2.0 * np.pi, k)
        keep = rng.uniform(0.0, 1.0, k) * (shape.major + tube) < shape.major + s * np.cos(ph)
        rad = shape.major + s * np.cos(ph)
        p = np.stack([rad * np.cos(th), rad * np.sin(th), s * np.sin(ph)], 1)[keep]
        out = np.concatenate([out, p])
    return shape.center + out[:count]


def many_surface_rays(shapes, rng: np.random.Generator, ray_range=(1e3, 1e6)):
    """Per surface 10^U(log10 lo, log10 hi) rays from uniform interior origins
    with isotropic directions, grouped by volume.  Returns (origins, dirs,
    volume of each ray, offsets) with the rays of surface k at
    offsets[k]:offsets[k+1] and volume k+1."""
    lo, hi = np.log10(ray_range[0]), np.log10(ray_range[1])
    counts = np.round(10.0 ** rng.uniform(lo, hi, len(shapes))).astype(np.int64)
    offsets = np.concatenate([[0], np.cumsum(counts)])
    o = np.empty((offsets[-1], 3))
    for k, sh in enumerate(shapes):
        o[offsets[k]:offsets[k + 1]] = interior_points(sh, int(counts[k]), rng)
    d = isotropic_dirs(rng, int(offsets[-1]))
    vol = np.repeat(np.arange(1, len(shapes) + 1, dtype=np.int32), counts)
    return np.ascontiguousarray(o), d, vol, offsets


# --------------------------------------------------------------------------
# Meshed volumes bounded by their own boundary faces
# --------------------------------------------------------------------------

def model_from_tets(tm: TetMesh, tet_volume: np.ndarray) -> Model:
    """A model whose volumes are sets of tets: volume v (ids from
    ``tet_volume``) is bounded by one surface (id v) made of the boundary
    faces of its tets -- the faces without a neighbour -- with the outward
    orientation of the tet face (MOAB faces of a positive tet point out).
    The implicit complement (id max+1) holds every surface in reverse.
    ``boundary_face_element`` maps each face id to its tet, as
    MeshManager::get_boundary_face_element does (moab/direct_access.h:250-281).
    """
    tet_volume = np.asarray(tet_volume, dtype=np.int32)
    vols = sorted(int(v) for v in np.unique(tet_volume))
    ipc = vols[-1] + 1
    t_idx, f_idx = np.nonzero(tm.adj < 0)
    tris = tm.conn[t_idx[:, None], tm.face_table[f_idx]]
    # keep the outward orientation explicit (normal away from the tet centroid)
    v = tm.vertices
    n = np.cross(v[tris[:, 1]] - v[tris[:, 0]], v[tris[:, 2]] - v[tris[:, 0]])
    out = v[tris].mean(1) - v[tm.conn[t_idx]].mean(1)
    flip = (n * out).sum(1) < 0
    tris[flip] = tris[flip][:, [0, 2, 1]]
    m = Model()
    bfe = []
    base = 0
    for vol in vols:
        sel = np.nonzero(tet_volume[t_idx] == vol)[0]
        ids = np.arange(base, base + len(sel), dtype=np.int32)
        base += len(sel)
        m.surfaces.append(Surface(vol, v, tris[sel].astype(np.int32), ids, vol, ipc))
        bfe.append(t_idx[sel])
    m.volumes = vols + [ipc]
    m.implicit_complement = ipc
    m.tets = tm
    m.elements = {vol: np.nonzero(tet_volume == vol)[0].astype(np.int32) for vol in vols}
    m.boundary_face_element = np.concatenate(bfe).astype(np.int32)
    return m


def tet_blocks(blocks, jitter=0.2, seed=11) -> Model:
    """Separate meshed boxes, each its own volume (1, 2, ...), with gaps of
    implicit complement between them.  ``blocks`` is a list of (origin, n,
    size): an n^3 x 6 Kuhn-tet cube of edge ``size`` at ``origin``."""
    verts, conns, vol = [], [], []
    nv = 0
    for b, (origin, n, size) in enumerate(blocks):
        tm = tet_cube(n, size, jitter, seed + b, origin)
        verts.append(tm.vertices)
        conns.append(tm.conn + nv)
        vol.append(np.full(len(tm.conn), b + 1, dtype=np.int32))
        nv += len(tm.vertices)
    conn = np.concatenate(conns).astype(np.int32)
    tm = TetMesh(vertices=np.concatenate(verts), conn=conn,
                 adj=face_adjacency(conn, MOAB_TET_FACES), face_table=MOAB_TET_FACES.copy(),
                 elem_ids=np.arange(len(conn), dtype=np.int32))
    return model_from_tets(tm, np.concatenate(vol))


def single_tet(vertices=None) -> Model:
    """One positively oriented tet as volume 1 (one surface of its four faces);
    volume 2 is the implicit complement."""
    v = np.asarray(vertices if vertices is not None else
                   [[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0]],
                   dtype=np.float64)
    conn = np.array([[0, 1, 2, 3]], dtype=np.int32)
    a, b, c, d = v
    if np.dot(np.cross(b - a, c - a), d - a) < 0:
        conn = conn[:, [0, 2, 1, 3]]
    tm = TetMesh(vertices=v, conn=conn, adj=np.full((1, 4), -1, dtype=np.int32),
                 face_table=MOAB_TET_FACES.copy(), elem_ids=np.zeros(1, dtype=np.int32))
    return model_from_tets(tm, np.ones(1, dtype=np.int32))
