"""The C++ tool loops (xdg_gb300/cpp/cuda_tools.*) against the Python engine.

tests/cpp/run_tools.cpp reads a model and a particle bank from binary files,
builds the C++ RayTracer backend over a MeshManager of that model, runs one
of walk_particles (the walk_elements tool loop), simulate_particles (the
particle_sim loop) or check_overlaps (the overlap_check tool) and writes the
results.  They must equal the Python engine's (XDG.walk_particles /
simulate_particles / check_overlaps, themselves checked against the oracle
in tests/test_gpu_transport.py and tests/test_gpu_overlap.py) bit for bit.
"""
import os
import struct
import subprocess

import numpy as np
import pytest

from conftest import ROOT
from xdg_gb300 import synth


def compile_tools(out_dir):
    from xdg_gb300 import build
    lib = build.build()
    lib_dir = os.path.dirname(lib)
    exe = os.path.join(out_dir, "run_tools")
    cpp = os.path.join(ROOT, "xdg_gb300", "cpp")
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", "-ffp-contract=off",
           "-I", os.path.join(ROOT, "include"), "-I", cpp,
           os.path.join(ROOT, "tests", "cpp", "run_tools.cpp"),
           os.path.join(cpp, "cuda_ray_tracer.cpp"), os.path.join(cpp, "cuda_tools.cpp"),
           "-L", lib_dir, "-lxdgcu", "-Wl,-rpath," + lib_dir, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


@pytest.fixture(scope="module")
def tools_exe(tmp_path_factory):
    return compile_tools(str(tmp_path_factory.mktemp("tools")))


def test_tools_compile_and_link(tools_exe):
    assert os.access(tools_exe, os.X_OK)


def _i32(*v):
    return struct.pack(f"<{len(v)}i", *v)


def write_model(path, m, bc=None):
    bc = bc or {}
    out = [_i32(len(m.surfaces))]
    for s in m.surfaces:
        out.append(_i32(s.surface_id, s.forward_volume, s.reverse_volume, len(s.face_ids)))
        out.append(np.ascontiguousarray(s.face_ids, dtype="<i4").tobytes())
        out.append(np.ascontiguousarray(s.tri_xyz(), dtype="<f8").tobytes())
    out.append(_i32(len(m.volumes)))
    out.append(np.asarray(m.volumes, dtype="<i4").tobytes())
    out.append(_i32(m.implicit_complement))
    out.append(_i32(len(bc)))
    for sid, code in bc.items():
        out.append(_i32(sid, code))
    tm = m.tets
    out.append(_i32(1 if tm is not None else 0))
    if tm is not None:
        out.append(_i32(len(tm.vertices)))
        out.append(np.ascontiguousarray(tm.vertices, dtype="<f8").tobytes())
        out.append(_i32(len(tm.conn)))
        out.append(np.ascontiguousarray(tm.conn, dtype="<i4").tobytes())
        out.append(np.ascontiguousarray(tm.adj, dtype="<i4").tobytes())
        out.append(np.ascontiguousarray(tm.elem_ids, dtype="<i4").tobytes())
        for v in m.volumes:
            e = m.volume_elements(v)
            e = np.zeros(0, dtype=np.int32) if e is None else np.asarray(e, dtype=np.int32)
            out.append(_i32(len(e)))
            out.append(e.astype("<i4").tobytes())
        bfe = m.boundary_face_element
        bfe = np.zeros(0, dtype=np.int32) if bfe is None else np.asarray(bfe, dtype=np.int32)
        out.append(_i32(len(bfe)))
        out.append(bfe.astype("<i4").tobytes())
    with open(path, "wb") as f:
        f.write(b"".join(out))


def write_bank_job(path, job, prec, cells, p, u, rng, mfp, max_events, extra=None):
    out = [_i32(job, prec, len(cells)), np.asarray(cells, dtype="<i4").tobytes(),
           np.ascontiguousarray(p, dtype="<f8").tobytes(),
           np.ascontiguousarray(u, dtype="<f8").tobytes(),
           np.ascontiguousarray(rng, dtype="<u8").tobytes(), struct.pack("<d", mfp),
           _i32(max_events)]
    if extra is not None:
        out.append(_i32(extra))
    with open(path, "wb") as f:
        f.write(b"".join(out))


def read_bank(path, n):
    raw = open(path, "rb").read()
    o = 0

    def take(dt, count):
        nonlocal o
        a = np.frombuffer(raw, dtype=dt, count=count, offset=o)
        o += a.nbytes
        return a

    cell = take("<i4", n)
    pos = take("<f8", 3 * n).reshape(n, 3)
    d = take("<f8", 3 * n).reshape(n, 3)
    rng = take("<u8", n)
    dist = take("<f8", n)
    ev = take("<i4", n)
    st = take("<i4", n)
    return dict(cell=cell, pos=pos, dir=d, rng=rng, distance=dist, events=ev, status=st)


def run(exe, tmp_path, model_path, job_path):
    out = str(tmp_path / "out.bin")
    r = subprocess.run([exe, model_path, job_path, out], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [0, 1])
def test_cpp_walk_particles(cuda, tools_exe, tmp_path, prec):
    from xdg_gb300.engine import XDG
    m = synth.tet_blocks([((0.0, 0.0, 0.0), 5, 4.0), ((6.0, 0.0, 0.0), 5, 4.0),
                          ((0.0, 6.0, 0.0), 5, 4.0)], jitter=0.2, seed=3)
    x = XDG(m)
    x.prepare_raytracer()
    rng0 = np.random.default_rng(9)
    n = 2000
    p = rng0.uniform(0.2, 3.8, (n, 3))
    _, eidx = x.find_element(p)
    u = synth.isotropic_dirs(rng0, n)
    u[: n // 2] = np.array([1.0, 0.0, 0.0])
    seeds = x.rti.seed_streams(123, n)
    ref = x.walk_particles(eidx, p, u, seeds, mfp=20.0, precision=prec)
    ids = m.tets.elem_ids
    model_path, job_path = str(tmp_path / "m.bin"), str(tmp_path / "j.bin")
    write_model(model_path, m)
    write_bank_job(job_path, 1, prec, ids[eidx], p, u, seeds, 20.0, 1_000_000)
    got = read_bank(run(tools_exe, tmp_path, model_path, job_path), n)
    ref_cell = np.where(ref["elem"] >= 0, ids[np.maximum(ref["elem"], 0)], -1)
    assert np.array_equal(got["cell"], ref_cell)
    for k in ("pos", "dir", "rng", "distance", "events", "status"):
        assert np.array_equal(got[k], ref[k]), k
    assert (ref["distance"] > 0).all()


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("case", ["vacuum", "graveyard", "reflecting"])
def test_cpp_simulate_particles(cuda, tools_exe, tmp_path, prec, case):
    from xdg_gb300.engine import BC_REFLECTING, BC_VACUUM, XDG
    m = synth.nested_spheres(n=4, level=3, jitter=1e-3, seed=7)
    bc = {4: 1} if case == "vacuum" else ({4: 2} if case == "reflecting" else {})
    x = XDG(m)
    x.prepare_raytracer()
    if bc:
        x.rti.set_surface_boundary({s: (BC_VACUUM if c == 1 else BC_REFLECTING)
                                    for s, c in bc.items()})
    n = 1500
    rng0 = np.random.default_rng(8)
    p = rng0.uniform(-2.5, 2.5, (n, 3))
    u = synth.isotropic_dirs(rng0, n)
    vols = x.find_volume(p, u)
    seeds = x.rti.seed_streams(7, n)
    max_ev = 200 if case == "reflecting" else 1_000_000
    ref = x.simulate_particles(vols, p, u, seeds, mfp=0.8, max_events=max_ev,
                               ipc_graveyard=(case == "graveyard"), precision=prec)
    model_path, job_path = str(tmp_path / "m.bin"), str(tmp_path / "j.bin")
    write_model(model_path, m, bc)
    write_bank_job(job_path, 2, prec, vols, p, u, seeds, 0.8, max_ev,
                   extra=1 if case == "graveyard" else 0)
    got = read_bank(run(tools_exe, tmp_path, model_path, job_path), n)
    assert np.array_equal(got["cell"], ref["volume"])
    for k in ("pos", "dir", "rng", "distance", "events", "status"):
        assert np.array_equal(got[k], ref[k]), k


def overlapping_spheres(level=2, shift=3.0):
    m = synth.Model()
    va, fa = synth.icosphere(level, 5.0)
    vb, fb = synth.icosphere(level, 5.0, center=(shift, 0.0, 0.0))
    m.surfaces.append(synth.Surface(1, va, fa, np.arange(len(fa), dtype=np.int32), 1, 3))
    m.surfaces.append(synth.Surface(2, vb, fb, np.arange(len(fa), len(fa) + len(fb),
                                                         dtype=np.int32), 2, 3))
    m.volumes = [1, 2, 3]
    m.implicit_complement = 3
    return m


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [0, 1])
def test_cpp_check_overlaps(cuda, tools_exe, tmp_path, prec):
    from xdg_gb300.engine import XDG
    m = overlapping_spheres()
    x = XDG(m)
    x.prepare_raytracer()
    ref = x.check_overlaps(check_edges=True, precision=prec)
    model_path, job_path = str(tmp_path / "m.bin"), str(tmp_path / "j.bin")
    write_model(model_path, m)
    with open(job_path, "wb") as f:
        f.write(_i32(3, prec, 1))
    raw = open(run(tools_exe, tmp_path, model_path, job_path), "rb").read()
    cnt = struct.unpack_from("<i", raw, 0)[0]
    o = 4
    got = {}
    for _ in range(cnt):
        k = struct.unpack_from("<i", raw, o)[0]
        vols = struct.unpack_from(f"<{k}i", raw, o + 4)
        loc = np.array(struct.unpack_from("<3d", raw, o + 4 + 4 * k))
        o += 4 + 4 * k + 24
        got[frozenset(vols)] = loc
    assert set(got) == set(ref) and frozenset({1, 2}) in got
    for key in got:
        assert np.array_equal(got[key], ref[key]), key


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [0, 1])
def test_cpp_track_segments(cuda, tools_exe, tmp_path, prec):
    """Tracks across three meshed blocks with gaps, starting and ending
    inside, outside and between the blocks, some of zero length."""
    from xdg_gb300.engine import XDG
    m = synth.tet_blocks([((0.0, 0.0, 0.0), 6, 10.0), ((12.0, 0.0, 0.0), 5, 10.0),
                          ((0.0, 11.0, 0.5), 4, 8.0)], jitter=0.2, seed=3)
    x = XDG(m)
    x.prepare_raytracer()
    rng = np.random.default_rng(5)
    n = 1500
    a = rng.uniform([-4, -4, -4], [26, 23, 14], (n, 3))
    b = rng.uniform([-4, -4, -4], [26, 23, 14], (n, 3))
    b[:10] = a[:10]
    el, ln, off = x.segments_global(a, b, precision=prec)
    model_path, job_path = str(tmp_path / "m.bin"), str(tmp_path / "j.bin")
    write_model(model_path, m)
    with open(job_path, "wb") as f:
        f.write(_i32(4, prec, n) + np.ascontiguousarray(a, dtype="<f8").tobytes()
                + np.ascontiguousarray(b, dtype="<f8").tobytes())
    raw = open(run(tools_exe, tmp_path, model_path, job_path), "rb").read()
    got_off = np.frombuffer(raw, dtype="<i8", count=n + 1)
    tot = int(got_off[-1])
    got_el = np.frombuffer(raw, dtype="<i4", count=tot, offset=8 * (n + 1))
    got_ln = np.frombuffer(raw, dtype="<f8", count=tot, offset=8 * (n + 1) + 4 * tot)
    assert np.array_equal(got_off, off)
    assert np.array_equal(got_el, el)
    assert np.array_equal(got_ln, ln)
    assert tot > n and (np.diff(off)[:10] == 0).all()
