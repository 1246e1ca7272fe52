"""Benchmark of the XDG ray-query hot path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl engine|reference]

Headline workload (one JSON line on rank 0): 8 nested, radially jittered
level-6 icospheres (radii 1..8, 9 volumes) and 1e7 rays from uniform points
in [-9,9]^3 with isotropic directions, each fired (EXITING) in the volume
point_in_volume/find_volume assigns it.  One step = one batched ray_fire of
all 1e7 rays, inputs resident in HBM; `value` is mixed-precision Mrays/s.
Beside it the line reports the all-FP64 path on the same rays, the 1e7
point_in_volume queries, and the tet-walk workload (50^3 hexes x 6 jittered
Kuhn tets = 750,000 tets, 1e6 tracks: find_element + walk_elements) in
Msegs/s for both precisions, plus id/distance agreement between the two
precisions and against the CPU oracle on a sample.

All inputs are seeded synthetic data (the reference's model files are not
available).  The streamed inputs (1e7 rays x 52 B = 520 MB) exceed the
129 MB L2, so no explicit L2 flush is done between steps; the BVHs (the
model) stay cache resident, as they would in production.

--impl reference times the reference algorithm on the host cores instead:
the C restatement of the reference's FP64 path (oracle/, BVH mode, OpenMP on
every core), on a bounded sample of the same rays per step.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from xdg_gb300 import dist, synth  # noqa: E402

METRIC = "ray_fire Mrays/s, tet-walk Msegs/s on 1 GB300: mixed vs FP64, 0 ID mismatches"
N_RAYS = 10_000_000
N_TRACKS = 1_000_000
MAX_SEGS = 512
WORKLOAD = "nested_spheres_8x_icosphere_L6_jitter1e-3_1e7_rays"
WALK_WORKLOAD = "tet_cube_50^3x6_kuhn_jitter0.2_1e6_tracks_exp5"
MANY_SURFACES = 256
MANY_WORKLOAD = "256_surfaces_sphere_torus_tris_10^U(3,5.7)_rays_10^U(3,6)"
TUNE_RAYS = 10_000_000      # autotuner sample of the headline: its size and distribution, its own
                            # seed (on a 1e6 sample static chunks won; on 1e7 rays the work queue
                            # does, by about 3 %)
TUNE_RAYS_MANY = 1_000_000  # autotuner sample of the many-surface rays
TUNE_TRACKS = 1_000_000     # the walk's length order pays off only on large batches
TRACE_KEYS = ("node_width", "leaf_max", "trace_occupancy", "trace_stack", "trace_node_iters",
              "trace_node_iters_fp64", "trace_flush_wait", "trace_grab", "trace_sort_min")
WALK_KEYS = ("walk_queue", "walk_flush_wait", "walk_sort_min")
CPU_SAMPLE = 4_000_000      # rays of the same workload timed on the host cores
TRANSPORT_WORKLOAD = "tet_cube_50^3x6_kuhn_jitter0.2_1e6_particles_mfp1_walk_elements_tool"
MFP = 1.0                   # tools/walk_elements.cpp: --mfp default
MAX_EVENTS = 1_000_000
TRANSPORT_CHECK = 2_000     # particles checked bit for bit against the oracle
TRANSPORT_CPU_SAMPLE = 50_000
OVERLAP_WORKLOAD = "nested_spheres_8x_icosphere_L6_overlap_check_vertices_and_edges"
OVERLAP_CPU_SAMPLE = 200_000
SURF_WORKLOAD = "nested_spheres_8x_icosphere_L6_3.7e6_sources_mfp1_ipc_graveyard_particle_sim"
SURF_PARTICLES = 10_000_000  # ray origins of the headline workload used as sources
SURF_HIST = 16
SURF_CHECK = 1_000
SURF_CPU_SAMPLE = 20_000
REF_STEP_SAMPLE = 1_000_000  # rays per step of --impl reference
CLOSEST_POINTS = 1_000_000   # closest-facet queries (the first points of the ray origins)
QUERY_CHECK = 100_000        # headline points whose point_in_volume / occluded the oracle repeats
CLOSEST_CHECK = 20_000       # of the closest queries, repeated by the oracle
BYTES_NODE = 112            # 4-wide FP32 node: 24 B boxes + 4 B child per child
BYTES_TRI32 = 40            # 36 B FP32 triangle + 4 B id
BYTES_TRI64 = 76            # 72 B FP64 triangle + 4 B id (escalations)
BYTES_IO = 68               # 48 B origin/dir + 4 B tree id in, 8 B t + 4 B surface + 4 B face out
# FP32 work of one ray (the survey's measurement convention): 110 flops per
# Plucker triangle test, 12 per box of a W-wide node (slab test)
FLOPS_TRI = 110
FLOPS_BOX = 12
BYTES_IO_ONLY = 64          # the convention's ray I/O: 48 B in, 8 B t + 4 B surface + 4 B status out
GLOBAL_TRACKS = 1_000_000    # tracks of the global track loop (XDG::segments(start, end))
GLOBAL_CHECK = 2_000         # of them repeated by the oracle's track loop
GLOBAL_WORKLOAD = "3_tet_blocks_30^3x6_jitter0.2_gaps_1e6_tracks_uniform_endpoints"
WALK_CHECK = 50_000          # C5 tracks walked by the oracle and compared bit for bit
WALK_CPU_SAMPLE = 1_000_000  # C5 tracks of the walk's CPU baseline (all of them)
FV_CHECK = 100_000           # headline points whose find_volume the oracle repeats
NOALLOC_MAX_TRACKS = 4_194_304
# Algorithmic work of one walk segment (one step of next_element +
# walk_elements, mesh_manager_interface.cpp:106-200), in FP64 operations with
# a division counted as one:
#   per step: cross(u, r) 9 (plucker.h:75), r += len * u and distance -= len 7;
#   per face tested exactly from the edge table: 3 coordinates x 11
#   (dot(u, e x lo) + dot(u x r, e)) + 14 for the hit distance (sum, 1/sum,
#   3 weights, the hit point component, its difference and quotient, u + v);
#   the all-FP64 path computes each coordinate from the vertices (23: edge,
#   cross, two dots, sum), 4 faces per step, one of which reaches the distance.
WALK_FP64_OPS_STEP = 16
WALK_FP64_OPS_FACE = 47
WALK_FP64_OPS_FP64_PATH = 16 + 4 * 69 + 14
# bytes per segment (conn 16 + adjacency 16 + 4 FP32 vertices 48 + output 12)
WALK_BYTES_SEG_MIXED = 92


def set_sizes(rays, tracks):
    global N_RAYS, N_TRACKS
    N_RAYS, N_TRACKS = int(rays), int(tracks)


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# --------------------------------------------------------------------------
# workloads
# --------------------------------------------------------------------------

def c2_rays(n, seed):
    rng = np.random.default_rng(seed)
    p = rng.uniform(-9.0, 9.0, (n, 3))
    d = synth.isotropic_dirs(rng, n)
    return np.ascontiguousarray(p), np.ascontiguousarray(d)


def c5_tracks(n, seed):
    rng = np.random.default_rng(seed)
    s = rng.uniform(0.0, 10.0, (n, 3))
    u = synth.isotropic_dirs(rng, n)
    with np.errstate(divide="ignore", invalid="ignore"):
        t1 = (0.0 - s) / u
        t2 = (10.0 - s) / u
    ex = np.where(u > 0, t2, np.where(u < 0, t1, np.inf)).min(axis=1)
    length = np.minimum(rng.exponential(5.0, n), ex)
    return np.ascontiguousarray(s), np.ascontiguousarray(u), np.ascontiguousarray(length)


# --------------------------------------------------------------------------
# clocks
# --------------------------------------------------------------------------

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            j = json.load(f)
        return float(j["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def measure_peaks(device):
    """FP64/FP32 issue rates and L2 read bandwidth of this GPU, from the
    microbenchmarks in xdg_gb300/csrc/peaks.cu (median of 5 launches)."""
    from xdg_gb300 import build as b
    lib = ctypes.CDLL(b.PEAKS_LIB)
    lib.xdgpk_measure.restype = ctypes.c_int
    lib.xdgpk_measure.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                  ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
    out = {}
    for kind, key, scale in ((0, "fp64_add_gops", 1e9), (1, "fp64_mul_gops", 1e9),
                             (2, "fp64_fma_gops", 1e9), (3, "fp32_fma_gops", 1e9),
                             (4, "l2_read_gbs", 1e9)):
        v, ms = ctypes.c_double(0.0), ctypes.c_double(0.0)
        rc = lib.xdgpk_measure(device, kind, 5, ctypes.byref(v), ctypes.byref(ms))
        if rc != 0:
            raise RuntimeError(f"peaks microbenchmark {key}: CUDA error {rc}")
        out[key] = v.value / scale
    out["how"] = ("peaks.cu: 8 independent chains per thread, SMs x 2048 threads, median of 5 "
                  "launches (CUDA events); L2: 32 MiB read 2048 times")
    return out


def profile_traffic():
    """Per-ray DRAM bytes of the dominant kernel from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "ray_fire_mixed_traffic.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)
    return None


# --------------------------------------------------------------------------
# reference arm (host cores)
# --------------------------------------------------------------------------

def run_reference(args, rank, world):
    if rank != 0:
        return 0
    from oracle import oracle as xo
    xo.build()
    cores = os.cpu_count() or 1
    model = synth.nested_spheres(8, 6, 1e-3, 7)
    trees = {v: xo.volume_tree(model, v) for v in model.volumes}
    p, d = c2_rays(REF_STEP_SAMPLE, dist.rank_seed(1234, 0))
    vols = oracle_find_volume(trees, model, p, d, cores)

    def step():
        for v in model.volumes:
            sel = np.nonzero(vols == v)[0]
            if len(sel):
                trees[v].ray_fire(p[sel], d[sel], threads=cores)

    for _ in range(args.warmup):
        step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    dt = (time.perf_counter() - t0) / args.steps
    value = REF_STEP_SAMPLE / dt / 1e6
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "Mrays/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": {"workload": WORKLOAD, "rays_per_step": REF_STEP_SAMPLE},
        "cpu_baseline": {"value": value, "unit": "Mrays/s", "cores": cores, "kind": "port",
                         "sample": f"{REF_STEP_SAMPLE} rays of the workload per step"},
        "e2e": {"value": value, "unit": "Mrays/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def oracle_find_volume(trees, model, p, d, cores):
    vols = np.full(len(p), model.implicit_complement, dtype=np.int32)
    todo = np.arange(len(p))
    for v in sorted(model.volumes):
        if v == model.implicit_complement or len(todo) == 0:
            continue
        ins = trees[v].point_in_volume(p[todo], d[todo], threads=cores).astype(bool)
        vols[todo[ins]] = v
        todo = todo[~ins]
    return vols


def oracle_queries(trees, model, p, d, vols, piv, occ, occ_dist, clo_d, clo_f, cores):
    """point_in_volume, occluded and closest of the headline workload repeated
    by the oracle on evenly spaced samples (each point in the volume it was
    queried in), compared with the mixed-precision results bit for bit.  The
    same oracle calls, timed on every host core, give each query's CPU
    baseline."""
    out = {}
    n = len(p)
    qsel = np.arange(0, n, max(1, n // QUERY_CHECK))
    csel = np.arange(0, len(clo_d), max(1, len(clo_d) // CLOSEST_CHECK))

    def per_volume(sel, fn):
        """[(indices, oracle result)] per volume, and the oracle's seconds."""
        parts, secs = [], 0.0
        for v in model.volumes:
            s = sel[vols[sel] == v]
            if len(s):
                t0 = time.perf_counter()
                res = fn(trees[v], s)
                secs += time.perf_counter() - t0
                parts.append((s, res))
        return parts, secs

    parts, secs = per_volume(qsel, lambda t, s: t.point_in_volume(p[s], d[s], threads=cores))
    out["point_in_volume"] = {
        "points": int(len(qsel)),
        "mismatches": sum(int((res != piv[s]).sum()) for s, res in parts),
        "cpu_Mpoints_s": len(qsel) / secs / 1e6}
    parts, secs = per_volume(qsel, lambda t, s: t.occluded(p[s], d[s], threads=cores))
    out["occluded"] = {
        "rays": int(len(qsel)),
        "flag_mismatches": sum(int((res[0] != occ[s]).sum()) for s, res in parts),
        "distance_mismatches": sum(int((res[1] != occ_dist[s]).sum()) for s, res in parts),
        "cpu_Mrays_s": len(qsel) / secs / 1e6}
    parts, secs = per_volume(csel, lambda t, s: t.closest(p[s], threads=cores))
    out["closest"] = {
        "points": int(len(csel)),
        "distance_mismatches": sum(int((res[0] != clo_d[s]).sum()) for s, res in parts),
        "face_mismatches": sum(int((res[1] != clo_f[s]).sum()) for s, res in parts),
        "cpu_Mpoints_s": len(csel) / secs / 1e6}
    return out


# --------------------------------------------------------------------------
# engine arm
# --------------------------------------------------------------------------

def timed(torch, fn, steps, warmup, world, stream):
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    dist.barrier(world)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    dist.barrier(world)
    ms = e0.elapsed_time(e1) / steps
    return dist.max_over_ranks(ms, world)


def bench_many_surfaces(torch, L, dev, stream, args, rank, world):
    """256 closed surfaces (alternating icospheres and tori, each its own
    volume), ~2.2e7 triangles, 10^U(3,6) rays per surface from interior
    points: ray_fire of every ray in its own volume as (a) one launch with a
    tree id per ray, (b) one launch per volume, (c) the launches of (b)
    captured once in a CUDA graph and replayed."""
    from xdg_gb300 import _lib
    from xdg_gb300.engine import EXITING, MIXED, XDG

    t0 = time.perf_counter()
    model, shapes = synth.many_surfaces(MANY_SURFACES, seed=5)
    rng = np.random.default_rng(dist.rank_seed(77, rank))
    o_h, d_h, vol_h, off = synth.many_surface_rays(shapes, rng)
    x = XDG(model, device=dev.index)
    x.prepare_raytracer()
    rti = x.rti
    lut = np.zeros(max(model.volumes) + 1, dtype=np.int32)
    for v, t in x.volume_to_surface_tree.items():
        lut[v] = t
    n = len(o_h)
    o = torch.from_numpy(o_h).to(dev)
    d = torch.from_numpy(d_h).to(dev)
    trees = torch.from_numpy(lut[vol_h]).to(dev)
    vol = torch.from_numpy(vol_h).to(dev)
    del o_h, d_h
    t_a = torch.empty(n, dtype=torch.float64, device=dev)
    s_a = torch.empty(n, dtype=torch.int32, device=dev)
    f_a = torch.empty(n, dtype=torch.int32, device=dev)
    t_b, s_b, f_b = torch.empty_like(t_a), torch.empty_like(s_a), torch.empty_like(f_a)
    log(f"[bench] many-surface setup {time.perf_counter() - t0:.1f}s, {n} rays")
    tuned = None
    if args.autotune:
        from xdg_gb300.engine import QUERY_RAY_FIRE
        sel = torch.arange(0, n, max(1, n // TUNE_RAYS_MANY), device=dev)
        t1 = time.perf_counter()
        _, tv = rti.autotune_trace(QUERY_RAY_FIRE, 0, o[sel], d[sel], precision=MIXED,
                                   ray_trees=trees[sel], reps=3)
        tuned = {"sample_rays": int(sel.numel()), "seconds": time.perf_counter() - t1,
                 "trace": {k: tv[k] for k in TRACE_KEYS}}
        log(f"[bench] many-surface autotune {tuned['seconds']:.1f}s: {tuned['trace']}")

    def one_launch():
        rc = L.xdgcu_ray_fire(rti.ctx, 0, ctypes.c_void_p(trees.data_ptr()), n,
                              ctypes.c_void_p(o.data_ptr()), ctypes.c_void_p(d.data_ptr()), None,
                              EXITING, None, None, ctypes.c_void_p(t_a.data_ptr()),
                              ctypes.c_void_p(s_a.data_ptr()), ctypes.c_void_p(f_a.data_ptr()),
                              None, MIXED, ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream))
        _lib.check(rc, rti.ctx, "ray_fire")

    def per_volume():
        sp = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
        for k in range(len(off) - 1):
            a, b = int(off[k]), int(off[k + 1])
            rc = L.xdgcu_ray_fire(rti.ctx, int(lut[k + 1]), None, b - a,
                                  ctypes.c_void_p(o.data_ptr() + 24 * a),
                                  ctypes.c_void_p(d.data_ptr() + 24 * a), None, EXITING, None, None,
                                  ctypes.c_void_p(t_b.data_ptr() + 8 * a),
                                  ctypes.c_void_p(s_b.data_ptr() + 4 * a),
                                  ctypes.c_void_p(f_b.data_ptr() + 4 * a), None, MIXED, sp)
            _lib.check(rc, rti.ctx, "ray_fire")

    steps = max(3, args.steps // 4)
    ms_one = timed(torch, one_launch, steps, args.warmup, world, stream)
    ms_per = timed(torch, per_volume, steps, args.warmup, world, stream)
    same_per = bool(torch.equal(t_a, t_b) and torch.equal(s_a, s_b) and torch.equal(f_a, f_b))
    s_b.fill_(-7)
    side = torch.cuda.Stream(dev)
    side.wait_stream(stream)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.stream(side):
        with torch.cuda.graph(g, stream=side, capture_error_mode="thread_local"):
            per_volume()
    torch.cuda.synchronize()
    ms_graph = timed(torch, g.replay, steps, args.warmup, world, stream)
    same_graph = bool(torch.equal(s_a, s_b) and torch.equal(t_a, t_b))
    own = bool(torch.equal(s_a, vol))
    total = dist.sum_over_ranks(n, world)
    return {
        "workload": MANY_WORKLOAD,
        "surfaces": MANY_SURFACES,
        "triangles": int(sum(len(s.face_ids) for s in model.surfaces)),
        "rays": n,
        "unit": "Mrays/s",
        "one_launch": total / (ms_one / 1e3) / 1e6,
        "per_volume_launches": total / (ms_per / 1e3) / 1e6,
        "per_volume_graph": total / (ms_graph / 1e3) / 1e6,
        "ms_one_launch": ms_one, "ms_per_volume": ms_per, "ms_graph": ms_graph,
        "all_rays_exit_own_surface": own,
        "per_volume_equals_one_launch": same_per,
        "graph_equals_one_launch": same_graph,
        "precision": "mixed",
        "tuning": tuned,
    }


def bench_small_configs(torch, L, dev, stream, sptr, args, rank, world):
    """The two small configurations, reported per configuration with the
    mixed path's escalation fraction and its agreement with the FP64 path
    and the oracle:
      C1 sphere in box: level-4 icosphere r 10 in a cube of half-width 20,
         1e5 rays from the ball r <= 9.9 (the ray-benchmark sampler, seed
         12345), ray_fire EXITING in the sphere's volume;
      C3 degenerate hits: level-6 icosphere r 5, 1e6 rays aimed at vertices
         (40 %), edge midpoints (40 %) and centroids (20 %) with a 10^U(-12,-6)
         jitter; every ray must hit (no lost hits)."""
    from xdg_gb300 import _lib
    from xdg_gb300.engine import FP64, MIXED, XDG
    out = {}
    cases = []
    m1 = synth.single_sphere_in_box(level=4, radius=10.0, half_width=20.0)
    o1, d1 = synth.lcg_benchmark_rays(100_000, (0.0, 0.0, 0.0), 9.9, seed=12345)
    cases.append(("C1_sphere_in_box_L4_1e5_rays", m1, o1, d1))
    v, tri = synth.icosphere(6, 5.0)
    m3 = synth.Model()
    m3.surfaces.append(synth.Surface(1, v, tri, np.arange(len(tri), dtype=np.int32), 1, 2))
    m3.volumes = [1, 2]
    m3.implicit_complement = 2
    o3, d3, _ = synth.watertight_rays(v, tri, 1_000_000, 4.99, seed=4)
    cases.append(("C3_degenerate_hits_L6_1e6_rays", m3, o3, d3))
    for name, m, o_h, d_h in cases:
        x = XDG(m, device=dev.index)
        x.prepare_raytracer()
        n = len(o_h)
        o, d = torch.from_numpy(o_h).to(dev), torch.from_numpy(d_h).to(dev)
        tree = x.volume_to_surface_tree[1]
        t = {p: torch.empty(n, dtype=torch.float64, device=dev) for p in (MIXED, FP64)}
        sf = {p: torch.empty(n, dtype=torch.int32, device=dev) for p in (MIXED, FP64)}
        fc = {p: torch.empty(n, dtype=torch.int32, device=dev) for p in (MIXED, FP64)}

        def rf(prec):
            def go():
                rc = L.xdgcu_ray_fire(x.rti.ctx, tree, None, n, ctypes.c_void_p(o.data_ptr()),
                                      ctypes.c_void_p(d.data_ptr()), None, 0, None, None,
                                      ctypes.c_void_p(t[prec].data_ptr()),
                                      ctypes.c_void_p(sf[prec].data_ptr()),
                                      ctypes.c_void_p(fc[prec].data_ptr()), None, prec, sptr)
                _lib.check(rc, x.rti.ctx, "ray_fire")
            return go

        ms = {p: timed(torch, rf(p), max(3, args.steps // 2), 3, world, stream)
              for p in (MIXED, FP64)}
        x.rti.set_counting(True)
        rf(MIXED)()
        torch.cuda.synchronize()
        cnt = x.rti.counters()
        x.rti.set_counting(False)
        rays = max(1, cnt["rays"])
        res = {
            "rays": n, "unit": "Mrays/s",
            "value": n / (ms[MIXED] / 1e3) / 1e6, "fp64_value": n / (ms[FP64] / 1e3) / 1e6,
            "escalations_per_ray": cnt["escalate"] / rays,
            "escalated_fraction_of_triangle_tests": cnt["escalate"] / max(1, cnt["prim"]),
            "id_mismatches_mixed_vs_fp64": int((sf[MIXED] != sf[FP64]).sum().item()
                                               + (fc[MIXED] != fc[FP64]).sum().item()),
            "t_mismatches_mixed_vs_fp64": int((t[MIXED] != t[FP64]).sum().item()),
            "max_rel_t_error_mixed_vs_fp64": float(((t[MIXED] - t[FP64]).abs()
                                                   / t[FP64].abs()).max().item()),
            "lost_hits": int((sf[MIXED] != 1).sum().item()),
        }
        if rank == 0 and not args.no_oracle:
            from oracle import oracle as xo
            cores = os.cpu_count() or 1
            k = min(n, 200_000)
            otree = xo.volume_tree(m, 1)
            # the trace loop alone on the host cores (tools/ray_benchmark.cpp:209-230:
            # the tree is built before the clock starts)
            tc = time.perf_counter()
            ot, os_, of = otree.ray_fire(o_h[:k], d_h[:k], threads=cores)
            dtc = time.perf_counter() - tc
            res["oracle_check"] = {"rays": k, "mismatches": int(
                (t[MIXED][:k].cpu().numpy() != ot).sum() + (fc[MIXED][:k].cpu().numpy() != of).sum()
                + (sf[MIXED][:k].cpu().numpy() != os_).sum())}
            res["cpu_baseline"] = {"value": k / dtc / 1e6, "unit": "Mrays/s", "cores": cores,
                                   "kind": "port",
                                   "sample": f"first {k} rays, FP64 ray_fire, BVH, OpenMP, "
                                             "trace loop only"}
        out[name] = res
    return out


def bench_overlap(torch, x, model, args, rank):
    """The overlap_check tool (tools/overlap.cpp:62-191) on the nested-sphere
    model through XDG.check_overlaps: every face vertex moved +/-1e-9 along
    normalize(0.1, 0.1, 0.1) and tested in all 9 volumes (3.9e6 points,
    3.5e7 point_in_volume queries), then a ray along every face edge in the 7
    volumes that are not its surface's parents (1.4e7 ray_fire queries).
    Timed end to end from host arrays (host-side batching included), best of
    three."""
    from xdg_gb300.engine import FP64, MIXED
    n_vert = 3 * sum(len(s.face_ids) for s in model.surfaces)
    nv = len(model.volumes)
    piv_q = 2 * n_vert * nv
    edge_q = sum(3 * len(s.face_ids) * (nv - 2) for s in model.surfaces)
    out = {"workload": OVERLAP_WORKLOAD, "unit": "Mqueries/s",
           "point_in_volume_queries": piv_q, "edge_ray_queries": edge_q}
    for name, prec in (("mixed", MIXED), ("fp64", FP64)):
        best = None
        for _ in range(3):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            found = x.check_overlaps(check_edges=True, precision=prec)
            torch.cuda.synchronize()
            dt = time.perf_counter() - t0
            best = dt if best is None else min(best, dt)
        out[f"seconds_{name}"] = best
        out["value" if name == "mixed" else "fp64_value"] = (piv_q + edge_q) / best / 1e6
        out[f"overlaps_found_{name}"] = len(found)
    if rank == 0 and not args.no_oracle:
        from oracle import oracle as xo
        cores = os.cpu_count() or 1
        verts = np.concatenate([s.tri_xyz().reshape(-1, 3) for s in model.surfaces])
        k = min(OVERLAP_CPU_SAMPLE, len(verts))
        dd = np.array([0.1, 0.1, 0.1])
        dd = dd / np.sqrt(dd[0] * dd[0] + dd[1] * dd[1] + dd[2] * dd[2])
        pts = verts[:k] + dd * 1e-9
        dirs = np.tile(dd, (k, 1))
        trees = [xo.volume_tree(model, v) for v in model.volumes]
        tc = time.perf_counter()
        inside = np.stack([t.point_in_volume(pts, dirs, threads=cores) for t in trees], 1)
        dtc = time.perf_counter() - tc
        got = x.rti.point_in_volumes(pts, [x.volume_to_surface_tree[v] for v in model.volumes],
                                     dirs)
        out["oracle_check"] = {"points": k, "volumes": nv,
                               "mismatches": int((got != inside).any(1).sum())}
        out["cpu_baseline"] = {"value": k * nv / dtc / 1e6, "unit": "Mqueries/s",
                               "cores": cores, "kind": "port",
                               "sample": f"vertex stage, first {k} vertices x {nv} volumes, "
                                         "FP64, BVH, OpenMP"}
    return out


def bench_surface_transport(torch, L, x, model, dev, stream, sptr, p, d, trees_h, args, rank,
                            world):
    """The particle_sim tool loop (tools/particle_sim.h:128-141) on the
    nested-sphere model: the ray origins of the headline workload that lie
    inside the spheres (3.7e6 of the 1e7) are particle sources (their volume from
    find_volume, the ray's direction), mean free path 1, transmission on
    every surface and the implicit complement as graveyard (the tool's
    --ipc-graveyard): each particle flies (ray_fire in its volume, history
    excluded), collides or crosses into the next shell until it leaves the
    outer sphere, all in one xdgcu_transport_surfaces launch per step."""
    from xdg_gb300 import _lib
    from xdg_gb300.engine import FP64, MIXED
    grave = x.volume_to_surface_tree[model.implicit_complement]
    sel_h = np.nonzero(trees_h[:SURF_PARTICLES] != grave)[0]
    n = len(sel_h)
    sel = torch.from_numpy(sel_h).to(dev)
    t0 = torch.from_numpy(trees_h[sel_h].astype(np.int32)).to(dev)
    p0, d0 = p[sel].contiguous(), d[sel].contiguous()
    seeds_h = x.rti.seed_streams(dist.rank_seed(4048, rank), n)
    s0 = torch.from_numpy(seeds_h.view(np.int64)).to(dev)
    T = {"tree": torch.empty_like(t0), "pos": torch.empty_like(p0), "dir": torch.empty_like(d0),
         "rng": torch.empty_like(s0),
         "hist": torch.zeros((n, SURF_HIST), dtype=torch.int32, device=dev),
         "hc": torch.empty(n, dtype=torch.int32, device=dev),
         "dist": torch.empty(n, dtype=torch.float64, device=dev),
         "ev": torch.empty(n, dtype=torch.int32, device=dev),
         "st": torch.empty(n, dtype=torch.int32, device=dev)}

    def step(prec):
        def go():
            T["tree"].copy_(t0)
            T["pos"].copy_(p0)
            T["dir"].copy_(d0)
            T["rng"].copy_(s0)
            T["hc"].zero_()
            T["dist"].zero_()
            T["ev"].zero_()
            a = [ctypes.c_void_p(T[k].data_ptr()) for k in ("tree", "pos", "dir", "rng")]
            rc = L.xdgcu_transport_surfaces(
                x.rti.ctx, n, *a, MFP, MAX_EVENTS, grave, SURF_HIST,
                ctypes.c_void_p(T["hist"].data_ptr()), ctypes.c_void_p(T["hc"].data_ptr()),
                ctypes.c_void_p(T["dist"].data_ptr()), ctypes.c_void_p(T["ev"].data_ptr()), None,
                ctypes.c_void_p(T["st"].data_ptr()), prec, sptr)
            _lib.check(rc, x.rti.ctx, "transport_surfaces")
        return go

    ms = timed(torch, step(MIXED), max(3, args.steps // 4), args.warmup, world, stream)
    events = int(T["ev"].sum().item())
    # work per event (untimed counting run): nodes, triangles, FP64 escalations
    x.rti.set_counting(True)
    step(MIXED)()
    torch.cuda.synchronize()
    cnt = x.rti.counters()
    x.rti.set_counting(False)
    per_event = {k: cnt[k] / max(1, events) for k in ("node", "prim", "escalate")}
    bad = int((T["st"] != 0).sum().item())
    keys = ("tree", "pos", "dir", "rng", "dist", "ev")
    mixed_state = {k: T[k].clone() for k in keys}
    ms64 = timed(torch, step(FP64), 3, 1, world, stream)
    mism = sum(int((mixed_state[k] != T[k]).reshape(n, -1).any(1).sum().item()) for k in keys)
    total = dist.sum_over_ranks(events, world)
    out = {
        "workload": SURF_WORKLOAD, "unit": "Mevents/s",
        "value": total / (ms / 1e3) / 1e6, "fp64_value": total / (ms64 / 1e3) / 1e6,
        "ms_per_step": ms, "fp64_ms_per_step": ms64, "particles": n, "events": events,
        "events_per_particle": events / max(1, n), "speedup_mixed_vs_fp64": ms64 / ms,
        "particles_differing_mixed_vs_fp64": mism, "particles_with_status": bad,
        "step": "reset sources + one xdgcu_transport_surfaces launch (all events)",
        "per_event": per_event,
    }
    if rank == 0 and not args.no_oracle:
        from oracle import oracle as xo
        sim = xo.SurfaceTransport(model, x.volume_to_surface_tree)
        k = min(SURF_CHECK, n)
        o = sim.run(t0[:k].cpu().numpy(), p0[:k].cpu().numpy(), d0[:k].cpu().numpy(),
                    seeds_h[:k], MFP, MAX_EVENTS, graveyard_tree=grave)
        got = [mixed_state[kk][:k].cpu().numpy() for kk in keys]
        got[3] = got[3].view(np.uint64)
        out["oracle_check"] = {"particles": k, "mismatches": int(sum(
            int((np.asarray(a) != np.asarray(b)).reshape(k, -1).any(1).sum())
            for a, b in zip(got, o[:6])))}
        kc = min(SURF_CPU_SAMPLE, n)
        cores = os.cpu_count() or 1
        tc = time.perf_counter()
        oc = sim.run(t0[:kc].cpu().numpy(), p0[:kc].cpu().numpy(), d0[:kc].cpu().numpy(),
                     seeds_h[:kc], MFP, MAX_EVENTS, graveyard_tree=grave, threads=cores)
        dtc = time.perf_counter() - tc
        out["cpu_baseline"] = {"value": float(oc[5].sum()) / dtc / 1e6, "unit": "Mevents/s",
                               "cores": cores, "kind": "port",
                               "sample": f"first {kc} particles, FP64 particle_sim loop, BVH, "
                                         "OpenMP"}
    return out


def bench_global_segments(torch, L, dev, stream, sptr, args, rank, world):
    """XDG::segments(start, end) (xdg.cpp:142-198) over three jittered meshed
    blocks (30^3 x 6 tets each, 486,000 tets) with gaps of implicit
    complement between them: GLOBAL_TRACKS tracks between uniform points of
    the box around them, every round of every track in one
    xdgcu_segments_global call (device arrays), both precisions; the oracle's
    track loop repeats a sample bit for bit."""
    from xdg_gb300 import _lib
    from xdg_gb300.engine import FP64, MIXED, XDG
    t0 = time.perf_counter()
    m = synth.tet_blocks([((0.0, 0.0, 0.0), 30, 10.0), ((12.0, 0.0, 0.0), 30, 10.0),
                          ((24.0, 0.0, 0.0), 30, 10.0)], jitter=0.2, seed=17)
    x = XDG(m, device=dev.index)
    x.prepare_raytracer()
    rng = np.random.default_rng(dist.rank_seed(777, rank))
    lo, hi = np.array([-3.0, -1.0, -1.0]), np.array([37.0, 11.0, 11.0])
    a_h = rng.uniform(lo, hi, (GLOBAL_TRACKS, 3))
    b_h = rng.uniform(lo, hi, (GLOBAL_TRACKS, 3))
    a, b = torch.from_numpy(a_h).to(dev), torch.from_numpy(b_h).to(dev)
    ipc = x.volume_to_surface_tree[m.implicit_complement]
    gt = x.rti.global_element_tree
    n = GLOBAL_TRACKS
    off = torch.empty(n + 1, dtype=torch.int64, device=dev)
    st = torch.empty(n, dtype=torch.int32, device=dev)
    se0, sl0, off0, _ = x.rti.segments_global(ipc, gt, a, b, 1, precision=MIXED)
    torch.cuda.synchronize()
    cap = int(off0[-1].item())
    se = torch.empty(cap, dtype=torch.int32, device=dev)
    sl = torch.empty(cap, dtype=torch.float64, device=dev)
    log(f"[bench] global segments setup {time.perf_counter() - t0:.1f}s, {len(m.tets.conn)} tets")

    def run(prec, e=se, ln=sl, o=off, s_=st):
        def go():
            rc = L.xdgcu_segments_global(x.rti.ctx, ipc, gt, n, ctypes.c_void_p(a.data_ptr()),
                                         ctypes.c_void_p(b.data_ptr()), 4096, 10_000, cap,
                                         ctypes.c_void_p(e.data_ptr()), ctypes.c_void_p(ln.data_ptr()),
                                         ctypes.c_void_p(o.data_ptr()), ctypes.c_void_p(s_.data_ptr()),
                                         prec, sptr)
            _lib.check(rc, x.rti.ctx, "segments_global")
        return go

    ms = timed(torch, run(MIXED), max(3, args.steps // 4), 2, world, stream)
    ref = (se.clone(), sl.clone(), off.clone())
    se64, sl64 = torch.empty_like(se), torch.empty_like(sl)
    off64, st64 = torch.empty_like(off), torch.empty_like(st)
    ms64 = timed(torch, run(FP64, se64, sl64, off64, st64), 3, 1, world, stream)
    same = bool(torch.equal(off64, ref[2]) and torch.equal(se64, ref[0]) and torch.equal(sl64, ref[1]))
    segs = int(ref[2][-1].item())
    out = {"workload": GLOBAL_WORKLOAD, "tracks": n, "tets": int(len(m.tets.conn)),
           "segments": segs, "unit": "Msegs/s",
           "value": dist.sum_over_ranks(segs, world) / (ms / 1e3) / 1e6,
           "fp64_value": dist.sum_over_ranks(segs, world) / (ms64 / 1e3) / 1e6,
           "ms_per_step": ms, "fp64_ms_per_step": ms64, "mixed_equals_fp64": same,
           "tracks_with_status": int((st != 0).sum().item()),
           "step": "one xdgcu_segments_global call (all rounds: find_element, implicit-complement "
                   "ray_fire + boundary-face re-entry, single-pass walk resumed across rounds)"}
    if rank == 0 and not args.no_oracle:
        from oracle import oracle as xo
        xo.build()
        g = xo.GlobalTracker(m)
        ksel = np.arange(0, n, max(1, n // GLOBAL_CHECK))
        oh = ref[2].cpu().numpy()
        eh, lh = ref[0].cpu().numpy(), ref[1].cpu().numpy()
        mism = 0
        for i in ksel:
            oe, ol = g.segments(a_h[i], b_h[i])
            e_i, l_i = eh[oh[i]:oh[i + 1]], lh[oh[i]:oh[i + 1]]
            mism += int(not (np.array_equal(e_i, oe) and np.array_equal(l_i, ol)))
        out["oracle_check"] = {"tracks": int(len(ksel)), "tracks_differing": mism}
    return out


def bench_transport(torch, L, wr, dev, stream, sptr, ws, wu, we_idx, tm, args, rank, world):
    """The walk_elements tool loop (tools/walk_elements.h:60-96) on the
    750,000-tet cube: the walk's 1e6 track starts as particle sources,
    isotropic directions, mean free path 1 (the tool's default), every event
    of every particle until it leaves the mesh (a convex mesh: no re-entry)
    in one xdgcu_transport_elements launch per step.  A step also resets the
    particle state from the sources (device copies, ~60 MB)."""
    from xdg_gb300 import _lib
    from xdg_gb300.engine import FP64, MIXED
    n = int(we_idx.numel())
    seeds_h = wr.rti.seed_streams(dist.rank_seed(2024, rank), n)
    s0 = torch.from_numpy(seeds_h.view(np.int64)).to(dev)
    e = torch.empty_like(we_idx)
    r = torch.empty_like(ws)
    u = torch.empty_like(wu)
    s = torch.empty_like(s0)
    d = torch.empty(n, dtype=torch.float64, device=dev)
    ev = torch.empty(n, dtype=torch.int32, device=dev)
    st = torch.empty(n, dtype=torch.int32, device=dev)

    def step(prec):
        def go():
            e.copy_(we_idx)
            r.copy_(ws)
            u.copy_(wu)
            s.copy_(s0)
            d.zero_()
            ev.zero_()
            rc = L.xdgcu_transport_elements(
                wr.rti.ctx, n, ctypes.c_void_p(e.data_ptr()), ctypes.c_void_p(r.data_ptr()),
                ctypes.c_void_p(u.data_ptr()), ctypes.c_void_p(s.data_ptr()), MFP, MAX_EVENTS,
                ctypes.c_void_p(d.data_ptr()), ctypes.c_void_p(ev.data_ptr()), None,
                ctypes.c_void_p(st.data_ptr()), prec, sptr)
            _lib.check(rc, wr.rti.ctx, "transport_elements")
        return go

    ms = timed(torch, step(MIXED), max(3, args.steps // 2), args.warmup, world, stream)
    events = int(ev.sum().item())
    bad = int((st != 0).sum().item())
    mixed_state = [x.clone() for x in (e, r, u, s, d, ev)]
    ms64 = timed(torch, step(FP64), 3, 1, world, stream)
    mism = sum(int((a != b).reshape(n, -1).any(1).sum().item())
               for a, b in zip(mixed_state, (e, r, u, s, d, ev)))
    total = dist.sum_over_ranks(events, world)
    out = {
        "workload": TRANSPORT_WORKLOAD, "unit": "Mevents/s",
        "value": total / (ms / 1e3) / 1e6, "fp64_value": total / (ms64 / 1e3) / 1e6,
        "ms_per_step": ms, "fp64_ms_per_step": ms64, "particles": n, "events": events,
        "events_per_particle": events / n, "speedup_mixed_vs_fp64": ms64 / ms,
        "particles_differing_mixed_vs_fp64": mism, "particles_with_status": bad,
        "step": "reset sources + one xdgcu_transport_elements launch (all events)",
    }
    if rank == 0 and not args.no_oracle:
        from oracle import oracle as xo
        walker = xo.TetWalker(tm.vertices, tm.conn, tm.adj, tm.face_table)
        k = min(TRANSPORT_CHECK, n)
        o = walker.transport(we_idx[:k].cpu().numpy(), ws[:k].cpu().numpy(),
                             wu[:k].cpu().numpy(), seeds_h[:k], MFP, MAX_EVENTS)
        got = [x[:k].cpu().numpy() for x in mixed_state]
        got[3] = got[3].view(np.uint64)
        out["oracle_check"] = {"particles": k, "mismatches": int(sum(
            int((np.asarray(a) != np.asarray(b)).reshape(k, -1).any(1).sum())
            for a, b in zip(got, o[:6])))}
        # CPU baseline: the oracle's particle loop on every host core
        kc = min(TRANSPORT_CPU_SAMPLE, n)
        cores = os.cpu_count() or 1
        tc = time.perf_counter()
        oc = walker.transport(we_idx[:kc].cpu().numpy(), ws[:kc].cpu().numpy(),
                              wu[:kc].cpu().numpy(), seeds_h[:kc], MFP, MAX_EVENTS,
                              threads=cores)
        dtc = time.perf_counter() - tc
        out["cpu_baseline"] = {"value": float(oc[5].sum()) / dtc / 1e6, "unit": "Mevents/s",
                               "cores": cores, "kind": "port",
                               "sample": f"first {kc} particles, FP64 particle loop, OpenMP"}
    return out


def run_engine(args, rank, world, local):
    import torch

    from xdg_gb300 import _lib
    from xdg_gb300.engine import FP64, MIXED, XDG

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream(dev)
    sptr = ctypes.c_void_p(stream.cuda_stream)
    L = _lib.load()
    pclk = ClockSampler(local)
    pclk.start()
    peaks = measure_peaks(local)
    peaks["clocks"] = pclk.stop()
    log(f"[bench] peaks {peaks}")

    # ---- C2: nested spheres -------------------------------------------
    t0 = time.perf_counter()
    model = synth.nested_spheres(8, 6, 1e-3, 7)
    x = XDG(model, device=local)
    x.prepare_raytracer()
    rti = x.rti
    p_h, d_h = c2_rays(N_RAYS, dist.rank_seed(1234, rank))
    vols_h = x.find_volume(p_h, d_h, precision=MIXED)  # volume of each ray origin
    lut = np.zeros(max(model.volumes) + 1, dtype=np.int32)
    for v, t in x.volume_to_surface_tree.items():
        lut[v] = t
    trees_h = lut[vols_h]
    p = torch.from_numpy(p_h).to(dev)
    d = torch.from_numpy(d_h).to(dev)
    trees = torch.from_numpy(trees_h).to(dev)
    t_out = torch.empty(N_RAYS, dtype=torch.float64, device=dev)
    s_out = torch.empty(N_RAYS, dtype=torch.int32, device=dev)
    f_out = torch.empty(N_RAYS, dtype=torch.int32, device=dev)
    log(f"[bench] C2 setup {time.perf_counter() - t0:.1f}s, "
        f"{sum(len(s.face_ids) for s in model.surfaces)} triangles")

    # ---- autotuner: launch settings picked on a separate sample ----------
    tuning = {"autotuned": False}
    if args.autotune:
        from xdg_gb300.engine import QUERY_RAY_FIRE
        ps_h, ds_h = c2_rays(min(TUNE_RAYS, N_RAYS), dist.rank_seed(999, rank))
        ts = torch.from_numpy(lut[x.find_volume(ps_h, ds_h, precision=MIXED)]).to(dev)
        ps, ds = torch.from_numpy(ps_h).to(dev), torch.from_numpy(ds_h).to(dev)
        t1 = time.perf_counter()
        ms_s, tuned = rti.autotune_trace(QUERY_RAY_FIRE, 0, ps, ds, precision=MIXED, ray_trees=ts,
                                         reps=3)
        tuning = {"autotuned": True, "trace_sample_rays": len(ps_h),
                  "trace_seconds": time.perf_counter() - t1, "trace_sample_ms": ms_s,
                  "trace": {k: tuned[k] for k in TRACE_KEYS}}
        del ps, ds, ts
        log(f"[bench] autotune trace {tuning['trace_seconds']:.1f}s: {tuning['trace']}")

    def rf(prec, t=t_out, s=s_out, f=f_out):
        def go():
            rc = L.xdgcu_ray_fire(rti.ctx, 0, ctypes.c_void_p(trees.data_ptr()), N_RAYS,
                                  ctypes.c_void_p(p.data_ptr()), ctypes.c_void_p(d.data_ptr()), None,
                                  0, None, None, ctypes.c_void_p(t.data_ptr()),
                                  ctypes.c_void_p(s.data_ptr()), ctypes.c_void_p(f.data_ptr()),
                                  None, prec, sptr)
            _lib.check(rc, rti.ctx, "ray_fire")
        return go

    clocks = ClockSampler(local)
    clocks.start()
    ms_mixed = timed(torch, rf(MIXED), args.steps, args.warmup, world, stream)
    # kernels of one timed step: the traversal, plus the order's key kernel and
    # radix-sort passes when the coherent order is on (it is off unless tuned on)
    launches_per_step = 1 if rti.get_tuning("trace_sort_min") in (0,) or \
        N_RAYS < rti.get_tuning("trace_sort_min") else 6
    clk = clocks.stop()
    t_mixed, s_mixed, f_mixed = t_out.clone(), s_out.clone(), f_out.clone()
    # the same mixed launch with the triangles' FP64 terms computed from the
    # vertices instead of read from the tree
    rti.set_tuning("trace_edge_table", 0)
    ms_mixed_noedge = timed(torch, rf(MIXED), max(3, args.steps // 4), 1, world, stream)
    rti.set_tuning("trace_edge_table", 1)
    edge_table_same = bool(torch.equal(t_out, t_mixed) and torch.equal(s_out, s_mixed)
                           and torch.equal(f_out, f_mixed))
    ms_fp64 = timed(torch, rf(FP64), max(3, args.steps // 4), max(1, args.warmup // 2), world,
                    stream)
    id_mism = int((s_out != s_mixed).sum().item()) + int((f_out != f_mixed).sum().item())
    t_mism = int((t_out != t_mixed).sum().item())
    hitm = s_mixed >= 0
    max_rel_t = float(((t_mixed[hitm] - t_out[hitm]).abs() / t_out[hitm].abs()).max().item()) \
        if bool(hitm.any()) else 0.0
    hit_frac = float((s_mixed >= 0).float().mean().item())

    # ---- e2e through the C ABI with pinned host buffers ------------------
    # (measured right after the device timing, before the host cores run the
    # oracle legs)
    org_h = torch.empty((N_RAYS, 3), dtype=torch.float64, pin_memory=True)
    dir_h = torch.empty((N_RAYS, 3), dtype=torch.float64, pin_memory=True)
    tr_h = torch.empty(N_RAYS, dtype=torch.int32, pin_memory=True)
    org_h.copy_(torch.from_numpy(p_h))
    dir_h.copy_(torch.from_numpy(d_h))
    tr_h.copy_(torch.from_numpy(trees_h))
    to_h = torch.empty(N_RAYS, dtype=torch.float64, pin_memory=True)
    so_h = torch.empty(N_RAYS, dtype=torch.int32, pin_memory=True)
    fo_h = torch.empty(N_RAYS, dtype=torch.int32, pin_memory=True)

    def e2e_call(bufs):
        tr, org, dr, to, so, fo = (ctypes.c_void_p(b.data_ptr()) if hasattr(b, "data_ptr")
                                   else b.ctypes.data_as(ctypes.c_void_p) for b in bufs)
        rc = L.xdgcu_ray_fire(rti.ctx, 0, tr, N_RAYS, org, dr, None, 0, None, None, to, so, fo,
                              None, MIXED, None)
        _lib.check(rc, rti.ctx, "ray_fire (host buffers)")

    def e2e_ms(bufs, host_direct):
        # host_direct 0: staged copies in chunks; 1: page-locked arrays read
        # and written in place by the kernel; 2: pageable arrays in place too;
        # 3: page-locked arrays of large calls staged in overlapping chunks;
        # 4: large calls' outputs staged; 5 (the default): 2, 3 or 4, chosen
        # by timing six of the first nine large calls, warm-up calls here
        old_hd = rti.get_tuning("host_direct")
        rti.set_tuning("host_direct", host_direct)
        for _ in range(2 + (9 if host_direct == 5 else 0)):
            e2e_call(bufs)
        torch.cuda.synchronize()
        dist.barrier(world)
        te = time.perf_counter()
        for _ in range(e2e_steps):
            e2e_call(bufs)
        torch.cuda.synchronize()
        choice = rti.get_tuning("host_direct_choice")
        rti.set_tuning("host_direct", old_hd)
        return dist.max_over_ranks((time.perf_counter() - te) / e2e_steps * 1e3, world), choice

    # one call is ~7.5 ms: 20 or more keep a single slow call from moving the
    # figure by more than a few tenths of a percent
    e2e_steps = max(20, args.steps)
    hd_default = rti.get_tuning("host_direct")
    pinned = (tr_h, org_h, dir_h, to_h, so_h, fo_h)
    # the explicit policies first, then the default (a fresh automatic
    # choice): the first host-array measurement after the device timings ran
    # up to 9 % slow in this process (1243 against 1357 Mrays/s for the same
    # policy), which a probe of the calls alone did not show
    ms_e2e_staged, _ = e2e_ms(pinned, 3)
    e2e_ok = bool(np.array_equal(so_h.numpy(), s_mixed.cpu().numpy()))
    ms_e2e_out_staged, _ = e2e_ms(pinned, 4)  # inputs read in place, outputs staged
    e2e_ok = e2e_ok and bool(np.array_equal(so_h.numpy(), s_mixed.cpu().numpy()))
    ms_e2e_in_place, _ = e2e_ms(pinned, 2)
    e2e_ok = e2e_ok and bool(np.array_equal(so_h.numpy(), s_mixed.cpu().numpy()))
    ms_e2e, hd_choice = e2e_ms(pinned, hd_default)
    e2e_ok = e2e_ok and bool(np.array_equal(so_h.numpy(), s_mixed.cpu().numpy()))
    policy = {
        0: "page-locked host arrays staged through device memory in overlapping chunks",
        2: "page-locked host arrays read and written in place by the kernel over the host link",
        3: "page-locked host arrays staged through device memory in overlapping chunks",
        4: "page-locked inputs read in place, outputs staged",
    }
    e2e_transfer = (f"the library's default (host_direct={hd_default}"
                    + (f", which timed its first large calls and chose {hd_choice}" if hd_default == 5
                       else "") + "): " + policy.get(hd_choice if hd_default == 5 else hd_default,
                                                     "see host_direct"))
    del org_h, dir_h, tr_h, to_h, so_h, fo_h
    # the same call on pageable NumPy arrays
    pg = (np.ascontiguousarray(trees_h), np.ascontiguousarray(p_h), np.ascontiguousarray(d_h),
          np.empty(N_RAYS), np.empty(N_RAYS, np.int32), np.empty(N_RAYS, np.int32))
    ms_e2e_pageable, _ = e2e_ms(pg, 0)  # pageable arrays staged
    e2e_ok = e2e_ok and bool(np.array_equal(pg[4], s_mixed.cpu().numpy()))
    pageable_direct = bool(rti.get_tuning("pageable_direct"))
    ms_e2e_pageable_direct = e2e_ms(pg, 3)[0] if pageable_direct else None
    e2e_ok = e2e_ok and bool(np.array_equal(pg[4], s_mixed.cpu().numpy()))
    del pg


    # point_in_volume of the same points in their own volume (all must be inside)
    piv_out = torch.empty(N_RAYS, dtype=torch.int32, device=dev)

    def piv(prec):
        def go():
            rc = L.xdgcu_point_in_volume(rti.ctx, 0, ctypes.c_void_p(trees.data_ptr()), N_RAYS,
                                         ctypes.c_void_p(p.data_ptr()), ctypes.c_void_p(d.data_ptr()),
                                         None, None, ctypes.c_void_p(piv_out.data_ptr()), None,
                                         prec, sptr)
            _lib.check(rc, rti.ctx, "point_in_volume")
        return go

    ms_piv = timed(torch, piv(MIXED), max(3, args.steps // 2), 2, world, stream)
    ipc = model.implicit_complement
    not_ipc = torch.from_numpy(vols_h != ipc).to(dev)
    piv_inside_frac = float(piv_out[not_ipc].float().mean().item()) if not_ipc.any() else 1.0
    piv_h = piv_out.cpu().numpy()
    ms_piv64 = timed(torch, piv(FP64), 3, 1, world, stream)
    piv_same = bool(np.array_equal(piv_out.cpu().numpy(), piv_h))

    # occluded (any hit, embree/ray_tracer.cpp:347-370) of the same rays, and
    # closest (the nearest facet, :328-345) of the first CLOSEST_POINTS points
    occ_out = torch.empty(N_RAYS, dtype=torch.int32, device=dev)
    occ_dist = torch.empty(N_RAYS, dtype=torch.float64, device=dev)

    def occ(prec):
        def go():
            rc = L.xdgcu_occluded(rti.ctx, 0, ctypes.c_void_p(trees.data_ptr()), N_RAYS,
                                  ctypes.c_void_p(p.data_ptr()), ctypes.c_void_p(d.data_ptr()),
                                  ctypes.c_void_p(occ_out.data_ptr()),
                                  ctypes.c_void_p(occ_dist.data_ptr()), None, prec, sptr)
            _lib.check(rc, rti.ctx, "occluded")
        return go

    ms_occ = timed(torch, occ(MIXED), max(3, args.steps // 4), 2, world, stream)
    occ_mixed = occ_out.clone()
    occ_h, occ_dist_h = occ_out.cpu().numpy(), occ_dist.cpu().numpy()
    ms_occ64 = timed(torch, occ(FP64), 3, 1, world, stream)
    occ_same = bool(torch.equal(occ_out, occ_mixed))
    del occ_dist
    n_clo = min(N_RAYS, CLOSEST_POINTS)
    clo_d = torch.empty(n_clo, dtype=torch.float64, device=dev)
    clo_f = torch.empty(n_clo, dtype=torch.int32, device=dev)

    def clo(prec):
        def go():
            rc = L.xdgcu_closest(rti.ctx, 0, ctypes.c_void_p(trees.data_ptr()), n_clo,
                                 ctypes.c_void_p(p.data_ptr()), ctypes.c_void_p(clo_d.data_ptr()),
                                 ctypes.c_void_p(clo_f.data_ptr()), None, prec, sptr)
            _lib.check(rc, rti.ctx, "closest")
        return go

    ms_clo = timed(torch, clo(MIXED), 3, 2, world, stream)
    clo_mixed = (clo_d.clone(), clo_f.clone())
    clo_d_h, clo_f_h = clo_d.cpu().numpy(), clo_f.cpu().numpy()
    ms_clo64 = timed(torch, clo(FP64), 3, 1, world, stream)
    clo_same = bool(torch.equal(clo_d, clo_mixed[0]) and torch.equal(clo_f, clo_mixed[1]))
    rti.set_tuning("closest_bound", 0)
    ms_clo_nb = timed(torch, clo(MIXED), 3, 1, world, stream)
    rti.set_tuning("closest_bound", 1)
    clo_same = clo_same and bool(torch.equal(clo_d, clo_mixed[0]) and torch.equal(clo_f, clo_mixed[1]))
    # every point searched by one lane to the end (no warp takes over)
    clo_budget = rti.get_tuning("closest_step_budget")
    rti.set_tuning("closest_step_budget", 0)
    ms_clo_lane = timed(torch, clo(MIXED), 3, 1, world, stream)
    rti.set_tuning("closest_step_budget", clo_budget)
    clo_same = clo_same and bool(torch.equal(clo_d, clo_mixed[0]) and torch.equal(clo_f, clo_mixed[1]))
    # the points in the caller's order instead of the Morton order
    clo_sort = rti.get_tuning("closest_sort_min")
    rti.set_tuning("closest_sort_min", 0)
    ms_clo_unsorted = timed(torch, clo(MIXED), 3, 1, world, stream)
    rti.set_tuning("closest_sort_min", clo_sort)
    clo_same = clo_same and bool(torch.equal(clo_d, clo_mixed[0]) and torch.equal(clo_f, clo_mixed[1]))
    del occ_mixed, clo_mixed

    # find_volume of the same points: one fused launch vs one launch per volume
    fv = torch.empty(N_RAYS, dtype=torch.int32, device=dev)
    fv_vols = [v for v in sorted(x.volume_to_surface_tree) if v != ipc]

    def fv_fused():
        rc = L.xdgcu_find_volume(rti.ctx, N_RAYS, ctypes.c_void_p(p.data_ptr()),
                                 ctypes.c_void_p(d.data_ptr()), ctypes.c_void_p(fv.data_ptr()),
                                 None, MIXED, sptr)
        _lib.check(rc, rti.ctx, "find_volume")

    fv_loop = torch.empty(N_RAYS, dtype=torch.int32, device=dev)

    def fv_per_volume():
        fv_loop.fill_(ipc)
        todo = torch.arange(N_RAYS, device=dev)
        for v in fv_vols:
            if todo.numel() == 0:
                break
            pin = rti.point_in_volume(x.volume_to_surface_tree[v], p[todo], d[todo],
                                      precision=MIXED).bool()
            fv_loop[todo[pin]] = v
            todo = todo[~pin]

    ms_fv = timed(torch, fv_fused, max(3, args.steps // 4), 2, world, stream)
    ms_fv_loop = timed(torch, fv_per_volume, 3, 1, world, stream)
    fv_same = bool(torch.equal(fv, fv_loop))
    fv_host_same = bool(np.array_equal(fv.cpu().numpy(), vols_h))

    # particle_sim loop on the same model
    surface_transport = bench_surface_transport(torch, L, x, model, dev, stream, sptr, p, d,
                                                trees_h, args, rank, world)

    # the small configurations, per configuration
    small_configs = bench_small_configs(torch, L, dev, stream, sptr, args, rank, world)

    # overlap_check tool on the same model (vertex and edge stages)
    overlap = bench_overlap(torch, x, model, args, rank)

    # algorithmic work counters (untimed run)
    rti.set_counting(True)
    rf(MIXED)()
    torch.cuda.synchronize()
    cnt = rti.counters()
    rti.set_counting(False)
    rays = max(1, cnt["rays"])
    per_ray = {k: cnt[k] / rays for k in ("node", "prim", "escalate")}
    bytes_per_ray = (BYTES_IO + BYTES_NODE * per_ray["node"] + BYTES_TRI32 * per_ray["prim"]
                     + BYTES_TRI64 * per_ray["escalate"])

    # oracle agreement on a sample (rank 0)
    oracle_mism = None
    fv_oracle = None
    query_oracle = {}
    cpu_baseline = None
    if rank == 0 and not args.no_oracle:
        from oracle import oracle as xo
        xo.build()
        cores = os.cpu_count() or 1
        t1 = time.perf_counter()
        otrees = {v: xo.volume_tree(model, v) for v in model.volumes}
        sample = np.arange(0, N_RAYS, max(1, N_RAYS // 100_000))
        th, sh = t_mixed.cpu().numpy(), s_mixed.cpu().numpy()
        mism = 0
        for v in model.volumes:
            sel = sample[vols_h[sample] == v]
            if len(sel):
                ot, os_, of = otrees[v].ray_fire(p_h[sel], d_h[sel], threads=cores)
                mism += int((ot != th[sel]).sum() + (os_ != sh[sel]).sum())
        oracle_mism = {"rays": int(len(sample)), "mismatches": mism}
        # find_volume of FV_CHECK of the headline points: the volume every
        # ray above was fired in
        fsel = np.arange(0, N_RAYS, max(1, N_RAYS // FV_CHECK))
        ovols = oracle_find_volume(otrees, model, p_h[fsel], d_h[fsel], cores)
        fv_h = fv.cpu().numpy()[fsel]
        fv_oracle = {"points": int(len(fsel)), "mismatches": int((ovols != fv_h).sum()),
                     "host_path_mismatches": int((ovols != vols_h[fsel]).sum()),
                     "volumes_seen": int(len(np.unique(ovols)))}
        query_oracle = oracle_queries(otrees, model, p_h, d_h, vols_h, piv_h, occ_h, occ_dist_h,
                                      clo_d_h, clo_f_h, cores)
        # CPU baseline: the oracle (C restatement of the FP64 path) on the host cores
        cs = min(CPU_SAMPLE, N_RAYS)
        tc = time.perf_counter()
        for v in model.volumes:
            sel = np.nonzero(vols_h[:cs] == v)[0]
            if len(sel):
                otrees[v].ray_fire(p_h[sel], d_h[sel], threads=cores)
        dtc = time.perf_counter() - tc
        cpu_baseline = {"value": cs / dtc / 1e6, "unit": "Mrays/s", "cores": cores, "kind": "port",
                        "sample": f"first {cs} rays of the workload, FP64, BVH, OpenMP"}
        log(f"[bench] oracle check + cpu baseline {time.perf_counter() - t1:.1f}s")

    # ---- C5: tet walk ------------------------------------------------------
    t0 = time.perf_counter()
    tm = synth.tet_cube(50, 10.0, 0.2, 11)
    wm = synth.Model(volumes=[1], tets=tm, elements={1: np.arange(len(tm.conn), dtype=np.int32)})
    wr = XDG(wm, device=local)
    wr.prepare_raytracer()
    s_h, u_h, len_h = c5_tracks(N_TRACKS, dist.rank_seed(4321, rank))
    ws = torch.from_numpy(s_h).to(dev)
    wu = torch.from_numpy(u_h).to(dev)
    wl = torch.from_numpy(len_h).to(dev)
    we_idx = torch.empty(N_TRACKS, dtype=torch.int32, device=dev)
    we_id = torch.empty(N_TRACKS, dtype=torch.int32, device=dev)
    seg_e = torch.empty((N_TRACKS, MAX_SEGS), dtype=torch.int32, device=dev)
    seg_l = torch.empty((N_TRACKS, MAX_SEGS), dtype=torch.float64, device=dev)
    seg_c = torch.empty(N_TRACKS, dtype=torch.int32, device=dev)
    wst = torch.empty(N_TRACKS, dtype=torch.int32, device=dev)
    et = wr.volume_to_point_location_tree[1]
    log(f"[bench] C5 setup {time.perf_counter() - t0:.1f}s")
    if args.autotune:
        ss_h, su_h, sl_h = c5_tracks(min(TUNE_TRACKS, N_TRACKS), dist.rank_seed(998, rank))
        _, sidx = wr.find_element(ss_h, precision=MIXED)
        sdev = [torch.from_numpy(a).to(dev) for a in (sidx.astype(np.int32), ss_h, su_h, sl_h)]
        t1 = time.perf_counter()
        ms_w, wt = wr.rti.autotune_walk(*sdev, max_segs=MAX_SEGS, precision=MIXED, reps=3)
        tuning.update({"walk_sample_tracks": len(ss_h), "walk_seconds": time.perf_counter() - t1,
                       "walk_sample_ms": ms_w, "walk": {k: wt[k] for k in WALK_KEYS}})
        del sdev
        log(f"[bench] autotune walk {tuning['walk_seconds']:.1f}s: {tuning['walk']}")

    def find_el(prec, idx):
        def go():
            rc = L.xdgcu_find_element(wr.rti.ctx, et, None, N_TRACKS, ctypes.c_void_p(ws.data_ptr()),
                                      ctypes.c_void_p(we_id.data_ptr()),
                                      ctypes.c_void_p(idx.data_ptr()), None, prec, sptr)
            _lib.check(rc, wr.rti.ctx, "find_element")
        return go

    def walk(prec, idx, e=seg_e, ln=seg_l, c=seg_c):
        def go():
            rc = L.xdgcu_walk_elements(wr.rti.ctx, N_TRACKS, ctypes.c_void_p(idx.data_ptr()),
                                       ctypes.c_void_p(ws.data_ptr()), ctypes.c_void_p(wu.data_ptr()),
                                       ctypes.c_void_p(wl.data_ptr()), MAX_SEGS,
                                       ctypes.c_void_p(e.data_ptr()), ctypes.c_void_p(ln.data_ptr()),
                                       ctypes.c_void_p(c.data_ptr()), ctypes.c_void_p(wst.data_ptr()),
                                       prec, sptr)
            _lib.check(rc, wr.rti.ctx, "walk_elements")
        return go

    # find_element of the track starts, then the walk alone (it reads the
    # start elements find_element wrote and nothing else of it)
    ms_find = timed(torch, find_el(MIXED, we_idx), max(3, args.steps // 4), 2, world, stream)
    we_id_mixed = we_id.clone()
    we_idx64 = torch.empty_like(we_idx)
    ms_find64 = timed(torch, find_el(FP64, we_idx64), 3, 1, world, stream)
    find_mism = int((we_idx64 != we_idx).sum().item()) + int((we_id != we_id_mixed).sum().item())
    ms_walk = timed(torch, walk(MIXED, we_idx), args.steps, args.warmup, world, stream)
    n_segs = int(seg_c.sum().item())
    walk_status_bad = int((wst != 0).sum().item())
    c_mixed = seg_c.clone()
    # FP64 operations of the mixed walk: per step the position update and
    # cross(u, r), plus the exact Plucker test of every face the FP32 filter
    # leaves open (the exit face: ~1.0004 faces per step)
    wr.rti.set_counting(True)
    walk(MIXED, we_idx)()
    torch.cuda.synchronize()
    wcnt = wr.rti.counters()
    wr.rti.set_counting(False)
    esc_per_step = wcnt["escalate"] / max(1, wcnt["steps"])
    fp64_ops_per_seg = WALK_FP64_OPS_STEP + WALK_FP64_OPS_FACE * esc_per_step
    # the same mixed walk with its FP64 edge coordinates computed from the
    # vertices instead of the mesh's edge table
    seg_ex, seg_lx, seg_cx = torch.empty_like(seg_e), torch.empty_like(seg_l), torch.empty_like(seg_c)
    wr.rti.set_tuning("walk_edge_table", 0)
    ms_walk_noedge = timed(torch, walk(MIXED, we_idx, seg_ex, seg_lx, seg_cx),
                           max(3, args.steps // 4), 1, world, stream)
    wr.rti.set_tuning("walk_edge_table", 1)
    vmask = torch.arange(MAX_SEGS, device=dev)[None, :] < c_mixed[:, None]
    walk_edge_table_same = (bool(torch.equal(seg_cx, c_mixed))
                            and bool(torch.equal(torch.where(vmask, seg_ex, 0),
                                                 torch.where(vmask, seg_e, 0)))
                            and bool(torch.equal(torch.where(vmask, seg_lx, 0.0),
                                                 torch.where(vmask, seg_l, 0.0))))
    del seg_ex, seg_lx, seg_cx, vmask
    # FP64 path (its own find_element) into separate buffers for the sequence comparison
    seg_e64 = torch.empty_like(seg_e)
    seg_l64 = torch.empty_like(seg_l)
    seg_c64 = torch.empty_like(seg_c)
    ms_walk64 = timed(torch, walk(FP64, we_idx64, seg_e64, seg_l64, seg_c64),
                      max(3, args.steps // 4), 1, world, stream)
    cols = torch.arange(MAX_SEGS, device=dev)[None, :]
    valid = cols < c_mixed[:, None]
    walk_elem_mism = int((seg_c64 != c_mixed).sum().item()) + int(
        ((seg_e64 != seg_e) & valid).sum().item())
    walk_len_mism = int(((seg_l64 != seg_l) & valid).sum().item())
    del seg_e64, seg_l64, seg_c64, valid
    # the packed walk (one walk in resumed rounds; count + emit walks beside
    # it) and its allocation-free variant
    cap = int(n_segs + N_TRACKS)
    pk_e = torch.empty(cap, dtype=torch.int32, device=dev)
    pk_l = torch.empty(cap, dtype=torch.float64, device=dev)
    pk_off = torch.empty(N_TRACKS + 1, dtype=torch.int64, device=dev)
    pk_st = torch.empty(N_TRACKS, dtype=torch.int32, device=dev)

    def packed(fn):
        def go():
            rc = fn(wr.rti.ctx, N_TRACKS, ctypes.c_void_p(we_idx.data_ptr()),
                    ctypes.c_void_p(ws.data_ptr()), ctypes.c_void_p(wu.data_ptr()),
                    ctypes.c_void_p(wl.data_ptr()), MAX_SEGS, cap, ctypes.c_void_p(pk_e.data_ptr()),
                    ctypes.c_void_p(pk_l.data_ptr()), ctypes.c_void_p(pk_off.data_ptr()),
                    ctypes.c_void_p(pk_st.data_ptr()), MIXED, sptr)
            _lib.check(rc, wr.rti.ctx, "walk_elements_packed")
        return go

    ms_packed = timed(torch, packed(L.xdgcu_walk_elements_packed), max(3, args.steps // 4), 2,
                      world, stream)
    pk_ref = (pk_e[:n_segs].clone(), pk_l[:n_segs].clone(), pk_off.clone())
    # the same entry point walking every track twice (count, then emit)
    wr.rti.set_tuning("packed_walk_passes", 2)
    ms_packed2 = timed(torch, packed(L.xdgcu_walk_elements_packed), max(3, args.steps // 4), 2,
                       world, stream)
    wr.rti.set_tuning("packed_walk_passes", 1)
    packed2_same = (bool(torch.equal(pk_off, pk_ref[2])) and bool(torch.equal(pk_e[:n_segs], pk_ref[0]))
                    and bool(torch.equal(pk_l[:n_segs], pk_ref[1])))
    ms_packed_na = (timed(torch, packed(L.xdgcu_walk_elements_packed_noalloc),
                          max(3, args.steps // 4), 2, world, stream)
                    if N_TRACKS <= NOALLOC_MAX_TRACKS else None)
    packed_same = (ms_packed_na is not None and bool(torch.equal(pk_off, pk_ref[2]))
                   and bool(torch.equal(pk_e[:n_segs], pk_ref[0]))
                   and bool(torch.equal(pk_l[:n_segs], pk_ref[1]))
                   and int(pk_off[-1].item()) == n_segs)
    del pk_e, pk_l, pk_off, pk_st, pk_ref

    # oracle agreement at full size: find_element and the walk of WALK_CHECK
    # tracks spread over the batch, element sequences (zero-length segments
    # included), lengths and status bit for bit; and the oracle's own
    # find_element + walk on the host cores (tools/tally_segments.h:50-62)
    walk_oracle = None
    walk_cpu = None
    if rank == 0 and not args.no_oracle:
        from oracle import oracle as xo
        xo.build()
        cores = os.cpu_count() or 1
        t1 = time.perf_counter()
        otree = xo.TetTree(tm.tet_xyz(), tm.elem_ids)
        owalk = xo.TetWalker(tm.vertices, tm.conn, tm.adj, tm.face_table)
        ksel = np.arange(0, N_TRACKS, max(1, N_TRACKS // WALK_CHECK))
        oid, oidx = otree.find_element(s_h[ksel], threads=cores)
        eid_h = we_id_mixed.cpu().numpy()[ksel]
        eidx_h = we_idx.cpu().numpy()[ksel]
        ok = oidx >= 0
        oe, ol, oc, ost = owalk.walk(np.where(ok, oidx, 0).astype(np.int32), s_h[ksel], u_h[ksel],
                                     np.where(ok, len_h[ksel], 0.0), max_segs=MAX_SEGS,
                                     threads=cores)
        kdev = torch.from_numpy(ksel).to(dev)
        ce = seg_e[kdev].cpu().numpy()
        cl = seg_l[kdev].cpu().numpy()
        cc = c_mixed[kdev].cpu().numpy()
        cs_ = wst[kdev].cpu().numpy()
        oc = np.where(ok, oc, 0)
        valid = np.arange(MAX_SEGS)[None, :] < oc[:, None]
        oe_ids = np.where(valid, tm.elem_ids[np.clip(oe, 0, len(tm.elem_ids) - 1)], 0)
        walk_oracle = {
            "tracks": int(len(ksel)), "segments": int(oc.sum()),
            "find_element_mismatches": int((oid != eid_h).sum() + (oidx != eidx_h).sum()),
            "count_mismatches": int((cc != oc).sum()),
            "element_mismatches": int(((np.where(valid, ce, 0) != oe_ids)).sum()),
            "length_mismatches": int(((np.where(valid, cl, 0.0) != np.where(valid, ol, 0.0))).sum()),
            "status_mismatches": int((cs_[ok] != ost[ok]).sum()),
            "max_rel_length_error": float(np.max(np.abs(np.where(valid, cl - ol, 0.0))
                                                 / np.maximum(np.abs(np.where(valid, ol, 1.0)), 1e-300),
                                                 initial=0.0)),
        }
        del oe, ol, ce, cl, valid, oe_ids
        # CPU baseline: find_element + walk of WALK_CPU_SAMPLE tracks
        nb = min(WALK_CPU_SAMPLE, N_TRACKS)
        tc = time.perf_counter()
        segs_cpu = 0
        for b0 in range(0, nb, 25_000):
            sl_ = slice(b0, min(nb, b0 + 25_000))
            _, bidx = otree.find_element(s_h[sl_], threads=cores)
            bok = bidx >= 0
            _, _, bc, _ = owalk.walk(np.where(bok, bidx, 0).astype(np.int32), s_h[sl_], u_h[sl_],
                                     np.where(bok, len_h[sl_], 0.0), max_segs=MAX_SEGS,
                                     threads=cores)
            segs_cpu += int(bc[bok].sum())
        dtc = time.perf_counter() - tc
        walk_cpu = {"value": segs_cpu / dtc / 1e6, "unit": "Msegs/s", "cores": cores,
                    "kind": "port",
                    "sample": f"first {nb} tracks: find_element + walk_elements, FP64, BVH, OpenMP"}
        log(f"[bench] walk oracle check + cpu baseline {time.perf_counter() - t1:.1f}s")

    # ---- device particle loop (walk_elements tool) over the same mesh ------
    global_segments = bench_global_segments(torch, L, dev, stream, sptr, args, rank, world)
    transport = bench_transport(torch, L, wr, dev, stream, sptr, ws, wu, we_idx, tm, args, rank,
                                world)

    # ---- many surfaces: one launch vs one launch per volume vs CUDA graph -----
    many = bench_many_surfaces(torch, L, dev, stream, args, rank, world) if args.many else None

    # ---- report -------------------------------------------------------------
    total_rays = dist.sum_over_ranks(N_RAYS, world)
    total_segs = dist.sum_over_ranks(n_segs, world)
    total_tracks = dist.sum_over_ranks(N_TRACKS, world)
    value = total_rays / (ms_mixed / 1e3) / 1e6
    peak, peak_kind = measured_peaks()
    achieved = bytes_per_ray * N_RAYS / (ms_mixed / 1e3) / 1e9
    prof = profile_traffic()
    traffic = None
    if prof and prof.get("dram_bytes_per_ray"):
        traffic = prof["dram_bytes_per_ray"] * N_RAYS
    h2d = N_RAYS * (24 + 24 + 4)
    d2h = N_RAYS * (8 + 4 + 4)
    walk_value = total_segs / (ms_walk / 1e3) / 1e6
    walk_fp64_value = total_segs / (ms_walk64 / 1e3) / 1e6
    # the walk's roofline: FP64 operations per segment against the measured
    # FP64 issue rate, and bytes per segment against HBM
    fp64_peak = peaks.get("fp64_add_gops")
    walk_fp64_achieved = fp64_ops_per_seg * n_segs / (ms_walk / 1e3) / 1e9
    walk_hbm_achieved = WALK_BYTES_SEG_MIXED * n_segs / (ms_walk / 1e3) / 1e9
    width = rti.get_tuning("node_width")
    flops_per_ray = FLOPS_TRI * per_ray["prim"] + FLOPS_BOX * width * per_ray["node"]
    fp32_peak = 2.0 * peaks["fp32_fma_gops"] / 1e3 if peaks.get("fp32_fma_gops") else None
    fp32_achieved = flops_per_ray * N_RAYS / (ms_mixed / 1e3) / 1e12
    fp32_roofline = {"flops_per_ray": flops_per_ray, "achieved": fp32_achieved,
                     "peak": fp32_peak, "unit": "TFLOP/s",
                     "frac": fp32_achieved / fp32_peak if fp32_peak else None,
                     "peak_kind": "measured in this run: FP32 FMA issue rate x 2 (peaks.cu)"}
    walk_roofline = {
        "bound": "fp64", "kernel": "k_walk<MOAB, mixed>",
        "achieved": walk_fp64_achieved, "peak": fp64_peak, "unit": "GFP64op/s",
        "frac": walk_fp64_achieved / fp64_peak if fp64_peak else None,
        "fp64_ops_per_segment": fp64_ops_per_seg,
        "fp64_faces_per_step": esc_per_step,
        "peak_kind": "measured in this run: FP64 add issue rate (peaks.cu)",
        "hbm": {"achieved": walk_hbm_achieved, "peak": peak, "unit": "GB/s",
                "frac": walk_hbm_achieved / peak, "bytes_per_segment": WALK_BYTES_SEG_MIXED},
        "fp64_path": {
            "achieved": WALK_FP64_OPS_FP64_PATH * n_segs / (ms_walk64 / 1e3) / 1e9,
            "frac": (WALK_FP64_OPS_FP64_PATH * n_segs / (ms_walk64 / 1e3) / 1e9 / fp64_peak
                     if fp64_peak else None),
            "fp64_ops_per_segment": WALK_FP64_OPS_FP64_PATH},
    }
    line = {
        "metric": METRIC,
        "value": value,
        "unit": "Mrays/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_mixed,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32+f64",
        "data": "synthetic",
        "config": {
            "workload": WORKLOAD if N_RAYS == 10_000_000 else f"{WORKLOAD}_profile_case_{N_RAYS}",
            "rays_per_gpu": N_RAYS,
            "triangles": int(sum(len(s.face_ids) for s in model.surfaces)),
            "volumes": len(model.volumes),
            "precision": "mixed (FP32 boxes + certified FP32 Plucker filter, FP64 escalation)",
            "l2": "streamed inputs 520 MB > 129 MB L2 per step; no flush",
            "parallelism": f"replicas{world} (rays sharded by rank, geometry replicated)",
        },
        "roofline": {
            "bound": "hbm",
            "achieved": achieved,
            "peak": peak,
            "unit": "GB/s",
            "frac": achieved / peak,
            "traffic": traffic,
            "peak_kind": f"{peak_kind} HBM copy bandwidth",
            "kernel": f"k_trace<RAY_FIRE, mixed, {rti.get_tuning('trace_occupancy')}>",
            "algorithmic_bytes_per_ray": bytes_per_ray,
            # the other bounds of the same launch: the algorithmic bytes
            # against the measured L2 read bandwidth (the tree is served from
            # L2), FP32 flops against the measured FP32 FMA rate (2 flops
            # each), and the ray I/O alone
            "l2": {"achieved": achieved, "peak": peaks.get("l2_read_gbs"), "unit": "GB/s",
                   "frac": achieved / peaks["l2_read_gbs"] if peaks.get("l2_read_gbs") else None},
            "fp32": fp32_roofline,
            "io_only": {"bytes_per_ray": BYTES_IO_ONLY,
                        "achieved": BYTES_IO_ONLY * N_RAYS / (ms_mixed / 1e3) / 1e9,
                        "frac": BYTES_IO_ONLY * N_RAYS / (ms_mixed / 1e3) / 1e9 / peak},
        },
        "cpu_baseline": cpu_baseline,
        "e2e": {"value": total_rays / (ms_e2e / 1e3) / 1e6, "unit": "Mrays/s",
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "matches_device_path": e2e_ok,
                "transfer": e2e_transfer,
                "staged_value": total_rays / (ms_e2e_staged / 1e3) / 1e6,
                "host_direct_choice": hd_choice,
                "outputs_staged_value": total_rays / (ms_e2e_out_staged / 1e3) / 1e6,
                "in_place_value": total_rays / (ms_e2e_in_place / 1e3) / 1e6,
                "pageable_staged_value": total_rays / (ms_e2e_pageable / 1e3) / 1e6,
                "pageable_direct_value": (total_rays / (ms_e2e_pageable_direct / 1e3) / 1e6
                                          if ms_e2e_pageable_direct else None)},
        # secondary workloads first: the end of the line carries the headline
        # comparisons and the parity checks
        "configs_small": small_configs,
        "overlap_check": overlap,
        "transport": transport,
        "global_segments": global_segments,
        "surface_transport": surface_transport,
        "many_surfaces": many,
        "tuning": tuning,
        "peaks_measured": peaks,
        "mixed_without_edge_table": {"value": total_rays / (ms_mixed_noedge / 1e3) / 1e6,
                                     "unit": "Mrays/s", "same_results": edge_table_same},
        "point_in_volume": {
            "value": total_rays / (ms_piv / 1e3) / 1e6, "unit": "Mpoints/s",
            "fp64_value": total_rays / (ms_piv64 / 1e3) / 1e6,
            "inside_fraction_own_volume": piv_inside_frac,
            "mixed_equals_fp64": piv_same,
            "oracle_check": query_oracle.get("point_in_volume"),
        },
        "occluded": {
            "value": total_rays / (ms_occ / 1e3) / 1e6, "unit": "Mrays/s",
            "fp64_value": total_rays / (ms_occ64 / 1e3) / 1e6,
            "mixed_equals_fp64": occ_same,
            "oracle_check": query_oracle.get("occluded"),
        },
        "closest": {
            "points": n_clo, "unit": "Mpoints/s",
            "value": dist.sum_over_ranks(n_clo, world) / (ms_clo / 1e3) / 1e6,
            "fp64_value": dist.sum_over_ranks(n_clo, world) / (ms_clo64 / 1e3) / 1e6,
            "value_without_triangle_bound": dist.sum_over_ranks(n_clo, world) / (ms_clo_nb / 1e3) / 1e6,
            "value_one_lane_per_point": dist.sum_over_ranks(n_clo, world) / (ms_clo_lane / 1e3) / 1e6,
            "value_caller_order": dist.sum_over_ranks(n_clo, world) / (ms_clo_unsorted / 1e3) / 1e6,
            "mixed_equals_fp64": clo_same,
            "oracle_check": query_oracle.get("closest"),
        },
        "find_volume": {
            "value": total_rays / (ms_fv / 1e3) / 1e6, "unit": "Mpoints/s",
            "per_volume_launches_value": total_rays / (ms_fv_loop / 1e3) / 1e6,
            "ms_fused": ms_fv, "ms_per_volume": ms_fv_loop,
            "fused_equals_per_volume": fv_same, "device_equals_host_path": fv_host_same,
            "volumes_tried_in_order": len(fv_vols),
            "oracle_check": fv_oracle,
        },
        "escalations_per_ray": per_ray["escalate"],
        "nodes_per_ray": per_ray["node"],
        "prims_per_ray": per_ray["prim"],
        "hit_fraction": hit_frac,
        "walk": {
            "workload": WALK_WORKLOAD,
            "value": walk_value, "unit": "Msegs/s",
            "fp64_value": walk_fp64_value,
            "step": "walk_elements alone (k_walk); find_element timed separately",
            "ms_per_step": ms_walk, "fp64_ms_per_step": ms_walk64,
            "find_element": {"unit": "Mpoints/s", "ms": ms_find, "fp64_ms": ms_find64,
                             "value": total_tracks / (ms_find / 1e3) / 1e6,
                             "fp64_value": total_tracks / (ms_find64 / 1e3) / 1e6,
                             "mismatches_mixed_vs_fp64": find_mism},
            "with_find_element_value": total_segs / ((ms_walk + ms_find) / 1e3) / 1e6,
            "value_without_edge_table": total_segs / (ms_walk_noedge / 1e3) / 1e6,
            "edge_table_same_segments": walk_edge_table_same,
            "packed_value": total_segs / (ms_packed / 1e3) / 1e6,
            "packed_two_pass_value": total_segs / (ms_packed2 / 1e3) / 1e6,
            "packed_two_pass_equals_packed": packed2_same,
            "packed_noalloc_value": (total_segs / (ms_packed_na / 1e3) / 1e6
                                     if ms_packed_na else None),
            "packed_noalloc_equals_packed": packed_same,
            "segments": n_segs, "tracks": N_TRACKS,
            "speedup_mixed_vs_fp64": ms_walk64 / ms_walk,
            "element_mismatches_mixed_vs_fp64": walk_elem_mism,
            "length_mismatches_mixed_vs_fp64": walk_len_mism,
            "tracks_with_status": walk_status_bad,
            "roofline": walk_roofline,
            "cpu_baseline": walk_cpu,
            "oracle_check": walk_oracle,
        },
        "fp64": {"value": total_rays / (ms_fp64 / 1e3) / 1e6, "unit": "Mrays/s",
                 "ms_per_step": ms_fp64},
        "speedup_mixed_vs_fp64": ms_fp64 / ms_mixed,
        "id_mismatches_mixed_vs_fp64": id_mism,
        "t_mismatches_mixed_vs_fp64": t_mism,
        "max_rel_t_error_mixed_vs_fp64": max_rel_t,
        "oracle_check": oracle_mism,
        "summary": {
            "ray_fire_Mrays_s": {"mixed": round(value, 1),
                                 "fp64": round(total_rays / (ms_fp64 / 1e3) / 1e6, 1),
                                 "e2e": round(total_rays / (ms_e2e / 1e3) / 1e6, 1)},
            "walk_Msegs_s": {"mixed": round(walk_value, 1), "fp64": round(walk_fp64_value, 1),
                             "fp64_frac": (round(walk_roofline["frac"], 3)
                                           if walk_roofline["frac"] else None),
                             "cpu": round(walk_cpu["value"], 1) if walk_cpu else None},
            "oracle_mismatches": {
                "ray_fire": oracle_mism["mismatches"] if oracle_mism else None,
                "find_volume": fv_oracle["mismatches"] if fv_oracle else None,
                "walk": (walk_oracle["count_mismatches"] + walk_oracle["element_mismatches"]
                         + walk_oracle["length_mismatches"] + walk_oracle["status_mismatches"]
                         + walk_oracle["find_element_mismatches"]) if walk_oracle else None,
                "point_in_volume": (query_oracle["point_in_volume"]["mismatches"]
                                    if query_oracle else None),
                "occluded": (query_oracle["occluded"]["flag_mismatches"]
                             + query_oracle["occluded"]["distance_mismatches"]
                             if query_oracle else None),
                "closest": (query_oracle["closest"]["distance_mismatches"]
                            + query_oracle["closest"]["face_mismatches"] if query_oracle else None)},
            "global_segments_Msegs_s": {
                "mixed": round(global_segments["value"], 1),
                "fp64": round(global_segments["fp64_value"], 1),
                "oracle_tracks_differing": (global_segments.get("oracle_check") or {}).get(
                    "tracks_differing")},
            "mixed_vs_fp64_mismatches": {"ray_fire": id_mism + t_mism,
                                         "walk": walk_elem_mism + walk_len_mism},
        },
        "gpu_launches": args.steps * launches_per_step,
        "clocks": clk,
    }
    if rank == 0:
        log(f"[bench] summary {json.dumps(line['summary'])}")
        print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--no-oracle", action="store_true")
    ap.add_argument("--rays", type=int, default=N_RAYS,
                    help="rays per GPU (smaller values are profiling cases, not the workload)")
    ap.add_argument("--tracks", type=int, default=N_TRACKS, help="walk tracks per GPU")
    ap.add_argument("--no-many", dest="many", action="store_false",
                    help="skip the 256-surface launch comparison")
    ap.add_argument("--no-autotune", dest="autotune", action="store_false",
                    help="keep the default launch settings instead of autotuning them")
    args = ap.parse_args()
    set_sizes(args.rays, args.tracks)
    args.warmup = max(3, args.warmup)
    rank, world, local = dist.env_rank()
    if world > 1:
        import torch
        import torch.distributed as tdist
        if args.impl == "engine":
            torch.cuda.set_device(local)
            tdist.init_process_group("nccl", device_id=torch.device("cuda", local))
        else:
            tdist.init_process_group("gloo")
    try:
        if args.impl == "reference":
            return run_reference(args, rank, world)
        return run_engine(args, rank, world, local)
    finally:
        if world > 1:
            import torch.distributed as tdist
            tdist.destroy_process_group()


if __name__ == "__main__":
    sys.exit(main())
