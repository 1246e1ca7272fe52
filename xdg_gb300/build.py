"""Build the CUDA engine (libxdgcu.so) for sm_103a, in-tree.

    python -m xdg_gb300.build          # or __graft_entry__.build()

Each .cu translation unit is compiled in parallel with

    nvcc -gencode arch=compute_103a,code=sm_103a -O3 -lineinfo -fmad=false ...

``-fmad=false`` keeps every FP64 product and sum separately rounded, which is
what makes the double-precision results bit-identical to the reference's C++
(host code is compiled with -ffp-contract=off for the same reason).  FP32
code that wants a fused multiply-add asks for it explicitly (__fmaf_rn).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libxdgcu.so")
# throughput microbenchmarks for the roofline denominators (not the engine)
PEAKS_SRC = "peaks.cu"
PEAKS_LIB = os.path.join(OUT_DIR, "libxdgpeaks.so")
SOURCES = ["api.cu", "bvh.cu", "noalloc.cu", "order.cu", "queries.cu", "segments.cu", "trace.cu", "tune.cu",
           "walk.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-fmad=false", "-std=c++17", "--expt-relaxed-constexpr",
              "-Xcompiler", "-fPIC,-ffp-contract=off,-O2", "-I", os.path.join(HERE, "..", "include")]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _newer(target: str, deps) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def _headers():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))] + [
        os.path.join(HERE, "..", "include", "xdgcu.h")]


def build(force: bool = False, verbose: bool = False, extra_flags=None) -> str:
    """Compile (if stale) and return the path of libxdgcu.so."""
    os.makedirs(OUT_DIR, exist_ok=True)
    headers = _headers()
    objs = []
    jobs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT_DIR, src.replace(".cu", ".o"))
        objs.append(o)
        if force or not _newer(o, [s] + headers):
            cmd = [nvcc()] + ARCH + NVCC_FLAGS + (extra_flags or []) + ["-c", s, "-o", o]
            jobs.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose:
            sys.stdout.write(r.stdout + r.stderr)

    ps = os.path.join(CSRC, PEAKS_SRC)
    if force or not _newer(PEAKS_LIB, [ps]):
        jobs.append([nvcc()] + ARCH + NVCC_FLAGS + ["-shared", ps, "-o", PEAKS_LIB])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(run, jobs))
    if jobs or not os.path.exists(LIB) or not _newer(LIB, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
