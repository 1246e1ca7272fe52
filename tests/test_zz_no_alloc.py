"""The allocation-free packed walk, xdgcu_walk_elements_packed_noalloc.

Callers whose device memory belongs to another allocator (a framework's
caching pool that reserves the free memory up front, or a transport code's
particle loop that must not enter the allocator once set up) cannot let the
library call cudaMalloc.  For them the library keeps the scratch of the
packed walk's offset scan in a static device array and this entry point
allocates nothing.  The test calls it through the C ABI, twice in a row on
the same inputs, and requires the same packed segments, offsets and status
as the allocating entry point, xdgcu_walk_elements_packed.

This file is named to run last, so a run that stops at the first failure has
already run every other test; it also passes on its own in a fresh process.
"""
import ctypes

import numpy as np
import pytest

from xdg_gb300 import _lib, synth
from xdg_gb300.engine import FP64, MIXED, CudaRayTracer

pytestmark = pytest.mark.gpu


def _tracks(n, seed):
    rng = np.random.default_rng(seed)
    s = rng.uniform(0.0, 10.0, (n, 3))
    u = synth.isotropic_dirs(rng, n)
    with np.errstate(divide="ignore", invalid="ignore"):
        t1 = (0.0 - s) / u
        t2 = (10.0 - s) / u
    ex = np.where(u > 0, t2, np.where(u < 0, t1, np.inf)).min(axis=1)
    return s, u, np.minimum(rng.exponential(5.0, n), ex)


@pytest.mark.parametrize("prec", [MIXED, FP64])
def test_noalloc_walk_matches_allocating_walk(cuda, prec):
    torch = cuda
    dev = torch.device("cuda")
    tm = synth.tet_cube(n=10, size=10.0, jitter=0.2, seed=13)
    rti = CudaRayTracer()
    rti.set_tet_mesh(tm)
    model = synth.Model(volumes=[1], tets=tm, elements={1: np.arange(len(tm.conn), dtype=np.int32)})
    et = rti.create_element_tree(model, 1)
    n = 20000
    s, u, ln = _tracks(n, 7)
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)  # noqa: E731
    ts, tu, tl = T(s), T(u), T(ln)
    _, idx = rti.find_element(et, ts, prec)
    L = _lib.load()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    P = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    max_segs = 512

    def run(fn, capacity):
        se = torch.full((capacity,), -7, dtype=torch.int32, device=dev)
        sl = torch.full((capacity,), -7.0, dtype=torch.float64, device=dev)
        off = torch.full((n + 1,), -7, dtype=torch.int64, device=dev)
        st = torch.full((n,), -7, dtype=torch.int32, device=dev)
        rc = fn(rti.ctx, n, P(idx), P(ts), P(tu), P(tl), max_segs, capacity, P(se), P(sl), P(off),
                P(st), prec, stream)
        _lib.check(rc, rti.ctx, fn.__name__)
        torch.cuda.synchronize()
        return se.cpu().numpy(), sl.cpu().numpy(), off.cpu().numpy(), st.cpu().numpy()

    # the allocating entry point gives the reference answer and the total size
    ref = run(L.xdgcu_walk_elements_packed, 1)
    total = int(ref[2][-1])
    ref = run(L.xdgcu_walk_elements_packed, total)
    assert ref[2][-1] == total and (ref[3] == 0).all()
    for call in range(2):  # the static scratch keeps the previous call's contents
        got = run(L.xdgcu_walk_elements_packed_noalloc, total)
        assert np.array_equal(got[2], ref[2]), call
        assert np.array_equal(got[3], ref[3]), call
        assert np.array_equal(got[0], ref[0]), call
        assert np.array_equal(got[1], ref[1]), call


def test_noalloc_walk_rejects_oversized_batches(cuda):
    torch = cuda
    tm = synth.tet_cube(n=2, size=1.0, jitter=0.0)
    rti = CudaRayTracer()
    rti.set_tet_mesh(tm)
    L = _lib.load()
    dummy = torch.zeros(8, dtype=torch.float64, device="cuda")
    p = ctypes.c_void_p(dummy.data_ptr())
    rc = L.xdgcu_walk_elements_packed_noalloc(rti.ctx, 4194305, p, p, p, p, 16, 0, None, None, p,
                                              None, MIXED, None)
    assert rc != 0
    assert b"XDGCU_NOALLOC_MAX_TRACKS" in L.xdgcu_last_error(rti.ctx)
