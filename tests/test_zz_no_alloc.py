"""The allocation-free packed walk, xdgcu_walk_elements_packed_noalloc.

Callers whose device memory belongs to another allocator (a framework's
caching pool that reserves the free memory up front, or a transport code's
particle loop that must not enter the allocator once set up) cannot let the
library call cudaMalloc.  For them the library keeps the scratch of the
packed walk's offset scan in a static device array and this entry point
allocates nothing.  The test calls it through the C ABI, twice in a row on
the same inputs, and requires the same packed segments, offsets and status
as the allocating entry point, xdgcu_walk_elements_packed.

The promise itself is checked too: the current memory pool of the device
(the one cudaMallocAsync draws on, which the allocating walk uses) keeps its
high-water mark across a call, and the free device memory is unchanged, so a
stream-ordered allocation or a leaked cudaMalloc inside the call would fail
the test.  A case at exactly XDGCU_NOALLOC_MAX_TRACKS fills the static
scratch to its last entry.

This file is named to run last, so a run that stops at the first failure has
already run every other test; it also passes on its own in a fresh process.
"""
import ctypes

import numpy as np
import pytest

from xdg_gb300 import _lib, synth
from xdg_gb300.engine import FP64, MIXED, CudaRayTracer

pytestmark = pytest.mark.gpu


class _PoolWatch:
    """High-water mark of the device's current memory pool, through the
    driver API (CUmemPool_attribute values from cuda.h)."""
    USED_MEM_CURRENT, USED_MEM_HIGH = 7, 8

    def __init__(self, ordinal):
        self.cu = ctypes.CDLL("libcuda.so.1")
        assert self.cu.cuInit(0) == 0
        dev = ctypes.c_int(0)
        assert self.cu.cuDeviceGet(ctypes.byref(dev), ordinal) == 0
        self.pool = ctypes.c_void_p(0)
        assert self.cu.cuDeviceGetMemPool(ctypes.byref(self.pool), dev) == 0

    def _get(self, attr):
        v = ctypes.c_uint64(0)
        assert self.cu.cuMemPoolGetAttribute(self.pool, attr, ctypes.byref(v)) == 0
        return v.value

    def reset(self):
        """Resets the high-water mark to the pool's current use; returns it."""
        zero = ctypes.c_uint64(0)
        assert self.cu.cuMemPoolSetAttribute(self.pool, self.USED_MEM_HIGH, ctypes.byref(zero)) == 0
        return self._get(self.USED_MEM_CURRENT)

    def high(self):
        return self._get(self.USED_MEM_HIGH)


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

    # no allocation inside a call (after the first call's set-up): the high-
    # water marks of the device's default pool and of the context's scratch
    # pool, and the free memory, stay as they were; the scratch pool's mark
    # sees the allocating entry point's scratch
    outs = [torch.empty(total, dtype=torch.int32, device=dev),
            torch.empty(total, dtype=torch.float64, device=dev),
            torch.empty(n + 1, dtype=torch.int64, device=dev),
            torch.empty(n, dtype=torch.int32, device=dev)]
    watch = _PoolWatch(torch.cuda.current_device())

    def call(fn):
        torch.cuda.synchronize()
        base = watch.reset()
        rti.set_tuning("scratch_bytes_high", 0)
        free0 = torch.cuda.mem_get_info()[0]
        rc = fn(rti.ctx, n, P(idx), P(ts), P(tu), P(tl), max_segs, total, P(outs[0]), P(outs[1]),
                P(outs[2]), P(outs[3]), prec, stream)
        _lib.check(rc, rti.ctx, fn.__name__)
        torch.cuda.synchronize()
        return (watch.high() - base, rti.get_tuning("scratch_bytes_high"),
                free0 - torch.cuda.mem_get_info()[0])

    _, scratch, _ = call(L.xdgcu_walk_elements_packed)
    assert scratch > 0  # the context's pool lends the allocating walk its scratch
    assert rti.get_tuning("scratch_bytes_reserved") > 0  # and keeps it for the next call
    grew, scratch, used = call(L.xdgcu_walk_elements_packed_noalloc)
    assert grew == 0 and scratch == 0 and used == 0
    assert np.array_equal(outs[2].cpu().numpy(), ref[2])


def test_noalloc_walk_at_the_size_limit(cuda):
    """n = XDGCU_NOALLOC_MAX_TRACKS short tracks: the scan's block sums fill
    the static scratch to its last entry; offsets and segments equal the
    allocating walk's."""
    torch = cuda
    dev = torch.device("cuda")
    tm = synth.tet_cube(n=4, size=4.0, jitter=0.2, seed=3)
    rti = CudaRayTracer()
    rti.set_tet_mesh(tm)
    model = synth.Model(volumes=[1], tets=tm, elements={1: np.arange(len(tm.conn), dtype=np.int32)})
    et = rti.create_element_tree(model, 1)
    n = 4194304  # XDGCU_NOALLOC_MAX_TRACKS
    g = torch.Generator(device=dev)
    g.manual_seed(11)
    ts = torch.rand((n, 3), generator=g, device=dev, dtype=torch.float64) * 3.6 + 0.2
    tu = torch.randn((n, 3), generator=g, device=dev, dtype=torch.float64)
    tu = tu / tu.norm(dim=1, keepdim=True)
    tl = torch.rand(n, generator=g, device=dev, dtype=torch.float64) * 0.15 + 1e-3
    _, idx = rti.find_element(et, ts, MIXED)
    assert bool((idx >= 0).all())
    L = _lib.load()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    P = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731

    def run(fn, capacity):
        se = torch.full((max(1, capacity),), -7, dtype=torch.int32, device=dev)
        sl = torch.full((max(1, capacity),), -7.0, dtype=torch.float64, device=dev)
        off = torch.full((n + 1,), -7, dtype=torch.int64, device=dev)
        st = torch.full((n,), -7, dtype=torch.int32, device=dev)
        rc = fn(rti.ctx, n, P(idx), P(ts), P(tu), P(tl), 64, capacity, P(se), P(sl), P(off),
                P(st), MIXED, stream)
        _lib.check(rc, rti.ctx, fn.__name__)
        torch.cuda.synchronize()
        return se, sl, off, st

    _, _, off0, _ = run(L.xdgcu_walk_elements_packed, 0)
    total = int(off0[-1].item())
    assert total >= n
    ref = run(L.xdgcu_walk_elements_packed, total)
    for _ in range(2):
        got = run(L.xdgcu_walk_elements_packed_noalloc, total)
        assert bool(torch.equal(got[2], ref[2])) and int(got[2][-1].item()) == total
        assert bool(torch.equal(got[3], ref[3])) and bool((got[3] == 0).all())
        assert bool(torch.equal(got[0], ref[0])) and bool(torch.equal(got[1], ref[1]))


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
