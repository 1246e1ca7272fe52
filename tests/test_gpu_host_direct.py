"""Host arrays that the kernels read and write in place (tuning key
host_direct) give the same bytes as host arrays staged through device memory
and as device arrays.

ray_fire runs on 4.5e6 rays (more than two staging chunks) with the inputs
and outputs in page-locked memory, pageable memory, or page-locked inputs
with pageable outputs (some arrays in place, the rest staged), under each
host_direct setting (2 keeps both kinds in place; 3 stages the page-locked
arrays of this large call in overlapping chunks; 4 stages only its
page-locked inputs and writes the outputs in place; staged chunks' kernels
alternate between two streams; 5, the default, picks 2, 3 or 4 by timing the
first large calls), and with the node steps of in-place launches
(trace_node_iters_direct) varied.  The packed tet walk and the walk_elements particle loop
(whose atomic tally is always staged) are checked the same way.
"""
import ctypes

import numpy as np
import pytest

from xdg_gb300 import _lib, synth
from xdg_gb300.engine import FP64, MIXED, XDG

pytestmark = pytest.mark.gpu


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _buffers(torch, kind, n, inputs):
    """Copies of `inputs` (numpy) and fresh outputs in memory of `kind`."""
    dev = torch.device("cuda", 0)

    def mk(a, where):
        t = torch.from_numpy(np.ascontiguousarray(a))
        if where == "device":
            return t.to(dev)
        if where == "pinned":
            return t.pin_memory()
        return t.clone()

    def out(dtype, where):
        if where == "device":
            return torch.empty(n, dtype=dtype, device=dev)
        return torch.empty(n, dtype=dtype, pin_memory=(where == "pinned"))

    src, dst = {"mixed": ("pinned", "pageable")}.get(kind, (kind, kind))
    ins = [mk(a, src) for a in inputs]
    outs = [out(torch.float64, dst), out(torch.int32, dst), out(torch.int32, dst),
            out(torch.int32, dst)]
    return ins, outs


@pytest.fixture(scope="module")
def rays(cuda):
    m = synth.nested_spheres(n=4, level=3, jitter=1e-3, seed=7)
    x = XDG(m)
    x.prepare_raytracer()
    rng = np.random.default_rng(5)
    n = 4_500_000
    p = rng.uniform(-4.5, 4.5, (n, 3))
    d = synth.isotropic_dirs(rng, n)
    vols = x.find_volume(p, d)
    lut = np.zeros(max(m.volumes) + 1, dtype=np.int32)
    for v, t in x.volume_to_surface_tree.items():
        lut[v] = t
    return x, p, d, lut[vols]


@pytest.mark.parametrize("prec", [MIXED, FP64])
def test_ray_fire_host_buffers(cuda, rays, prec):
    torch = cuda
    x, p, d, trees = rays
    rti = x.rti
    L = _lib.load()
    n = len(p)
    old = rti.get_tuning("host_direct")

    def fire(kind, direct):
        rti.set_tuning("host_direct", direct)
        (tr, o, u), outs = _buffers(torch, kind, n, [trees, p, d])
        rc = L.xdgcu_ray_fire(rti.ctx, 0, _ptr(tr), n, _ptr(o), _ptr(u), None, 0, None, None,
                              *[_ptr(t) for t in outs], prec, None)
        _lib.check(rc, rti.ctx, "ray_fire")
        torch.cuda.synchronize()
        return [t.cpu().numpy() for t in outs]

    old_iters = rti.get_tuning("trace_node_iters_direct")
    try:
        ref = fire("device", 1)
        assert (ref[1] >= 0).mean() > 0.5
        for kind in ("pinned", "pageable", "mixed"):
            for direct in (0, 1, 2, 3, 4, 5):
                got = fire(kind, direct)
                for a, b, what in zip(got, ref, ("t", "surface", "face", "status")):
                    assert np.array_equal(a, b), f"{kind} host_direct={direct}: {what}"
        # the node steps of launches reading their rays in place
        for iters in (1, 3, 16):
            rti.set_tuning("trace_node_iters_direct", iters)
            got = fire("pinned", 2)
            for a, b, what in zip(got, ref, ("t", "surface", "face", "status")):
                assert np.array_equal(a, b), f"trace_node_iters_direct={iters}: {what}"
    finally:
        rti.set_tuning("host_direct", old)
        rti.set_tuning("trace_node_iters_direct", old_iters)


def test_automatic_policy_choice(cuda, rays):
    """host_direct 5 runs the first nine large page-locked calls in place,
    staged and with the inputs in place and the outputs staged in turn, times
    the last six (the first of each pays one-time costs), then keeps the
    fastest; every call gives the same results, and setting 5 again starts a
    new choice."""
    torch = cuda
    x, p, d, trees = rays
    rti = x.rti
    L = _lib.load()
    n = len(p)
    old = rti.get_tuning("host_direct")
    try:
        rti.set_tuning("host_direct", 5)
        assert rti.get_tuning("host_direct_choice") == -1
        (tr, o, u), outs = _buffers(torch, "pinned", n, [trees, p, d])
        ref = None
        for call in range(11):
            rc = L.xdgcu_ray_fire(rti.ctx, 0, _ptr(tr), n, _ptr(o), _ptr(u), None, 0, None, None,
                                  *[_ptr(t) for t in outs], MIXED, None)
            _lib.check(rc, rti.ctx, "ray_fire")
            got = [t.clone() for t in outs]
            if ref is None:
                ref = got
            else:
                assert all(bool(torch.equal(a, b)) for a, b in zip(got, ref)), call
            choice = rti.get_tuning("host_direct_choice")
            assert (choice == -1) if call < 8 else (choice in (2, 3, 4)), (call, choice)
        rti.set_tuning("host_direct", 5)
        assert rti.get_tuning("host_direct_choice") == -1
    finally:
        rti.set_tuning("host_direct", old)


def test_walk_and_transport_host_buffers(cuda):
    torch = cuda
    tm = synth.tet_cube(12, 10.0, 0.2, 11)
    m = synth.Model(volumes=[1], tets=tm, elements={1: np.arange(len(tm.conn), dtype=np.int32)})
    x = XDG(m)
    x.prepare_raytracer()
    rti = x.rti
    rng = np.random.default_rng(3)
    n = 50_000
    s = rng.uniform(0.1, 9.9, (n, 3))
    u = synth.isotropic_dirs(rng, n)
    ln = rng.exponential(5.0, n)
    _, eidx = x.find_element(s)
    eidx = np.asarray(eidx, dtype=np.int32)
    old = rti.get_tuning("host_direct")
    dev = torch.device("cuda", 0)

    def conv(a, kind):
        t = torch.from_numpy(np.ascontiguousarray(a))
        return t.to(dev) if kind == "device" else (t.pin_memory() if kind == "pinned" else t)

    def walk(kind):
        args = [conv(a, kind) for a in (eidx, s, u, ln)]
        se, sl, off, st = rti.walk_elements_packed(*args, 64 * n, precision=MIXED)
        torch.cuda.synchronize()
        tot = int(off[-1])
        return se.cpu().numpy()[:tot], sl.cpu().numpy()[:tot], off.cpu().numpy(), st.cpu().numpy()

    def transport(kind):
        seeds = rti.seed_streams(99, n).view(np.int64)
        state = [conv(a.copy(), kind) for a in (eidx, s, u, seeds, np.zeros(n), np.zeros(n, np.int32))]
        tally = conv(np.zeros(len(tm.conn)), kind)
        st = rti.transport_elements(state[0], state[1], state[2], state[3], 2.0, 1_000_000,
                                    state[4], state[5], tally=tally, precision=MIXED)
        torch.cuda.synchronize()
        return [t.cpu().numpy() for t in state] + [st.cpu().numpy(), tally.cpu().numpy()]

    try:
        ref_w = walk("device")
        ref_t = transport("device")
        assert ref_w[2][-1] > n and (ref_t[5] > 0).all()
        for kind in ("pinned", "pageable"):
            for direct in (0, 1, 2, 3, 4, 5):
                rti.set_tuning("host_direct", direct)
                for a, b in zip(walk(kind), ref_w):
                    assert np.array_equal(a, b), f"walk {kind} host_direct={direct}"
                got = transport(kind)
                for a, b in zip(got[:-1], ref_t[:-1]):
                    assert np.array_equal(a, b), f"transport {kind} host_direct={direct}"
                # atomic additions in any order: the tally agrees to rounding
                assert np.allclose(got[-1], ref_t[-1], rtol=1e-12, atol=0)
    finally:
        rti.set_tuning("host_direct", old)
