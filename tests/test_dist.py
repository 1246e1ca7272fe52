"""Multi-rank host logic of bench.py on CPU: rays shard by index range with no
collective on the data path; only the timing is reduced (max over ranks) and
the unit counts summed.  Two gloo ranks on 127.0.0.1."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import torch.distributed as dist
    from xdg_gb300 import dist as xd
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, w, local = xd.env_rank()
        lo, hi = xd.shard_range(10_000_001, r, w)
        ms = xd.max_over_ranks(10.0 + r, w)
        total = xd.sum_over_ranks(hi - lo, w)
        xd.barrier(w)
        q.put((r, lo, hi, ms, total, xd.rank_seed(1234, r)))
    finally:
        dist.destroy_process_group()


def test_two_rank_sharding_and_timing():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, lo0, hi0, ms0, tot0, s0), (r1, lo1, hi1, ms1, tot1, s1) = out
    assert (lo0, hi1) == (0, 10_000_001) and hi0 == lo1
    assert abs((hi0 - lo0) - (hi1 - lo1)) <= 1
    assert ms0 == ms1 == 11.0          # max over ranks
    assert tot0 == tot1 == 10_000_001  # every ray counted once
    assert s0 != s1                    # independent inputs per rank


def test_shard_range_covers_everything():
    from xdg_gb300.dist import shard_range
    for n in (0, 1, 7, 100, 12345):
        for w in (1, 2, 3, 8):
            parts = [shard_range(n, r, w) for r in range(w)]
            assert parts[0][0] == 0 and parts[-1][1] == n
            assert all(parts[i][1] == parts[i + 1][0] for i in range(w - 1))


@pytest.mark.parametrize("n", [1])
def test_single_rank_is_identity(n):
    from xdg_gb300 import dist as xd
    assert xd.max_over_ranks(3.5, 1) == 3.5
    assert xd.sum_over_ranks(3.5, 1) == 3.5


def _split_worker(rank, world, port, q):
    """One rank of a sharded ray_fire: the rank traces its shard_range slice of
    a shared batch (here with the CPU oracle, standing in for the engine on a
    rank's GPU) and the slices are gathered by rank order."""
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import numpy as np
    import torch
    import torch.distributed as dist
    from oracle import oracle as xo
    from xdg_gb300 import dist as xd
    from xdg_gb300 import synth
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, w, _ = xd.env_rank()
        m = synth.single_sphere_in_box(level=3)
        o, d = synth.lcg_ball_rays(3001, 9.9, seed=12345)
        lo, hi = xd.shard_range(len(o), r, w)
        t, s, f = xo.volume_tree(m, 1).ray_fire(o[lo:hi], d[lo:hi], threads=1)
        # gather the slices (sizes differ by at most one): pad, all_gather, trim
        cap = xd.shard_range(len(o), 0, w)[1]
        buf = torch.full((cap, 3), -2.0, dtype=torch.float64)
        buf[:hi - lo, 0] = torch.from_numpy(t)
        buf[:hi - lo, 1] = torch.from_numpy(s.astype(np.float64))
        buf[:hi - lo, 2] = torch.from_numpy(f.astype(np.float64))
        parts = [torch.empty_like(buf) for _ in range(w)]
        dist.all_gather(parts, buf)
        if r == 0:
            rows = [parts[k][:xd.shard_range(len(o), k, w)[1] - xd.shard_range(len(o), k, w)[0]]
                    for k in range(w)]
            q.put(torch.cat(rows).numpy())
        else:
            q.put(None)
    finally:
        dist.destroy_process_group()


def test_sharded_batch_equals_one_rank():
    """A batch split with shard_range over two gloo ranks, each tracing its own
    slice, gives the single-process results once gathered in rank order."""
    import numpy as np
    import torch.multiprocessing as mp
    from oracle import oracle as xo
    from xdg_gb300 import synth
    xo.build()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_split_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=180) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    got = next(x for x in res if x is not None)
    m = synth.single_sphere_in_box(level=3)
    o, d = synth.lcg_ball_rays(3001, 9.9, seed=12345)
    t, s, f = xo.volume_tree(m, 1).ray_fire(o, d, threads=1)
    assert got.shape == (3001, 3)
    assert np.array_equal(got[:, 0], t)
    assert np.array_equal(got[:, 1].astype(np.int32), s)
    assert np.array_equal(got[:, 2].astype(np.int32), f)
