"""Sharding of independent solves: balanced contiguous ranges, and the
world-size-2 host-side gather over gloo (CPU, no GPU)."""
import os
import socket

import numpy as np
import pytest

from zml_gb300 import shard


def test_ranges_cover_and_balance():
    rng = np.random.default_rng(0)
    ns = rng.integers(8, 257, 20000)
    for world in (1, 2, 3, 4, 8):
        rr = shard.balanced_ranges(ns.astype(float) ** 3, world)
        assert rr[0][0] == 0 and rr[-1][1] == len(ns)
        assert all(a[1] == b[0] for a, b in zip(rr, rr[1:]))
        w = np.array([np.sum(ns[lo:hi].astype(float) ** 3) for lo, hi in rr])
        assert w.max() / w.mean() < 1.01          # contiguous cuts of many small items
    # fewer items than ranks, zero work, single heavy item
    assert shard.balanced_ranges([1.0, 1.0], 4) == [(0, 1), (1, 1), (1, 2), (2, 2)]
    assert shard.balanced_ranges([0.0] * 6, 3) == [(0, 2), (2, 4), (4, 6)]
    assert shard.balanced_ranges([1, 1000, 1], 2) == [(0, 2), (2, 3)]
    assert shard.balanced_ranges([], 2) == [(0, 0), (0, 0)]
    with pytest.raises(ValueError):
        shard.balanced_ranges([1.0], 0)


def test_single_process_gather_is_identity():
    assert shard.gather({"a": 1}) == [{"a": 1}]
    items = list(range(10))
    assert shard.sharded_map(lambda x: x * x, items, [1.0] * 10, 0, 1) == [x * x for x in items]


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, ns, outq):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        work = np.asarray(ns, dtype=float) ** 3
        # the "solve" of system i: a deterministic function of (i, n_i)
        res = shard.sharded_map(lambda t: (t[0], int(t[1]) * 7 + t[0] % 3), list(enumerate(ns)),
                                work, rank, world)
        lo, hi = shard.shard(ns, rank, world)
        outq.put((rank, res, (lo, hi)))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_rank_gloo_sharded_map_matches_one_process():
    import torch.multiprocessing as mp
    ns = list(np.random.default_rng(1).integers(8, 257, 301))
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, ns, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    expect = [(i, int(n) * 7 + i % 3) for i, n in enumerate(ns)]
    got.sort()
    assert got[0][1] == expect and got[1][1] == expect       # every rank has all results
    (lo0, hi0), (lo1, hi1) = got[0][2], got[1][2]
    assert lo0 == 0 and hi0 == lo1 and hi1 == len(ns) and 0 < hi0 < len(ns)
