"""Multi-process path on CPU (gloo, world size 2): each rank factors its own work-balanced slice
of one batch with no data-path collective; gathering the slices reproduces the single-process
result exactly, and the step time is the max over ranks."""
import os
import socket

import numpy as np
import torch.distributed as dist
import torch.multiprocessing as mp

from matflat_gb300.shard import lu_work, shard_bounds


def test_shard_bounds_cover_and_balance():
    rng = np.random.default_rng(0)
    n = rng.integers(8, 129, size=1000)
    for world in (1, 2, 3, 8):
        b = shard_bounds(lu_work(n), world)
        assert b[0][0] == 0 and b[-1][1] == len(n)
        assert all(b[i][1] == b[i + 1][0] for i in range(world - 1))
        w = [lu_work(n[s:e]).sum() for s, e in b]
        assert max(w) - min(w) <= 2 * lu_work(128)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    from oracle import oracle
    from matflat_gb300.shard import lu_work, shard_bounds
    import torch
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    rng = np.random.default_rng(42)
    n = rng.integers(1, 40, size=64).astype(np.int32)
    s, e = shard_bounds(lu_work(n), world)[rank]
    mats = [rng.standard_normal(int(k) * int(k)) for k in n]
    out = []
    for i in range(s, e):
        a = mats[i].copy()
        piv = np.zeros(n[i], np.int32)
        sign = oracle.lu(int(n[i]), int(n[i]), a, int(n[i]), piv)
        out.append((i, a, piv, sign))
    gathered = [None] * world
    dist.all_gather_object(gathered, out)
    t = torch.tensor([float(rank + 1)])
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    if rank == 0:
        flat = sorted([x for part in gathered for x in part], key=lambda r: r[0])
        ok = [r[0] for r in flat] == list(range(len(n)))
        for i, a, piv, sign in flat:
            ref = mats[i].copy()
            rp = np.zeros(n[i], np.int32)
            rs = oracle.lu(int(n[i]), int(n[i]), ref, int(n[i]), rp)
            ok = ok and np.array_equal(a.view(np.uint64), ref.view(np.uint64)) and \
                np.array_equal(piv, rp) and sign == rs
        q.put((ok, float(t.item())))
    dist.destroy_process_group()


def test_two_ranks_reproduce_single_process():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    ok, tmax = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
    assert ok
    assert tmax == 2.0
