"""The multi-rank path on CPU: queries dealt round-robin to ranks (gloo,
world size 2), each rank counting its share with the CPU oracle, the total and
the max-over-ranks time reduced across ranks as bench.py does on GPUs."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from clustersm_gb300.workloads import shard


def free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def worker(rank, world, port, out):
    import torch
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import oracle
    from clustersm_gb300.workloads import load
    wl = load("er1k")
    qs, want, _ = wl.queries()
    host = wl.graph()
    mine = shard(len(qs), rank, world)
    local = sum(oracle.count(host, qs[i], threads=1) for i in mine)
    t = torch.tensor([local, len(mine)], dtype=torch.int64)
    dist.all_reduce(t)
    mx = torch.tensor([float(rank + 1)])
    dist.all_reduce(mx, op=dist.ReduceOp.MAX)
    out[rank] = (int(t[0]), int(t[1]), float(mx[0]), sum(want))
    dist.destroy_process_group()


def test_shard_partitions():
    for n in (0, 1, 7, 96):
        for w in (1, 2, 3, 8):
            got = sorted(i for r in range(w) for i in shard(n, r, w))
            assert got == list(range(n))
    with pytest.raises(ValueError):
        shard(5, 2, 2)


def test_two_ranks_gloo():
    ctx = mp.get_context("spawn")
    out = ctx.Manager().dict()
    port = free_port()
    procs = [ctx.Process(target=worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=180)
        assert p.exitcode == 0
    for r in range(2):
        total, nq, mx, want = out[r]
        assert total == want and nq == 96 and mx == 2.0
