"""The multi-rank bench logic on CPU with gloo, world size 2: each rank runs
an independent replica (distinct seeds), the job time is the slowest rank's,
and the rate counts every rank's work.  No GPU involved."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    t = [0.5, 2.0][rank]
    tmax = bench.max_over_ranks(t, world)
    bench.barrier(world)
    rate = bench.aggregate_rate(1000.0, world, tmax)
    q.put((rank, bench.replica_seed(rank), tmax, rate))
    dist.destroy_process_group()


def test_two_rank_replicas_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=5) for _ in range(2))
    assert [r[1] for r in res] == [1, 2]          # distinct replica seeds
    assert all(r[2] == 2.0 for r in res)          # slowest rank's time
    assert all(r[3] == pytest.approx(1000.0) for r in res)  # 2 x 1000 / 2.0
