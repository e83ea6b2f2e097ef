"""Multi-rank host logic of the benchmark on CPU (gloo, world size 2).

The engine shards nothing inside a series: several GPUs run independent
replicas, and the only cross-rank step is the max of the per-rank times.
"""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import torch.distributed as dist

    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        m = bench.reduce_max(1.5 + rank)
        rate = bench.replica_rate(1000, 2, world, m)
        q.put((rank, m, rate))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_reduce_max_over_two_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    assert [r[1] for r in res] == [2.5, 2.5]
    assert res[0][2] == pytest.approx(1000 * 2 * 2 / 2.5)


def test_single_process_is_identity():
    import bench
    assert bench.reduce_max(3.25) == 3.25
