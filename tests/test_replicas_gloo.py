"""The replica throughput reduction with two gloo ranks on CPU."""
import os

import pytest
import torch.multiprocessing as mp


def _worker(rank, world, port, q):
    import torch.distributed as dist

    from astronomix_gb300.replicas import replica_throughput

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    # rank 0: 100 units in 2 s, rank 1: 300 units in 4 s -> 400 / 4
    v = replica_throughput(100.0 if rank == 0 else 300.0, 2.0 if rank == 0 else 4.0)
    q.put((rank, v))
    dist.destroy_process_group()


def test_replica_throughput_two_ranks():
    import socket

    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = dict(q.get(timeout=10) for _ in range(2))
    assert res[0] == pytest.approx(100.0) and res[1] == pytest.approx(100.0)


def test_replica_throughput_single_process():
    from astronomix_gb300.replicas import replica_throughput

    assert replica_throughput(10.0, 2.0) == pytest.approx(5.0)
