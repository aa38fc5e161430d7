"""The multi-GPU path of bench.py is independent replicas: each rank runs
the whole workload and the job reports ranks * steps / (max time over
ranks). Checked here with two gloo ranks on the CPU."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    ms = [2.0, 3.5][rank]
    got = bench.max_over_ranks(ms, dist, "cpu")
    q.put((rank, got, bench.replica_throughput(world, got)))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_two_gloo_ranks():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [3.5, 3.5]
    assert abs(res[0][2] - 2 * 1e3 / 3.5) < 1e-9


def test_single_process_is_identity():
    import bench

    assert bench.max_over_ranks(4.25, None) == 4.25
    assert bench.replica_throughput(1, 2.0) == 500.0
