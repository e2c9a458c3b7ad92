"""The multi-rank benchmark path (replicas only) on CPU with gloo, world
size 2: the job's time is the slowest rank's and its throughput counts every
rank's cells."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    sys.path.insert(0, ROOT)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms, val = bench.replica_throughput(10.0 + 5.0 * rank, 1000, 4, world, dist,
                                       torch.device("cpu"))
    dist.barrier()
    q.put((rank, ms, val))
    dist.destroy_process_group()


def test_replica_throughput_gloo_world2():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, val in out:
        assert ms == 15.0
        assert val == pytest.approx(1000 * 4 * 2 / 0.015 / 1e6)


def test_replica_throughput_single():
    sys.path.insert(0, ROOT)
    import bench
    ms, val = bench.replica_throughput(20.0, 500, 10, 1, None, None)
    assert ms == 20.0 and val == pytest.approx(500 * 10 / 0.02 / 1e6)
