"""The N > 1 bench path: independent replicas, whole-job throughput from the
slowest rank (max over ranks), computed with a gloo process group on CPU."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms = 10.0 * (rank + 1)                     # rank 1 is the slow replica
    ms_max = bench.replica_time(ms, world, torch.device("cpu"))
    value = bench.replica_throughput(1000.0, world, ms_max)
    q.put((rank, ms_max, value))
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_gloo():
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
    for rank, ms_max, value in out:
        assert ms_max == pytest.approx(20.0)
        assert value == pytest.approx(2 * 1000.0 / 0.020)


def test_single_rank_is_identity():
    import bench
    assert bench.replica_time(3.5, 1) == 3.5
    assert bench.replica_throughput(10.0, 1, 1000.0) == pytest.approx(10.0)
