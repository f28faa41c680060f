"""Multi-GPU is replicas only: each rank runs the whole workload and the
job time is the max over ranks.  The reduction runs here on CPU ranks over
gloo (world size 2)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms = bench.replica_time(10.0 + 5.0 * rank, dist, "cpu")
    out[rank] = ms
    dist.destroy_process_group()


def test_replica_time_is_max_over_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    assert out[0] == 15.0 and out[1] == 15.0


def test_replica_time_single_process():
    import bench
    assert bench.replica_time(7.5) == 7.5
