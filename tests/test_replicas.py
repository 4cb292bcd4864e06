"""Multi-GPU runs are replicas only: each rank advances its own copy of the workload and the
whole-job rate is (particles of all ranks x steps) / (slowest rank's time), with no collective on
the data path.  The aggregation is exercised here with two gloo ranks on the CPU."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    import torch.distributed as dist
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms_local = 10.0 if rank == 0 else 25.0
    n_local = 1000 + rank
    ms, value = bench.aggregate(ms_local, n_local, steps=4, dist=dist, device="cpu")
    out[rank] = (ms, value)
    dist.barrier()
    dist.destroy_process_group()


def test_replica_aggregation_gloo():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    mgr = mp.Manager()
    out = mgr.dict()
    port = _free_port()
    mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
    for rank in (0, 1):
        ms, value = out[rank]
        assert ms == 25.0                      # the slowest rank
        assert value == pytest.approx((1000 + 1001) * 4 / 25e-3)


def test_single_rank_aggregation():
    import bench
    ms, value = bench.aggregate(8.0, 500, steps=2)
    assert ms == 8.0 and value == pytest.approx(500 * 2 / 8e-3)
