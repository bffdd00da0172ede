"""bench.py --gpus N runs N independent replicas (the single-rank path has no
exchange step).  The job's throughput is the summed work of all ranks over the
slowest rank's time; checked here with two gloo ranks on the CPU."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    import sys
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    seconds = [2.0, 3.0][rank]
    units = [100.0, 50.0][rank]
    out[rank] = bench.aggregate_over_ranks(seconds, units)
    dist.destroy_process_group()


def test_aggregate_over_two_gloo_ranks():
    world = 2
    out = mp.get_context("spawn").Manager().dict()
    mp.spawn(_rank, args=(world, _free_port(), out), nprocs=world, join=True)
    for r in range(world):
        t, u, thr = out[r]
        assert t == 3.0 and u == 150.0 and thr == pytest.approx(50.0)


def test_aggregate_single_process():
    import sys
    sys.path.insert(0, ROOT)
    import bench
    assert bench.aggregate_over_ranks(2.0, 10.0) == (2.0, 10.0, 5.0)
