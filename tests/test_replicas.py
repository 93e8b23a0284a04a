"""CPU: the multi-replica host logic of bench.py on two gloo ranks (one process per GPU in the
real run; the path has no exchange step, so the only collective is the max over rank times)."""
import os
import sys

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, ROOT)
    import bench
    times = [3.5, 2.25]
    out[rank] = (bench.max_over_ranks(times[rank], world, "cpu"), bench.replica_seed(rank))
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_take_the_slowest_time_and_their_own_frames():
    port = 29500 + os.getpid() % 1000
    with mp.Manager() as m:
        out = m.dict()
        mp.start_processes(_rank, args=(2, port, out), nprocs=2, start_method="spawn")
        res = dict(out)
    assert res[0][0] == 3.5 and res[1][0] == 3.5
    assert res[0][1] != res[1][1]


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(1.25, 1, "cpu") == 1.25
