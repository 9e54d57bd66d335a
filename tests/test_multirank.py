"""The multi-rank path of bench.py on CPU: ranks are independent replicas (one snapshot
each, no data-path collective); the job's time is the maximum over ranks."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    import torch.distributed as dist

    sys.path.insert(0, REPO)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    # each replica reports its own time; the job time is the slowest
    t = bench.max_over_ranks(1.0 + rank * 0.25)
    # replicas solve different snapshots: the workload seed follows the rank
    import argparse

    f = bench.workload(argparse.Namespace(n=12), rank)
    out[rank] = (t, float(f["ax"].sum()))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_take_the_max_and_differ_in_data():
    world = 2
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_worker, args=(world, _free_port(), out), nprocs=world, start_method="spawn", join=True)
    assert out[0][0] == out[1][0] == 1.25
    assert out[0][1] != out[1][1]


def test_single_process_identity():
    sys.path.insert(0, REPO)
    import bench

    assert bench.max_over_ranks(3.5) == 3.5
