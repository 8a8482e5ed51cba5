"""Replica (N > 1) logic of bench.py on CPU: two gloo ranks run the bench's
own process-group set-up, barrier and max-over-ranks timing reduction, and
the whole-job throughput is the replicas' sum paced by the slowest rank."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    sys.path.insert(0, ROOT)
    import argparse

    import bench

    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "WORLD_SIZE": str(world),
                       "RANK": str(rank), "LOCAL_RANK": str(rank)})
    w, r, _ = bench.dist_setup(argparse.Namespace(impl="reference"))  # the reference arm uses gloo
    assert (w, r) == (world, rank)
    bench.barrier(w)
    ms = 10.0 + 5.0 * rank  # rank 1 is the slow one
    m = bench.allmax(w, ms)
    out[rank] = (m, bench.replica_value(w, m))
    dist.destroy_process_group()


def test_two_gloo_ranks_reduce_to_the_slowest():
    world, port = 2, _free_port()
    with mp.get_context("spawn").Manager() as mgr:
        out = mgr.dict()
        mp.start_processes(_rank, args=(world, port, out), nprocs=world, start_method="spawn", join=True)
        res = dict(out)
    assert res[0] == res[1] == (15.0, 2 * 1000.0 / 15.0)


def test_single_rank_is_unchanged():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.allmax(1, 3.5) == 3.5
    assert bench.replica_value(1, 4.0) == 250.0
