"""Replica scaling host logic (world size 2, gloo, CPU).

The path does not shard within one impact (gravity couples every particle),
so N GPUs run N independent simulations; the job's throughput is all ranks'
particle-steps over the slowest rank's time.  This checks that reduction with
two real gloo ranks, uneven work and uneven times.
"""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import bench
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    units = [1_000_000 * 10, 750_000 * 10][rank]
    ms = [40.0, 55.0][rank]
    rate, slowest = bench.replica_rate(units, ms, dist, "cpu")
    out[rank] = (rate, slowest)
    dist.barrier()
    dist.destroy_process_group()


def test_replica_rate_two_gloo_ranks():
    port = _free_port()
    with mp.get_context("spawn").Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_rank_main, args=(2, port, out), nprocs=2, join=True)
        res = dict(out)
    expect = (1_000_000 * 10 + 750_000 * 10) / 0.055
    for r in (0, 1):
        rate, slowest = res[r]
        assert slowest == 55.0
        assert abs(rate - expect) < 1e-6 * expect


def test_replica_rate_single_process():
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    rate, ms = bench.replica_rate(5_000_000, 25.0)
    assert ms == 25.0 and abs(rate - 2.0e8) < 1.0
