"""The N>1 bench path: replicas with no data exchange, job time = the slowest
rank's, value = all ranks' cell-updates / that time.  Two gloo ranks on CPU."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as tmp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def worker(rank, world, port, seconds, units, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import argparse
    import bench
    w, r, local, dist = bench.dist_setup(argparse.Namespace())
    assert (w, r, local) == (world, rank, rank)
    value, total = bench.replica_throughput(seconds[rank], units, w, dist)
    out[rank] = (value, total)
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_replica_throughput_takes_slowest_rank(world):
    ctx = tmp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    seconds = [1.0 + 0.5 * r for r in range(world)]
    units = 1_000_000
    tmp.start_processes(worker, args=(world, free_port(), seconds, units, out), nprocs=world, join=True,
                        start_method="spawn")
    expect_total = max(seconds)
    for r in range(world):
        value, total = out[r]
        assert total == expect_total
        assert value == pytest.approx(world * units / expect_total, rel=1e-15)


def test_single_rank_has_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    value, total = bench.replica_throughput(2.0, 100, 1, None)
    assert (value, total) == (50.0, 2.0)
