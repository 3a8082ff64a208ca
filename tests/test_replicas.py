"""Replica runs of the bench (one process per GPU, no data-path
collective): the whole-job throughput is every rank's units over the
slowest rank's time.  Checked with two gloo ranks on the CPU."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, seconds, q):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, w, local = bench.dist_env()
        value, slowest = bench.replica_throughput(1000, seconds[rank], w, "cpu")
        q.put((r, w, local, value, slowest))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("seconds", [(1.0, 2.0), (4.0, 0.5)])
def test_two_replicas_use_the_slowest_rank(seconds):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, seconds, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    slowest = max(seconds)
    for r, (rank, world, local, value, s) in enumerate(got):
        assert (rank, world, local) == (r, 2, r)
        assert s == slowest
        assert value == pytest.approx(2 * 1000 / slowest)


def test_single_process_needs_no_group():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.replica_throughput(500, 2.0, 1) == (250.0, 2.0)
