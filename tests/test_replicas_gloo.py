"""The multi-GPU form is replicas only: every rank runs its own scenario and
the job's time is the slowest rank's.  The aggregation is tested with two
gloo ranks on the CPU (no GPU, no data-path collective)."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = 100.0 + 50.0 * rank                  # rank 1 is the slower replica
        m = bench.max_over_ranks(ms, dist)
        out[rank] = (m, bench.replica_value(1000, 10, m, world))
    finally:
        dist.destroy_process_group()


def test_two_replicas_take_the_slowest_rank():
    world = 2
    port = _free_port()
    with mp.Manager() as mgr:
        out = mgr.dict()
        ctx = mp.get_context("spawn")
        procs = [ctx.Process(target=_rank, args=(r, world, port, out)) for r in range(world)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        res = dict(out)
    assert res[0][0] == res[1][0] == 150.0
    assert res[0][1] == pytest.approx(2 * 1000 * 10 / 0.150)


def test_single_process_needs_no_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(12.5, None) == 12.5
    assert bench.replica_value(4, 5, 1000.0, 1) == 20.0
