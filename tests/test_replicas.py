"""The multi-rank bench path (one replica per GPU, no collective on the data
path): the timed region is the slowest rank's and the throughput counts every
rank's solves.  Run here as two gloo ranks on the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist
import torch.multiprocessing as tmp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        ms = 100.0 + 50.0 * rank               # rank 1 is the slow one
        slow = bench.slowest_rank_ms(ms, world, torch.device("cpu"))
        out[rank] = (slow, bench.replica_throughput(5, slow, world))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_report_the_slowest():
    world, port = 2, _free_port()
    with tmp.Manager() as m:
        out = m.dict()
        tmp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert res[0] == res[1]
    slow, value = res[0]
    assert slow == 150.0
    assert value == pytest.approx(2 * 5 / 0.150)


def test_single_rank_is_unchanged():
    import bench
    assert bench.slowest_rank_ms(42.0, 1, None) == 42.0
    assert bench.replica_throughput(3, 1500.0, 1) == pytest.approx(2.0)
