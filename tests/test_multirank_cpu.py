"""The N > 1 path of bench.py on CPU: independent replicas, the timed region is
the slowest rank's (max over ranks), and the whole-job value counts every
replica's particles.  world_size 2 over gloo, rendezvous on 127.0.0.1."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms = 100.0 + 50.0 * rank  # rank 1 is the slow one
    got = bench.max_over_ranks(ms, device="cpu")
    out[rank] = (got, bench.replica_throughput(1000, world, 10, got))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_replicas_report_the_slowest_rank():
    world = 2
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert res[0][0] == res[1][0] == 150.0
    assert res[0][1] == pytest.approx(1000 * 2 * 10 / 0.150)


def test_single_process_is_its_own_max():
    import bench
    assert bench.max_over_ranks(12.5, device="cpu") == 12.5
