"""bench.py's multi-GPU mode runs independent replicas (the draw path does
not shard within a frame): the whole-job number is every rank's work over
the slowest rank's time. Checked here with two gloo ranks on the CPU."""
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


def _rank(rank, world, port, out):
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r took 10 * (r + 1) ms for 1000 * (r + 1) fragments
        rate, ms = bench.replica_throughput(10.0 * (rank + 1), 1000.0 * (rank + 1), world, "cpu")
        out[rank] = (rate, ms)
    finally:
        dist.destroy_process_group()


def test_replica_throughput_two_gloo_ranks():
    world = 2
    port = _free_port()
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    # slowest rank: 20 ms; all ranks: 3000 fragments
    for rank in range(world):
        rate, ms = res[rank]
        assert ms == pytest.approx(20.0)
        assert rate == pytest.approx(3000.0 / 0.020)


def test_replica_throughput_single_rank():
    import bench
    rate, ms = bench.replica_throughput(4.0, 800.0, 1, "cpu")
    assert ms == 4.0 and rate == pytest.approx(200000.0)
