"""bench.py's N > 1 path (independent replicas, max-over-ranks timing) on two
gloo ranks on the CPU."""

import os

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _worker(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    ms = [120.0, 150.0][rank]
    slow = bench.max_over_ranks(ms, dist)
    dist.barrier()
    q.put((rank, slow, bench.replica_value(1780, slow, world)))
    dist.destroy_process_group()


def test_two_rank_max_and_value():
    import socket

    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, slow, value in out:
        assert slow == 150.0
        assert abs(value - 2 * 1780 / 0.150) < 1e-6
