"""Multi-rank bench logic on the CPU with the gloo backend (world size 2):
each rank reports its own replica's time; the job's throughput uses the
slowest rank and counts every rank's nodes."""

import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    import sys
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    total_ms = [40.0, 55.0][rank]
    value, ms = bench.aggregate(total_ms, 128 ** 3, 10, world, dist, "cpu")
    q.put((rank, value, ms))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_throughput_uses_slowest_rank():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs)
    got = sorted(q.get(timeout=10) for _ in range(world))
    for rank, value, ms in got:
        assert ms == pytest.approx(5.5)
        assert value == pytest.approx(2 * 128 ** 3 / 5.5e-3 / 1e6)
