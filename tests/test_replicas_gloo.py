"""The bench's N > 1 host logic (independent replicas, max-over-ranks time, whole-job
throughput) with two gloo ranks on the CPU."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, results):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = [1000.0, 1250.0][rank]   # the slower rank sets the job time
    got_ms, value = bench.replica_throughput(ms, world, steps=5, device="cpu")
    dist.barrier()
    results.put((rank, got_ms, value))
    dist.destroy_process_group()


def test_two_replicas_take_the_slowest_rank():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    sys.path.insert(0, ROOT)
    import bench
    for _, got_ms, value in out:
        assert got_ms == 1250.0
        assert abs(value - 2 * bench.LAYERS * 5 / 1.25) < 1e-9   # 2 replicas x 40 layers x 5 steps in 1.25 s
