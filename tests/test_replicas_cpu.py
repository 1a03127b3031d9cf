"""Multi-GPU on this path is replicas only: every rank runs its own
multiplies, and the only collective is the timing reduction.  Checked here
with two gloo ranks on CPU."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    sys.path.insert(0, ROOT)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    mine = [0.5, 0.8][rank]              # this rank's seconds per step
    slowest = bench.max_over_ranks(mine, world, device="cpu")
    val = bench.replica_throughput(8.796, world, slowest)
    q.put((rank, slowest, val))
    dist.destroy_process_group()


def test_replica_timing_two_gloo_ranks():
    import socket
    import torch.multiprocessing as mp
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
    for rank, slowest, val in out:
        assert slowest == 0.8
        assert val == pytest.approx(2 * 8.796 / 0.8)
