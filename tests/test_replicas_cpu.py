"""Multi-GPU is replicas only: every rank solves its own stream and the bench
takes the slowest rank's time and the sum of all ranks' work.  The aggregation
runs here with the gloo backend on two CPU ranks."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    total_ms, upd = bench.aggregate_replicas(torch, 10.0 * (rank + 1), 1000 * (rank + 1), world, "cpu")
    q.put((rank, total_ms, upd))
    dist.destroy_process_group()


def test_replica_aggregation_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    for _, total_ms, upd in got:
        assert total_ms == 20.0   # the slowest rank
        assert upd == 3000.0      # every rank's work


def test_single_rank_needs_no_collective():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.aggregate_replicas(torch, 5.0, 7, 1, "cpu") == (5.0, 7.0)
