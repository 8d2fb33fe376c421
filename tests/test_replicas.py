"""Replica bookkeeping of bench.py under torch.distributed (gloo, world size 2, CPU):
the barrier around the timed region and the max of the per-rank times.  The path has
no data-path collective; each rank solves its own replica."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import bench

    dist = bench.replica_group(world)
    bench.replica_barrier(dist)
    out.put((rank, bench.replica_max(dist, 1.5 + rank)))
    bench.replica_barrier(dist)
    dist.destroy_process_group()


def test_replica_max_over_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == {0: 2.5, 1: 2.5}


def test_single_process_needs_no_group():
    import bench

    assert bench.replica_group(1) is None
    assert bench.replica_max(None, 3.0) == 3.0
