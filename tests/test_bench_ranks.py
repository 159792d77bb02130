"""CPU test of the multi-replica path of bench.py with two gloo ranks: every
rank runs an independent replica, the timed region is the slowest rank's, and
the reported throughput counts the histories of all ranks."""
from __future__ import annotations

import os
import socket
import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, str(REPO))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ws, r, local = bench._dist()
    seconds = 1.0 + r  # rank 1 is the slow replica
    slowest = bench.max_over_ranks(seconds, dist, device="cpu")
    value = bench.replica_throughput(ws, 1_000_000, 5, slowest)
    dist.barrier()
    dist.destroy_process_group()
    out.put((r, ws, slowest, value))


def test_two_replicas_take_the_slowest_rank():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r, ws, slowest, value in res:
        assert ws == 2 and slowest == 2.0
        assert value == pytest.approx(2 * 1_000_000 * 5 / 2.0)
