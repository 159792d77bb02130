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


def test_reference_arm_line():
    """bench.py --impl reference on a small sample: one JSON line with the base
    contract's keys, the CPU baseline's description (cores, share of them, sample)
    and e2e equal to the line's value; the process loads no product library."""
    import json
    import subprocess
    # run bench.py as __main__, then list the shared objects the process mapped
    code = ("import runpy, sys; sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '0', "
            "'--histories', '1e6']; runpy.run_path(sys.argv[0], run_name='__main__'); "
            "maps = open('/proc/self/maps').read(); "
            "print('MAPS', sorted({l.split()[-1] for l in maps.splitlines() if l.split()[-1].endswith('.so')}))")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600, cwd=str(REPO))
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [x for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1
    maps = [x for x in r.stdout.splitlines() if x.startswith("MAPS")]
    assert maps and "libdxmc_gpu" not in maps[0] and "liboracle_port" in maps[0], maps
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "config"):
        assert key in d, key
    assert d["impl"] == "reference" and d["higher_is_better"] is True and d["value"] > 0
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert len(cb["core_share"]) == 1 and 0.0 < cb["core_share"][0] < 1.5
    assert d["e2e"] == {"value": d["value"], "unit": "histories/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert d["config"]["workload"] == "ct_helical_512x512x200"
