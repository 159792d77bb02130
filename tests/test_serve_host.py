"""CPU tests of the serving loop's host logic (dxmclib_gb300/serve.py) on a
simulated device backend: admission by the memory budget in arrival order,
resident-world reuse and least-recently-used eviction, requests that can never
fit, continuous batching of late arrivals, and the latency metrics."""
from __future__ import annotations

import threading
import time

import numpy as np
import pytest

from dxmclib_gb300 import _capi as A
from dxmclib_gb300.serve import DoseServer, poisson_arrivals


class FakeWorld:
    def __init__(self, n):
        self.n = n

    def size(self):
        return self.n

    def isValid(self):
        return True

    def directionCosines(self):
        return (1, 0, 0, 0, 1, 0)

    def materialMap(self):
        return []


class FakeExposures:
    def __init__(self, h):
        self.n_histories = np.array([h])

    def __len__(self):
        return 1


class FakeSource:
    def __init__(self, h):
        self.h = h

    def updateFromWorld(self, w):
        pass

    def validate(self):
        pass

    def isValid(self):
        return True

    def exposures(self, cos=None):
        return FakeExposures(self.h)

    def spectrum(self):
        return None

    def heel(self):
        return None

    def bowtie(self):
        return None

    def maxPhotonEnergyProduced(self):
        return 60.0


class FakeJob:
    def __init__(self, req, t_end, nbytes):
        self.req, self.t_end, self.nbytes = req, t_end, nbytes


class FakeBackend:
    """Jobs finish after histories / rate seconds; chains run jobs back to back."""

    def __init__(self, budget, rate=1e9, chains=2):
        self.budget, self.in_use = budget, 0
        self.rate, self.chains = rate, chains
        self.chain_free = [0.0] * chains
        self.uploads, self.frees = [], []
        self.max_inflight = 0
        self.inflight = 0
        self.batches = []
        self.lock = threading.Lock()

    def memory(self):
        return self.budget, self.in_use

    def world_bytes(self, world):
        return world.n

    def job_bytes(self, req):
        return req.world.n // 2

    def upload_world(self, world):
        self.in_use += world.n
        self.uploads.append(world)
        return world

    def free_world(self, handle):
        self.in_use -= handle.n
        self.frees.append(handle)

    def lut(self, wh, req):
        return "lut"

    def submit(self, items):
        now = time.perf_counter()
        jobs = []
        for req, wh, lut in items:
            nbytes = self.job_bytes(req)
            if self.in_use + nbytes > self.budget:
                raise A.DxmcError(A.DXMC_ERR_OOM, "over budget")
            self.in_use += nbytes
            c = int(np.argmin(self.chain_free))
            start = max(now, self.chain_free[c])
            self.chain_free[c] = start + req.histories / self.rate
            jobs.append(FakeJob(req, self.chain_free[c], nbytes))
        self.inflight += len(jobs)
        self.max_inflight = max(self.max_inflight, self.inflight)
        self.batches.append(len(jobs))
        return object(), jobs

    def done(self, job):
        return time.perf_counter() >= job.t_end

    def collect(self, job, req):
        self.in_use -= job.nbytes
        self.inflight -= 1
        n = req.world.n
        return np.full(4, req.seed, float), np.zeros(4), None, {"histories": req.histories}, []

    def close_batch(self, b):
        pass

    def close(self):
        pass


def test_all_requests_complete_with_metrics():
    be = FakeBackend(budget=10_000)
    srv = DoseServer(backend=be, reserve_bytes=0)
    worlds = [FakeWorld(1000), FakeWorld(2000)]
    futs = [srv.submit(worlds[i % 2], FakeSource(1_000_000 * (1 + i % 3)), seed=i, world_key=i % 2) for i in range(20)]
    assert srv.drain(timeout=30)
    res = [f.result() for f in futs]
    assert [int(r.dose[0]) for r in res] == list(range(20))  # each future gets its own job's result
    m = srv.metrics()
    assert m["jobs"] == 20 and m["errors"] == 0
    assert m["histories"] == sum(1_000_000 * (1 + i % 3) for i in range(20))
    assert 0 < m["p50_ms"] <= m["p99_ms"]
    assert m["histories_per_s"] > 0
    assert len(be.uploads) == 2  # resident worlds are uploaded once
    srv.close()
    assert be.in_use == 0  # worlds freed at close, job memory released after each result


def test_admission_respects_budget_in_arrival_order():
    # the world (4000) stays resident; each job needs 2000: at most 3 jobs fit in 10000
    be = FakeBackend(budget=10_000, rate=2e8)
    srv = DoseServer(backend=be, reserve_bytes=0)
    w = FakeWorld(4000)
    futs = [srv.submit(w, FakeSource(2_000_000), seed=i, world_key="w") for i in range(12)]
    assert srv.drain(timeout=30)
    res = [f.result() for f in futs]
    assert be.max_inflight <= 3
    admitted = [r.admitted for r in res]
    assert admitted == sorted(admitted)  # admission follows arrival order
    assert max(r.queue_s for r in res) > 0.005  # later requests waited for memory
    srv.close()


def test_lru_eviction_of_idle_worlds():
    # budget holds two 4000-voxel worlds plus one job (2000)
    be = FakeBackend(budget=10_500, rate=1e10)
    srv = DoseServer(backend=be, reserve_bytes=0)
    a, b, c = FakeWorld(4000), FakeWorld(4000), FakeWorld(4000)
    for w, key in [(a, "a"), (b, "b"), (a, "a"), (c, "c")]:
        srv.submit(w, FakeSource(1000), world_key=key).result(timeout=30)
    # "b" was least recently used when "c" needed room
    assert be.frees == [b]
    assert set(srv.worlds.keys()) == {"a", "c"}
    srv.submit(b, FakeSource(1000), world_key="b").result(timeout=30)
    assert be.uploads.count(b) == 2
    srv.close()


def test_request_larger_than_budget_fails_cleanly():
    be = FakeBackend(budget=5_000)
    srv = DoseServer(backend=be, reserve_bytes=0)
    f = srv.submit(FakeWorld(10_000), FakeSource(1000), world_key="big")
    with pytest.raises(A.DxmcError):
        f.result(timeout=30)
    ok = srv.submit(FakeWorld(1000), FakeSource(1000), world_key="small").result(timeout=30)
    assert ok.numberOfHistories == 1000
    assert srv.metrics()["errors"] == 1
    srv.close()


def test_late_arrivals_join_while_others_run():
    # a long job is on the GPU when short ones arrive: they run on the other chain and finish first
    be = FakeBackend(budget=1 << 40, rate=1e8, chains=2)
    srv = DoseServer(backend=be, reserve_bytes=0)
    w = FakeWorld(100)
    long_f = srv.submit(w, FakeSource(50_000_000), world_key="w")  # 0.5 s
    time.sleep(0.05)
    short = [srv.submit(w, FakeSource(1_000_000), world_key="w") for _ in range(3)]  # 10 ms each
    for f in short:
        r = f.result(timeout=30)
        assert not long_f.done()
        assert r.latency_s < 0.3
    assert long_f.result(timeout=30).latency_s >= 0.45
    assert len(be.batches) >= 2  # the late requests were launched as their own batch
    srv.close()


def test_poisson_arrivals():
    t = poisson_arrivals(100.0, 20000, seed=3)
    assert np.all(np.diff(t) >= 0)
    assert abs(t[-1] / 20000 - 0.01) < 0.0005


class FakeHostLib:
    """dxmc_gpu_host_alloc / _free over ordinary host memory, counting calls."""

    def __init__(self):
        import ctypes as C
        self.C = C
        self.live = {}
        self.allocs = 0
        self.lock = threading.Lock()

    def dxmc_gpu_host_alloc(self, nbytes, out):
        buf = self.C.create_string_buffer(int(nbytes))
        with self.lock:
            self.allocs += 1
            self.live[self.C.addressof(buf)] = buf
        out._obj.value = self.C.addressof(buf)
        return 0

    def dxmc_gpu_host_free(self, ptr):
        with self.lock:
            self.live.pop(ptr.value, None)


def test_pinned_pool_refills_in_the_background():
    """A get that leaves a size without idle buffers makes the background thread
    allocate spares, so that the next gets of that size reuse page-locked memory
    instead of allocating on the collector's thread; returned buffers are reused."""
    from dxmclib_gb300.serve import _PinnedPool
    lib = FakeHostLib()
    pool = _PinnedPool(lib, keep_bytes=1 << 30, spares=2)
    try:
        a = pool.get(100_000)
        assert lib.allocs == 1  # nothing idle yet: allocated on the spot
        deadline = time.time() + 5
        while lib.allocs < 3 and time.time() < deadline:
            time.sleep(0.01)
        assert lib.allocs == 3  # two spares of that size arrived
        size = pool._size(100_000)
        assert a.nbytes == size and len(pool.free_lists[size]) == 2
        b = pool.get(100_000)
        c = pool.get(100_000)
        assert lib.allocs >= 3 and b.nbytes == size and c.nbytes == size
        for buf in (a, b, c):
            buf.give_back()
        assert len(pool.free_lists[size]) >= 3
        d = pool.get(99_000)  # the same size class
        assert d.nbytes == size
    finally:
        pool.close()
    assert len(lib.live) == 1  # closing frees every idle buffer; d is still held


def test_pinned_pool_keeps_at_most_keep_bytes_idle():
    from dxmclib_gb300.serve import _PinnedPool
    lib = FakeHostLib()
    pool = _PinnedPool(lib, keep_bytes=300_000, spares=0)
    try:
        bufs = [pool.get(100_000) for _ in range(5)]
        size = bufs[0].nbytes
        for b in bufs:
            b.give_back()
        assert pool.idle <= 300_000 and pool.idle == size * len(pool.free_lists[size])
    finally:
        pool.close()
