"""Dose-serving loop: continuous batching of transport jobs on one GPU.

DXMClib runs one ``Transport<T>::operator()`` call at a time
(``transport.hpp:135-202``): every call validates the world, builds the LUT,
transports and post-processes, and nothing stays on a device between calls.
This module adds the serving layer around the same transport:

* requests (world, source, model, seed, output mode) arrive from any thread;
  ``submit`` prepares the source tables on the caller's thread and returns a
  future;
* one scheduler thread admits requests in arrival order while their device
  memory (tallies, source tables and, when the world is not resident yet, the
  world itself) fits the context's budget, evicting idle resident worlds
  least-recently-used first;
* worlds and LUTs stay resident on the device and are shared by the jobs that
  use them (keyed by the caller's ``world_key``, default: the World object);
* every pass of the loop launches whatever has been admitted as one batch in the
  concurrent mode of ``dxmc_gpu_batch_submit``: the jobs queue behind the work
  already on the context's chains, so requests that arrive while others run are
  on the GPU as soon as memory and a chain free up (continuous batching);
* finished jobs are collected by a collector thread in groups: each job's
  post-processing and copies into page-locked buffers from a pool are queued
  behind it on the result stream (asynchronous results), then the group is
  waited for, so that results stream back over the link without a host round
  trip per job; each job's device memory is released once its copies are done,
  and the latency from arrival to result is recorded for p50 / p99.

The device side is behind a small backend interface so that the scheduling
logic (admission, eviction, ordering, metrics) is tested on the CPU with a
simulated backend.
"""
from __future__ import annotations

import collections
import ctypes as C
import math
import queue
import threading
import time
from concurrent.futures import Future
from dataclasses import dataclass, field
from typing import Any, Dict, Hashable, List, Optional

import numpy as np

from . import _capi as A

GIB = 1 << 30


@dataclass
class ServeRequest:
    world: Any
    source: Any
    model: int
    seed: int
    output_mode: int
    calibration: float
    world_key: Hashable
    histories: int
    exposures: Any = None
    spectrum: Any = None
    heel: Any = None
    bowtie: Any = None
    max_energy: float = 0.0
    arrival: float = 0.0
    admitted: float = 0.0
    future: Future = field(default_factory=Future)


@dataclass
class ServedResult:
    """Result of one served job: ``dose``/``variance`` (float64, or float32 for a
    server made with ``result_dtype=np.float32``: Result<float>) and ``nEvents``
    (uint32) per voxel, in the output mode of the request.  The arrays live in
    page-locked buffers of the server's pool: call ``release()`` to hand them
    back once consumed (they are freed when the result is garbage otherwise)."""
    dose: np.ndarray
    variance: np.ndarray
    nEvents: Optional[np.ndarray]
    numberOfHistories: int
    latency_s: float
    queue_s: float
    stats: dict
    _buffers: list = field(default_factory=list, repr=False)
    arrival: float = 0.0   # perf_counter() at submit
    admitted: float = 0.0  # perf_counter() at admission

    def release(self):
        for b in self._buffers:
            b.give_back()
        self._buffers = []
        self.dose = self.variance = self.nEvents = None


class _Pinned:
    """One page-locked host buffer (dxmc_gpu_host_alloc)."""

    def __init__(self, pool: "_PinnedPool", nbytes: int):
        self.pool, self.nbytes = pool, nbytes
        self.ptr = C.c_void_p()
        A.check(pool.lib.dxmc_gpu_host_alloc(nbytes, C.byref(self.ptr)), None, "dxmc_gpu_host_alloc")

    def array(self, dtype, count: int) -> np.ndarray:
        buf = (C.c_char * self.nbytes).from_address(self.ptr.value)
        buf._owner = self  # the array keeps the page-locked memory alive
        return np.frombuffer(buf, dtype=dtype, count=count)

    def give_back(self):
        if self.pool is not None:
            self.pool.put(self)

    def free(self):
        if self.ptr:
            self.pool.lib.dxmc_gpu_host_free(self.ptr)
            self.ptr = C.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class _PinnedPool:
    """Page-locked buffers reused by size; at most ``keep_bytes`` kept idle.
    Page-locking costs milliseconds per hundred megabytes, so buffers are kept
    and reused: sizes are rounded up to 1/16 of their power of two (at most
    6 % waste), ``prewarm`` allocates the buffers a world's results need when
    the world becomes resident, and a background thread allocates another
    buffer of a size whenever a ``get`` leaves none of it idle, so that results
    held by clients do not make the collector page-lock memory itself."""

    def __init__(self, lib, keep_bytes: int = 32 * GIB, spares: int = 2):
        self.lib = lib
        self.keep_bytes = keep_bytes
        self.spares = spares
        self.free_lists: Dict[int, List[_Pinned]] = collections.defaultdict(list)
        self.idle = 0
        self.pending: Dict[int, int] = collections.defaultdict(int)  # refills queued per size
        self.lock = threading.Lock()
        self._refills: "queue.Queue[Optional[int]]" = queue.Queue()
        self._refiller = threading.Thread(target=self._refill_loop, name="dxmc-pinned-refill", daemon=True)
        self._refiller.start()

    def _refill_loop(self):
        while True:
            size = self._refills.get()
            if size is None:
                return
            with self.lock:
                self.pending[size] -= 1
                if self.idle + size > self.keep_bytes:
                    continue
            try:
                self.put(_Pinned(self, size))
            except Exception:  # out of page-locked memory: the collector allocates on demand
                pass

    def _request_refill(self, size: int):
        # caller holds the lock
        while len(self.free_lists.get(size, [])) + self.pending[size] < self.spares:
            self.pending[size] += 1
            self._refills.put(size)

    @staticmethod
    def _size(nbytes: int) -> int:
        nbytes = max(4096, int(nbytes))
        step = max(4096, (1 << (nbytes - 1).bit_length()) >> 4)
        return (nbytes + step - 1) // step * step

    def prewarm(self, nbytes: int, count: int):
        """Makes sure ``count`` idle buffers of ``nbytes`` exist (within keep_bytes)."""
        size = self._size(nbytes)
        with self.lock:
            have = len(self.free_lists.get(size, []))
        for _ in range(max(0, count - have)):
            with self.lock:
                if self.idle + size > self.keep_bytes:
                    return
            self.put(_Pinned(self, size))

    def get(self, nbytes: int) -> _Pinned:
        size = self._size(nbytes)
        with self.lock:
            lst = self.free_lists.get(size)
            buf = None
            if lst:
                self.idle -= size
                buf = lst.pop()
            self._request_refill(size)
        return buf if buf is not None else _Pinned(self, size)

    def put(self, b: _Pinned):
        with self.lock:
            if self.idle + b.nbytes <= self.keep_bytes:
                self.free_lists[b.nbytes].append(b)
                self.idle += b.nbytes
                return
        b.free()

    def close(self):
        self._refills.put(None)
        self._refiller.join()
        with self.lock:
            for lst in self.free_lists.values():
                for b in lst:
                    b.free()
            self.free_lists.clear()
            self.idle = 0


# ---- backends ---------------------------------------------------------------------------

class GpuBackend:
    """Device side of the server: the C ABI through dxmclib_gb300.api."""

    def __init__(self, ctx, chains: int = 4, want_events: bool = True, result_dtype=np.float64):
        from . import api
        self.api = api
        self.ctx = ctx
        self.chains = chains
        self.want_events = want_events
        self.result_dtype = np.dtype(result_dtype)
        self.pool = _PinnedPool(ctx.lib)
        self.luts: "collections.OrderedDict[Hashable, Any]" = collections.OrderedDict()
        self.max_luts = 256
        # the chains' photon-queue buffers (allocated by the first batch, only when the context
        # pre-generates photons) are kept out of admission
        log2 = getattr(ctx, "options", {}).get("queue_log2_chunk", 0)
        self.chain_reserve = chains * 48 * (1 << log2) if log2 > 0 else 0

    def memory(self):
        return self.ctx.memory()

    def world_bytes(self, world) -> int:
        return int(world.size()) * 9  # 8-byte voxels + the 1-byte palette layout

    def job_bytes(self, req: ServeRequest) -> int:
        n = int(req.world.size())
        # one 32-byte FP64 tally record per voxel, the job's tables and counters
        return n * 32 + 80 * len(req.exposures) + (1 << 20)

    def result_bytes(self, n: int):
        e = self.result_dtype.itemsize
        return [n * e, n * e] + ([n * 4] if self.want_events else [])

    def upload_world(self, world):
        dw = self.api.DeviceWorld(self.ctx, world)
        # page-lock the result buffers of two jobs on this world ahead of their results
        for nbytes in self.result_bytes(int(world.size())):
            self.pool.prewarm(nbytes, 2)
        return dw, dw.max_density()

    def free_world(self, handle):
        handle[0].close()

    def lut(self, world_handle, req: ServeRequest):
        """Resident LUT for the world's materials, maximum densities and the source's
        maximum energy (the table depends on nothing else)."""
        dw, max_density = world_handle
        mats = req.world.materialMap()
        key = (tuple((m.name(), m.standardDensity()) for m in mats), tuple(float(d) for d in max_density),
               float(req.max_energy))
        dl = self.luts.get(key)
        if dl is None or not dl.handle:
            blob = self.api.LutBlob.cached(mats, max_density, req.max_energy)
            dl = self.api.DeviceLut(self.ctx, blob)
            dl._blob = blob
            self.luts[key] = dl
            if len(self.luts) > self.max_luts:
                # queued jobs hold the device image alive until they finish: the free waits for them
                self.luts.popitem(last=False)[1].close()
        self.luts.move_to_end(key)
        return dl

    def submit(self, items):
        """items: list of (req, world_handle, lut); returns (batch, jobs)."""
        entries = [self.api.BatchEntry(wh[0], lut, r.exposures, r.spectrum, r.heel, r.bowtie, r.seed, r.model, -1)
                   for r, wh, lut in items]
        batch = self.api.Batch(self.ctx, entries, mode=A.BATCH_CONCURRENT, chains=self.chains)
        return batch, list(batch.jobs)

    def done(self, job) -> bool:
        rc = job.wait(0)
        if rc == A.DXMC_OK:
            return True
        if rc == A.DXMC_ERR_TIMEOUT:
            return False
        A.check(rc, self.ctx.handle, "dxmc_gpu_job_wait")
        return True

    def collect_begin(self, job, req: ServeRequest):
        """Queues the job's post-processing and result copies behind it (asynchronous
        result into page-locked buffers of the pool); returns the buffers."""
        n = int(req.world.size())
        sizes = self.result_bytes(n)
        bufs = [self.pool.get(b) for b in sizes]
        dose = bufs[0].array(self.result_dtype, n)
        var = bufs[1].array(self.result_dtype, n)
        nev = bufs[2].array(np.uint32, n) if self.want_events else None
        job.result_async(req.output_mode, req.calibration, out=(dose, var, nev), dtype=self.result_dtype)
        return (dose, var, nev), bufs

    def collect_end(self, job, req: ServeRequest, arrays, bufs):
        """Waits for the result queued by collect_begin and releases the job's device memory."""
        *_, stats = job.result_wait()
        job.release()
        dose, var, nev = arrays
        return dose, var, nev, stats, bufs

    def collect(self, job, req: ServeRequest):
        arrays, bufs = self.collect_begin(job, req)
        return self.collect_end(job, req, arrays, bufs)

    def close_batch(self, batch):
        batch.close()

    def close(self):
        for dl in self.luts.values():
            dl.close()
        self.luts.clear()
        self.pool.close()


# ---- the server ---------------------------------------------------------------------------

@dataclass
class _WorldSlot:
    handle: Any
    bytes: int
    users: int = 0
    last_used: float = 0.0


class DoseServer:
    """Continuous-batching dose server on one GPU context.

    ``submit(world, source, ...)`` returns a ``concurrent.futures.Future`` that
    resolves to a ``ServedResult``.  ``metrics()`` reports the served jobs,
    histories, aggregate histories/s and the p50 / p99 latency."""

    def __init__(self, ctx=None, chains: int = 4, max_batch_jobs: int = 64, want_events: bool = True,
                 backend=None, reserve_bytes: Optional[int] = None, result_dtype=np.float64):
        if backend is None:
            if ctx is None:
                from .api import GpuContext
                ctx = GpuContext()
            backend = GpuBackend(ctx, chains, want_events, result_dtype)
        self.backend = backend
        self.max_batch_jobs = max_batch_jobs
        self.reserve = getattr(backend, "chain_reserve", 0) if reserve_bytes is None else reserve_bytes
        self.inbox: "queue.Queue[ServeRequest]" = queue.Queue()
        self.waiting: "collections.deque[ServeRequest]" = collections.deque()
        self.admitted: List[tuple] = []       # (req, world_handle, lut) not yet launched
        self.inflight: List[tuple] = []       # (req, job, batch_id)
        self.batches: Dict[int, list] = {}    # batch_id -> [batch, jobs left]
        self.worlds: "collections.OrderedDict[Hashable, _WorldSlot]" = collections.OrderedDict()
        self.latencies: List[float] = []
        self.queue_times: List[float] = []
        self.histories_done = 0
        self.jobs_done = 0
        self.batch_sizes: List[int] = []
        self.first_arrival: Optional[float] = None
        self.last_done: Optional[float] = None
        self.errors: List[BaseException] = []
        self._stop = False
        self._idle = threading.Event()
        self._idle.set()
        self._submitted = 0
        self._finished = 0
        self._lock = threading.Lock()
        self._next_batch = 0
        self.to_collect: "queue.Queue" = queue.Queue()
        self.completed: "queue.Queue" = queue.Queue()
        self._collecting = 0
        self.collector = threading.Thread(target=self._collector, name="dxmc-collect", daemon=True)
        self.collector.start()
        self.thread = threading.Thread(target=self._loop, name="dxmc-serve", daemon=True)
        self.thread.start()

    # -- client side --------------------------------------------------------------------
    def submit(self, world, source, *, model: int = 1, seed: int = 1, output_mode: int = A.OUTPUT_EV_PER_HISTORY,
               calibration: float = 1.0, world_key: Optional[Hashable] = None) -> Future:
        source.updateFromWorld(world)
        source.validate()
        if not world.isValid() or not source.isValid():
            f = Future()
            f.set_exception(ValueError("invalid world or source"))
            return f
        exposures = source.exposures(world.directionCosines())
        req = ServeRequest(world=world, source=source, model=int(model), seed=int(seed), output_mode=int(output_mode),
                           calibration=float(calibration), world_key=world_key if world_key is not None else id(world),
                           histories=int(np.sum(exposures.n_histories)), exposures=exposures,
                           spectrum=source.spectrum(), heel=source.heel(), bowtie=source.bowtie(),
                           max_energy=float(source.maxPhotonEnergyProduced()))
        req.arrival = time.perf_counter()
        with self._lock:
            self._submitted += 1
            self._idle.clear()
            if self.first_arrival is None:
                self.first_arrival = req.arrival
        self.inbox.put(req)
        return req.future

    def drain(self, timeout: Optional[float] = None) -> bool:
        """Waits until every submitted request has finished."""
        return self._idle.wait(timeout)

    def close(self):
        self.drain()
        self._stop = True
        self.inbox.put(None)
        self.thread.join()
        self.to_collect.put(None)
        self.collector.join()
        for slot in self.worlds.values():
            self.backend.free_world(slot.handle)
        self.worlds.clear()
        self.backend.close()

    def reset_metrics(self):
        """Starts the latency / throughput record afresh (e.g. after a warm-up)."""
        self.drain()
        self.latencies.clear()
        self.queue_times.clear()
        self.histories_done = self.jobs_done = 0
        self.batch_sizes.clear()
        self.errors.clear()
        with self._lock:
            self.first_arrival = self.last_done = None

    def metrics(self) -> dict:
        with self._lock:
            lat = np.asarray(self.latencies) * 1e3
        span = (self.last_done - self.first_arrival) if self.jobs_done else 0.0
        return dict(jobs=self.jobs_done, histories=self.histories_done, span_s=span,
                    histories_per_s=self.histories_done / span if span > 0 else 0.0,
                    p50_ms=float(np.percentile(lat, 50)) if len(lat) else None,
                    p99_ms=float(np.percentile(lat, 99)) if len(lat) else None,
                    mean_ms=float(lat.mean()) if len(lat) else None,
                    mean_queue_ms=float(np.mean(self.queue_times) * 1e3) if self.queue_times else None,
                    batches=len(self.batch_sizes),
                    mean_batch_jobs=float(np.mean(self.batch_sizes)) if self.batch_sizes else 0.0,
                    resident_worlds=len(self.worlds), errors=len(self.errors))

    # -- scheduler ------------------------------------------------------------------------
    def _loop(self):
        idle_polls = 0
        while True:
            busy = bool(self.waiting or self.admitted or self.inflight or self._collecting)
            try:
                # block while there is nothing to do; poll while work is in flight
                req = self.inbox.get_nowait() if busy else self.inbox.get()
            except queue.Empty:
                req = False
            while req is not False:
                if req is None:
                    self._stop = True
                else:
                    self.waiting.append(req)
                try:
                    req = self.inbox.get_nowait()
                except queue.Empty:
                    req = False
            progressed = self._collect()
            progressed |= self._admit()
            progressed |= self._launch()
            if self._stop and not (self.waiting or self.admitted or self.inflight or self._collecting):
                return
            if progressed:
                idle_polls = 0
            elif self.inflight or self.waiting or self._collecting:
                # poll the running jobs with a growing pause (50 us to 1 ms): a tight loop
                # of completion queries takes the interpreter from the collector thread
                time.sleep(min(5e-5 * (1 << min(idle_polls, 5)), 1e-3))
                idle_polls += 1

    def _fail(self, req: ServeRequest, exc: BaseException):
        self.errors.append(exc)
        req.future.set_exception(exc)
        self._finish_one()

    def _finish_one(self):
        with self._lock:
            self._finished += 1
            if self._finished == self._submitted:
                self._idle.set()

    def _free_bytes(self) -> int:
        budget, in_use = self.backend.memory()
        # admitted jobs allocate their tallies when their batch is submitted
        pending = sum(self.backend.job_bytes(r) for r, _, _ in self.admitted)
        return budget - in_use - self.reserve - pending

    def _evict_for(self, need: int, keep: Hashable) -> int:
        free = self._free_bytes()
        for key in list(self.worlds.keys()):  # least recently used first
            if free >= need:
                break
            slot = self.worlds[key]
            if slot.users == 0 and key != keep:
                self.backend.free_world(slot.handle)
                del self.worlds[key]
                free = self._free_bytes()
        return free

    def _admit(self) -> bool:
        progressed = False
        while self.waiting:
            req = self.waiting[0]
            slot = self.worlds.get(req.world_key)
            need = self.backend.job_bytes(req) + (0 if slot else self.backend.world_bytes(req.world))
            free = self._free_bytes()
            if free < need:
                free = self._evict_for(need, req.world_key)
            if free < need:
                if not (self.inflight or self.admitted):
                    self.waiting.popleft()
                    self._fail(req, A.DxmcError(A.DXMC_ERR_OOM, "request does not fit the device memory budget"))
                    progressed = True
                    continue
                break  # arrival order: wait for memory to free up
            self.waiting.popleft()
            try:
                if slot is None:
                    handle = self.backend.upload_world(req.world)
                    slot = _WorldSlot(handle, self.backend.world_bytes(req.world))
                    self.worlds[req.world_key] = slot
                lut = self.backend.lut(slot.handle, req)
            except Exception as exc:  # noqa: BLE001 - reported through the future
                self._fail(req, exc)
                progressed = True
                continue
            slot.users += 1
            slot.last_used = time.perf_counter()
            self.worlds.move_to_end(req.world_key)
            req.admitted = slot.last_used
            self.admitted.append((req, slot.handle, lut))
            progressed = True
        return progressed

    def _launch(self) -> bool:
        if not self.admitted:
            return False
        items, self.admitted = self.admitted[: self.max_batch_jobs], self.admitted[self.max_batch_jobs:]
        try:
            batch, jobs = self.backend.submit(items)
        except Exception as exc:  # noqa: BLE001
            if isinstance(exc, A.DxmcError) and exc.status == A.DXMC_ERR_OOM and self.inflight:
                self.admitted = items + self.admitted  # retry once memory frees up
                return False
            for req, _, _ in items:
                self._release_world(req)
                self._fail(req, exc)
            return True
        bid = self._next_batch
        self._next_batch += 1
        self.batches[bid] = [batch, len(jobs)]
        self.batch_sizes.append(len(jobs))
        for (req, _, _), job in zip(items, jobs):
            self.inflight.append((req, job, bid))
        return True

    def _release_world(self, req: ServeRequest):
        slot = self.worlds.get(req.world_key)
        if slot is not None:
            slot.users -= 1
            slot.last_used = time.perf_counter()

    def _collect(self) -> bool:
        """Scheduler side: hands finished jobs to the collector thread and books the
        ones it has finished (world users, batch retirement)."""
        progressed = False
        while True:
            try:
                req, bid = self.completed.get_nowait()
            except queue.Empty:
                break
            self._release_world(req)
            self._retire(bid)
            self._collecting -= 1
            progressed = True
        still = []
        for req, job, bid in self.inflight:
            try:
                finished = self.backend.done(job)
            except Exception as exc:  # noqa: BLE001
                self._release_world(req)
                self._fail(req, exc)
                self._retire(bid)
                progressed = True
                continue
            if not finished:
                still.append((req, job, bid))
                continue
            self._collecting += 1
            self.to_collect.put((req, job, bid))
            progressed = True
        self.inflight = still
        return progressed

    def _collector(self):
        """Collector thread: post-processing and result copies of finished jobs (the
        copies of a large grid take milliseconds; the scheduler keeps admitting and
        launching meanwhile).  Jobs that finished together are collected as a group:
        all their asynchronous results are queued first, then waited for in order."""
        staged = hasattr(self.backend, "collect_begin")
        stop = False
        while not stop:
            group = [self.to_collect.get()]
            while len(group) < 64:
                try:
                    group.append(self.to_collect.get_nowait())
                except queue.Empty:
                    break
            if any(item is None for item in group):
                stop = True
                group = [item for item in group if item is not None]
            pending = []
            for req, job, bid in group:
                try:
                    pending.append((req, job, bid, self.backend.collect_begin(job, req) if staged else None))
                except Exception as exc:  # noqa: BLE001
                    self._fail(req, exc)
                    self.completed.put((req, bid))
            for req, job, bid, begun in pending:
                try:
                    if staged:
                        dose, var, nev, stats, bufs = self.backend.collect_end(job, req, *begun)
                    else:
                        dose, var, nev, stats, bufs = self.backend.collect(job, req)
                except Exception as exc:  # noqa: BLE001
                    self._fail(req, exc)
                    self.completed.put((req, bid))
                    continue
                now = time.perf_counter()
                res = ServedResult(dose, var, nev, req.histories, now - req.arrival, req.admitted - req.arrival, stats,
                                   bufs, req.arrival, req.admitted)
                with self._lock:
                    self.latencies.append(now - req.arrival)
                    self.queue_times.append(req.admitted - req.arrival)
                    self.histories_done += req.histories
                    self.jobs_done += 1
                    self.last_done = now
                self.completed.put((req, bid))
                req.future.set_result(res)
                self._finish_one()

    def _retire(self, bid: int):
        entry = self.batches.get(bid)
        if entry is None:
            return
        entry[1] -= 1
        if entry[1] == 0:
            self.backend.close_batch(entry[0])
            del self.batches[bid]


def percentile_ms(latencies_s, q: float) -> float:
    return float(np.percentile(np.asarray(latencies_s) * 1e3, q))


def poisson_arrivals(rate_per_s: float, n: int, seed: int) -> np.ndarray:
    """Arrival times (s from the start) of a Poisson process."""
    rng = np.random.default_rng(seed)
    return np.cumsum(rng.exponential(1.0 / rate_per_s, n)) if rate_per_s > 0 else np.zeros(n)


def log_uniform(rng, lo: float, hi: float) -> int:
    return int(math.exp(rng.uniform(math.log(lo), math.log(hi))))
