"""Launch-parameter autotuner for the transport kernels.

The reference has nothing to tune (one std::thread per core,
``transport.hpp:745-778``).  The GPU transport has four launch parameters whose
best values depend on the job (grid size and layout, spectrum, correction
model):

* ``queue_log2_chunk`` -- histories per photon-generation pass (2^n), or -1 to
  generate photons inside the transport kernel;
* ``regen_threshold`` -- how many lanes of a warp must be idle before they are
  refilled together (the refill cadence);
* ``interact_threshold`` -- how many lanes must wait for an interaction before
  the per-type interaction passes run (the event-sorting cadence);
* ``blocks_per_sm`` -- resident blocks per SM (occupancy);
* ``block_size`` -- threads per block (128 or 256);
* ``woodcock_burst`` -- Woodcock steps a lane may take per loop iteration before
  the warp checks for refills and interactions again.

For a job class (correction model, grid size in factors of 8, number of
materials, maximum energy in 20 keV bins) the tuner times a sample of the job -- an even
subset of its exposures with the histories scaled to ``sample_histories`` --
under coordinate descent over those parameters, starting from the library
defaults, and keeps the fastest setting.  Results are cached per device in a
JSON file so that a class is tuned once; the measured gain over the defaults is
stored with it.  For batches it picks the number of concurrent chains the same
way, on the batch itself.
"""
from __future__ import annotations

import json
import math
import os
import threading
from dataclasses import replace
from pathlib import Path
from typing import Dict, List, Optional, Sequence

import numpy as np

from . import _capi as A

SPACE: Dict[str, List[int]] = {
    "queue_log2_chunk": [23, 25, 0],
    "regen_threshold": [4, 8, 12, 16],
    "interact_threshold": [4, 6, 8, 12],
    "blocks_per_sm": [2, 3, 4, 8],
    "woodcock_burst": [4, 8, 12],
    "block_size": [128, 256],
}
DEFAULTS = {"queue_log2_chunk": 0, "regen_threshold": 0, "interact_threshold": 0, "blocks_per_sm": 0,
            "woodcock_burst": 0, "block_size": 0}  # 0: the library's default
CHAINS = [1, 2, 3, 4, 6]


def job_class(world, model: int, max_energy: float) -> str:
    """Correction model, grid size in factors of 8 (2^3n voxels), material count and
    maximum energy in 20 keV bins."""
    n = int(world.size())
    return (f"m{int(model)}|v{int(round(math.log2(max(n, 1)) / 3))}|mat{len(world.materialMap())}"
            f"|e{int(max_energy // 20) * 20}")


def sample_exposures(exposures, target_histories: int, max_exposures: int = 64):
    """Even subset of the exposures with histories per exposure scaled so the
    sample holds about ``target_histories``."""
    n = len(exposures)
    idx = np.unique(np.linspace(0, n - 1, min(n, max_exposures)).round().astype(int))
    per = max(1, int(target_histories // len(idx)))
    sub = replace(exposures, position=exposures.position[idx], cosines=exposures.cosines[idx],
                  beam_direction=exposures.beam_direction[idx], collimation=exposures.collimation[idx],
                  weight=exposures.weight[idx], n_histories=np.full(len(idx), per, np.uint64),
                  mono_energy=exposures.mono_energy[idx])
    return sub


class Autotuner:
    def __init__(self, ctx, cache_file: Optional[str] = None, sample_histories: int = 4_000_000, repeats: int = 2,
                 rounds: int = 2):
        self.ctx = ctx
        self.sample_histories = int(sample_histories)
        self.repeats = int(repeats)
        self.rounds = int(rounds)
        self.cache_file = Path(cache_file) if cache_file else None
        self.cache: Dict[str, dict] = {}
        self.lock = threading.Lock()
        if self.cache_file and self.cache_file.exists():
            try:
                self.cache = json.loads(self.cache_file.read_text())
            except (OSError, ValueError):
                self.cache = {}

    def _save(self):
        if self.cache_file:
            tmp = self.cache_file.with_suffix(".tmp")
            tmp.write_text(json.dumps(self.cache, indent=1, sort_keys=True))
            os.replace(tmp, self.cache_file)

    def _time_job(self, dworld, dlut, exposures, spectrum, heel, bowtie, model, launch) -> float:
        from .api import Job
        best = math.inf
        for r in range(self.repeats + 1):  # the first run warms caches and is dropped
            job = Job(self.ctx, dworld, dlut, exposures, spectrum, heel, bowtie, seed=77 + r, model=model, launch=launch)
            job.wait()
            st = A.JobStats()
            rc = self.ctx.lib.dxmc_gpu_job_result(job.handle, A.OUTPUT_RAW, 1.0, None, None, None, A.C.byref(st))
            job.close()
            if rc not in (A.DXMC_OK, A.DXMC_ERR_REJECTION_CAP):
                A.check(rc, self.ctx.handle, "autotune job")
            if r:
                best = min(best, st.job_ms)
        return best

    def tune_job(self, world, dworld, dlut, exposures, spectrum, heel, bowtie, model: int, max_energy: float) -> dict:
        key = "job|" + job_class(world, model, max_energy)
        with self.lock:
            hit = self.cache.get(key)
        if hit is not None:
            return hit
        sample = sample_exposures(exposures, self.sample_histories)
        hist = int(np.sum(sample.n_histories))
        current = dict(DEFAULTS)
        timings = {}

        def measure(params):
            k = json.dumps(params, sort_keys=True)
            if k not in timings:
                launch = {p: v for p, v in params.items() if v != 0}
                timings[k] = self._time_job(dworld, dlut, sample, spectrum, heel, bowtie, model, launch)
            return timings[k]

        base = measure(current)
        best_t = base
        for _ in range(self.rounds):
            changed = False
            for name, values in SPACE.items():
                for v in values:
                    trial = dict(current, **{name: v})
                    t = measure(trial)
                    if t < best_t * 0.99:  # 1 % hysteresis against timing noise
                        best_t, current, changed = t, trial, True
            if not changed:
                break
        result = {"launch": {k: v for k, v in current.items() if v != 0}, "default_ms": base, "tuned_ms": best_t,
                  "speedup": base / best_t, "sample_histories": hist, "trials": len(timings)}
        with self.lock:
            self.cache[key] = result
            self._save()
        return result

    def tune_chains(self, entries: Sequence, label: str) -> dict:
        """Number of concurrent chains for a batch of BatchEntry (times the batch itself)."""
        from .api import Batch
        key = "batch|" + label
        with self.lock:
            hit = self.cache.get(key)
        if hit is not None:
            return hit
        times = {}
        for c in CHAINS:
            best = math.inf
            for r in range(self.repeats + 1):
                b = Batch(self.ctx, entries, mode=A.BATCH_CONCURRENT, chains=c)
                b.wait()
                ms = b.kernel_ms()
                b.close()
                if r:
                    best = min(best, ms)
            times[c] = best
        chains = min(times, key=times.get)
        result = {"chains": chains, "ms": times, "speedup_vs_2": times[2] / times[chains]}
        with self.lock:
            self.cache[key] = result
            self._save()
        return result
