"""GPU test of the serving loop: a small mixed stream (pencil, DX and CT jobs
with Poisson arrivals) goes through DoseServer, whose requests arrive while
earlier ones are on the GPU and are batched continuously.  Every served result
must equal the same job run alone through the single-job entry point with the
same seed: per-history random streams make the transport independent of what
else is in flight, so dose and variance agree up to the order of the FP64
atomic additions (rtol 1e-9) and the event counts exactly."""
from __future__ import annotations

import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_served_results_equal_alone(gpu_ctx):
    import dxmclib_gb300 as dx
    from dxmclib_gb300 import _capi as A
    from dxmclib_gb300.serve import DoseServer
    from dxmclib_gb300.workloads import serving_stream

    ctx = gpu_ctx
    stream = serving_stream(n_jobs=12, rate_per_s=400.0, seed=99, histories_range=(100_000, 2_000_000),
                            ct_slices=(24,), dx_sizes=(64, 96))
    server = DoseServer(ctx, chains=3)
    t0 = time.perf_counter()
    futures = []
    for job in stream:
        delay = job.arrival - (time.perf_counter() - t0)
        if delay > 0:
            time.sleep(delay)
        futures.append(server.submit(job.world, job.source, model=1, seed=job.seed, world_key=job.world_key))
    served = [f.result(timeout=120) for f in futures]
    m = server.metrics()
    assert m["jobs"] == len(stream) and m["errors"] == 0
    assert m["batches"] >= 2  # late arrivals were launched while earlier work ran
    assert m["p50_ms"] <= m["p99_ms"]
    server.close()

    for job, res in zip(stream, served):
        src = job.source
        dworld = dx.DeviceWorld(ctx, job.world)
        blob = dx.LutBlob.cached(job.world.materialMap(), dworld.max_density(), src.maxPhotonEnergyProduced())
        dlut = dx.DeviceLut(ctx, blob)
        alone = dx.Job(ctx, dworld, dlut, src.exposures(job.world.directionCosines()), src.spectrum(), src.heel(),
                       src.bowtie(), seed=job.seed, model=1)
        dose, var, nev, stats = alone.result(A.OUTPUT_EV_PER_HISTORY)
        alone.close()
        dlut.close()
        dworld.close()
        tag = f"{job.kind} {job.world_key} seed {job.seed}"
        assert res.numberOfHistories == stats["histories"], tag
        assert res.stats["steps"] == stats["steps"] and res.stats["deposits"] == stats["deposits"], tag
        np.testing.assert_allclose(res.dose, dose, rtol=1e-9, atol=1e-12 * dose.max(), err_msg=tag)
        np.testing.assert_allclose(res.variance, var, rtol=1e-9, atol=1e-12 * var.max(), err_msg=tag)
        np.testing.assert_array_equal(res.nEvents, nev, err_msg=tag)
        res.release()
