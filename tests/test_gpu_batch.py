"""GPU tests of the batched entry point (dxmc_gpu_batch_*): many jobs with
worlds, LUTs, sources and correction models of their own run as one graph,
either as single-job kernels on parallel chains (concurrent mode) or drained
by one persistent multi-job kernel per model (persistent mode).

Every history draws its own random stream (seeded from the job seed and the
history id), so a job's tallies must not depend on whether it ran alone or in
a batch, nor on which warps picked up its work items: raw tallies agree up to
the order of the FP64 atomic additions (rtol 1e-9), event counts and the
step / deposit counters exactly.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _entries(dx, ctx, golden):
    from dxmclib_gb300.workloads import dx_batch
    out = []
    for k, wl in enumerate(dx_batch(n_jobs=4, seed=777, histories_range=(150_000, 600_000))):
        wl.source.updateFromWorld(wl.world)
        wl.source.validate()
        layout = 1 if k == 3 else 0  # one job on the 8-byte voxel layout
        dworld = dx.DeviceWorld(ctx, wl.world, layout=layout)
        blob = dx.LutBlob(wl.world.materialMap(), dworld.max_density(), wl.source.maxPhotonEnergyProduced())
        dlut = dx.DeviceLut(ctx, blob)
        src = wl.source
        out.append(dict(dworld=dworld, dlut=dlut, blob=blob, exposures=src.exposures(wl.world.directionCosines()),
                        spectrum=src.spectrum(), heel=src.heel(), bowtie=src.bowtie(), seed=1000 + k, model=k % 3))
    # the cone world of the golden fixtures with a measurement map (forced photoelectric scoring)
    g = golden("transport_cone_m1.npz")
    world = dx.World()
    world.setDimensions(tuple(int(x) for x in g["dims"]))
    world.setSpacing(tuple(g["spacing"]))
    world.setDensityArray(g["density"])
    world.setMaterialIndexArray(g["material"])
    meas = np.zeros(world.size(), np.uint8)
    meas[: world.size() // 2] = 1
    world.setMeasurementMapArray(meas)
    for n in g["names"]:
        world.addMaterialToMap(dx.Material(str(n)))
    src = dx.IsotropicSource()
    src.setPosition((0, 0, -500))
    src.setCollimationAngles(-0.12, 0.12, -0.1, 0.1)
    src.setSpecter(g["spec_weights"], g["spec_energies"])
    src.setTotalExposures(12)
    src.setHistoriesPerExposure(30_000)
    dworld = dx.DeviceWorld(ctx, world)
    blob = dx.LutBlob(world.materialMap(), dworld.max_density(), src.maxPhotonEnergyProduced())
    out.append(dict(dworld=dworld, dlut=dx.DeviceLut(ctx, blob), blob=blob, exposures=src.exposures(),
                    spectrum=src.spectrum(), heel=None, bowtie=None, seed=99, model=2))
    return out


def _args(e):
    return (e["exposures"], e["spectrum"], e["heel"], e["bowtie"], e["seed"], e["model"], 0)


def test_batch_matches_single_jobs(gpu_ctx, golden):
    import dxmclib_gb300 as dx
    from dxmclib_gb300 import _capi as A

    ctx = gpu_ctx
    entries = _entries(dx, ctx, golden)
    alone = []
    for e in entries:
        job = dx.Job(ctx, e["dworld"], e["dlut"], *_args(e))
        alone.append(job.result(A.OUTPUT_RAW))
        job.close()
        assert alone[-1][0].sum() > 0

    # each mode twice, in two job orders: work distribution differs between runs, results must not
    runs = [(mode, rep) for mode in (dx.Batch.CONCURRENT, dx.Batch.PERSISTENT) for rep in range(2)]
    for mode, rep in runs:
        order = list(range(len(entries)))[::-1] if rep else list(range(len(entries)))
        batch = dx.Batch(ctx, [dx.BatchEntry(entries[i]["dworld"], entries[i]["dlut"], *_args(entries[i])) for i in order],
                         mode=mode, chains=2 + rep)
        assert batch.wait() == A.DXMC_OK
        assert batch.kernel_ms() > 0
        for pos, i in enumerate(order):
            e_b, e2_b, nev_b, st_b = batch.jobs[pos].result(A.OUTPUT_RAW)
            e_a, e2_a, nev_a, st_a = alone[i]
            tag = f"mode {mode} rep {rep} job {i}"
            assert st_b["histories"] == st_a["histories"] == int(np.sum(entries[i]["exposures"].n_histories)), tag
            assert st_b["steps"] == st_a["steps"] and st_b["deposits"] == st_a["deposits"], tag
            assert st_b["rejection_overflows"] == st_a["rejection_overflows"], tag
            np.testing.assert_allclose(e_b, e_a, rtol=1e-9, atol=1e-12 * e_a.max(), err_msg=tag)
            np.testing.assert_allclose(e2_b, e2_a, rtol=1e-9, atol=1e-12 * e2_a.max(), err_msg=tag)
            np.testing.assert_array_equal(nev_b, nev_a, err_msg=tag)
        batch.close()
    for e in entries:
        e["dlut"].close()
        e["dworld"].close()


def test_batch_rejects_incomplete_entries(gpu_ctx):
    from dxmclib_gb300 import _capi as A
    ctx = gpu_ctx
    arr = (A.BatchEntry * 1)()
    out = C.c_void_p()
    rc = ctx.lib.dxmc_gpu_batch_submit(ctx.handle, arr, 1, None, C.byref(out))
    assert rc == A.DXMC_ERR_INVALID and not out.value
    assert b"incomplete" in ctx.lib.dxmc_gpu_last_error(ctx.handle)


def test_autotuned_launch_gives_identical_results(gpu_ctx, tmp_path):
    """Launch parameters change how the histories are scheduled, not which random
    numbers they draw: a tuned job equals the default one, and the tuner's cache
    file serves the second request."""
    import dxmclib_gb300 as dx
    from dxmclib_gb300 import _capi as A
    from dxmclib_gb300.autotune import Autotuner
    from dxmclib_gb300.workloads import dx_batch

    ctx = gpu_ctx
    wl = dx_batch(n_jobs=1, seed=4321, histories_range=(400_000, 400_001))[0]
    src = wl.source
    src.updateFromWorld(wl.world)
    src.validate()
    dworld = dx.DeviceWorld(ctx, wl.world)
    dlut = dx.DeviceLut(ctx, dx.LutBlob(wl.world.materialMap(), dworld.max_density(), src.maxPhotonEnergyProduced()))
    ex = src.exposures(wl.world.directionCosines())
    tuner = Autotuner(ctx, cache_file=str(tmp_path / "tune.json"), sample_histories=300_000, repeats=1, rounds=1)
    res = tuner.tune_job(wl.world, dworld, dlut, ex, src.spectrum(), src.heel(), src.bowtie(), 1,
                         src.maxPhotonEnergyProduced())
    assert res["tuned_ms"] <= res["default_ms"] and res["trials"] >= 10
    for k, v in res["launch"].items():
        assert k in A.JobDesc.__dict__ or k in dict(A.JobDesc._fields_), k
    again = Autotuner(ctx, cache_file=str(tmp_path / "tune.json"))
    assert again.tune_job(wl.world, dworld, dlut, ex, None, None, None, 1, src.maxPhotonEnergyProduced()) == res
    outs = []
    # in-kernel generation and the pre-generated photon queue (two chunks), other
    # thresholds, bursts and block sizes: the same histories
    for launch in (None, res["launch"], {"queue_log2_chunk": -1, "regen_threshold": 16, "interact_threshold": 4,
                                          "blocks_per_sm": 2},
                   {"queue_log2_chunk": 18, "woodcock_burst": 9, "block_size": 128}):
        job = dx.Job(ctx, dworld, dlut, ex, src.spectrum(), src.heel(), src.bowtie(), seed=5, model=1, launch=launch)
        outs.append(job.result(A.OUTPUT_RAW))
        job.close()
    for o in outs[1:]:
        np.testing.assert_allclose(o[0], outs[0][0], rtol=1e-9, atol=1e-12 * outs[0][0].max())
        np.testing.assert_array_equal(o[2], outs[0][2])
        assert o[3]["steps"] == outs[0][3]["steps"]
    dlut.close()
    dworld.close()
