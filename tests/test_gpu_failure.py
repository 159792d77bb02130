"""GPU tests of failure handling without a GPU fault: a wait that runs out
reports DXMC_ERR_TIMEOUT and leaves the job running; a cancelled job (host-set
flag that the kernel reads when its warps take new histories) ends early and
reports zeros with DXMC_ERR_CANCELLED, as the reference's cancelled run does
(transport.hpp:176-185); invalid input and the memory budget are refused on
the host with a status and a message, and the context stays usable."""
from __future__ import annotations

import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_timeout_then_cancel(gpu_ctx):
    import dxmclib_gb300 as dx
    from dxmclib_gb300 import _capi as A
    from dxmclib_gb300.workloads import ct_helical
    ctx = gpu_ctx
    wl = ct_helical(nz=64, histories=3_000_000_000)  # about a second of work
    src = wl.source
    dworld = dx.DeviceWorld(ctx, wl.world)
    dlut = dx.DeviceLut(ctx, dx.LutBlob(wl.world.materialMap(), dworld.max_density(), src.maxPhotonEnergyProduced()))
    job = dx.Job(ctx, dworld, dlut, src.exposures(wl.world.directionCosines()), src.spectrum(), src.heel(), None,
                 seed=3, model=1)
    assert job.wait(0) == A.DXMC_ERR_TIMEOUT
    assert b"timed out" in ctx.lib.dxmc_gpu_last_error(ctx.handle)
    t0 = time.perf_counter()
    job.cancel()
    assert job.wait(30_000) == A.DXMC_OK
    waited = time.perf_counter() - t0
    dose, var, nev, stats = job.result(A.OUTPUT_EV_PER_HISTORY, check=False)
    assert stats["status"] == A.DXMC_ERR_CANCELLED
    assert not dose.any() and not var.any() and not nev.any()
    assert stats["histories"] < 3_000_000_000  # the kernel stopped taking histories
    assert waited < 1.0
    job.close()
    # the context is still usable: a small job runs to completion
    small = ct_helical(nz=64, histories=2_000_000).source
    job = dx.Job(ctx, dworld, dlut, small.exposures(wl.world.directionCosines()), small.spectrum(), small.heel(), None,
                 seed=4, model=1)
    dose, var, nev, stats = job.result(A.OUTPUT_EV_PER_HISTORY)
    assert stats["histories"] == int(np.sum(small.exposures(wl.world.directionCosines()).n_histories))
    assert dose.sum() > 0
    job.close()
    dlut.close()
    dworld.close()


def test_invalid_input_and_budget_are_refused(gpu_ctx):
    import dxmclib_gb300 as dx
    from dxmclib_gb300 import _capi as A
    from dxmclib_gb300.workloads import pencil_water
    ctx = gpu_ctx
    wl = pencil_water(n=16, histories=10_000)
    # material index outside the material map: found by the device check at upload
    # (16 indices per load, then a tail: the last byte of a load, the tail, the first voxel)
    for side, where in ((16, 100), (16, 15), (5, 124), (5, 0)):
        bad = dx.World()
        bad.setDimensions((side, side, side))
        bad.setSpacing((1, 1, 1))
        bad.setDensityArray(np.ones(side ** 3, np.float32))
        mat = np.zeros(side ** 3, np.uint8)
        mat[where] = 3
        bad.setMaterialIndexArray(mat)
        bad.addMaterialToMap(dx.Material("Water, Liquid"))
        bad._valid = True  # bypass the host-side check to reach the device-side one
        with pytest.raises(A.DxmcError) as e:
            dx.DeviceWorld(ctx, bad)
        assert e.value.status == A.DXMC_ERR_INVALID and "material index" in str(e.value), (side, where)
    # unknown correction model
    dworld = dx.DeviceWorld(ctx, wl.world)
    dlut = dx.DeviceLut(ctx, dx.LutBlob(wl.world.materialMap(), dworld.max_density(), 60.0))
    with pytest.raises(A.DxmcError) as e:
        dx.Job(ctx, dworld, dlut, wl.source.exposures(), None, None, None, model=7)
    assert e.value.status == A.DXMC_ERR_INVALID
    # a bow-tie profile without a positive mean weight (its normalisation divides by it)
    for weights in ([0.0, 0.0, 0.0], [1.0, -2.0, 0.5], [1.0, float("nan"), 1.0]):
        with pytest.raises(A.DxmcError) as e:
            dx.Job(ctx, dworld, dlut, wl.source.exposures(), None, None, ([0.0, 0.1, 0.2], weights), model=1)
        assert e.value.status == A.DXMC_ERR_INVALID and "bow-tie" in str(e.value), weights
    # a context whose budget is smaller than the world
    tiny = dx.GpuContext(memory_budget=1 << 12)  # 4 KB: less than the 32 KB of voxels
    with pytest.raises(A.DxmcError) as e:
        dx.DeviceWorld(tiny, wl.world)
    assert e.value.status == A.DXMC_ERR_OOM
    tiny.close()
    # the first context still works
    job = dx.Job(ctx, dworld, dlut, wl.source.exposures(), None, None, None, model=1)
    dose, _, _, stats = job.result(A.OUTPUT_EV_PER_HISTORY)
    assert stats["histories"] == 10_000 and dose.sum() > 0
    job.close()
    dlut.close()
    dworld.close()


def test_progress_and_dose_preview(gpu_ctx):
    """A running job reports the histories its kernels have taken and a preview of
    the energy scored so far (what a ProgressBar shows); once it has finished the
    preview equals the raw energy tally of the result."""
    import dxmclib_gb300 as dx
    from dxmclib_gb300 import _capi as A
    from dxmclib_gb300.workloads import ct_helical
    ctx = gpu_ctx
    wl = ct_helical(nz=64, histories=1_500_000_000)
    src = wl.source
    dworld = dx.DeviceWorld(ctx, wl.world)
    dlut = dx.DeviceLut(ctx, dx.LutBlob(wl.world.materialMap(), dworld.max_density(), src.maxPhotonEnergyProduced()))
    job = dx.Job(ctx, dworld, dlut, src.exposures(wl.world.directionCosines()), src.spectrum(), src.heel(), None,
                 seed=5, model=1)
    seen, sums = [], []
    while job.wait(0) == A.DXMC_ERR_TIMEOUT and len(seen) < 50:
        started, total = job.progress()
        seen.append(started)
        sums.append(job.preview().sum())
        time.sleep(0.01)
    assert job.wait() == A.DXMC_OK
    assert len(seen) >= 2, "the job finished before it could be observed"
    assert seen == sorted(seen) and seen[-1] <= total
    assert sums == sorted(sums) and sums[-1] > 0
    final_preview = job.preview()
    started, total = job.progress()
    assert started == total
    e, _, _, stats = job.result(A.OUTPUT_RAW, want_events=False)
    np.testing.assert_array_equal(final_preview, e)
    job.close()
    dlut.close()
    dworld.close()
