"""GPU test of the two ways results reach the host: into pageable arrays
(post-processing into a device buffer, then copies) and into page-locked
buffers (the post-processing kernel writes them through their device mapping).
Both must give the same values, for every output mode and tally precision."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("tally_mode", [0, 1])
def test_mapped_results_equal_copied_results(gpu_ctx, tally_mode):
    import torch
    import dxmclib_gb300 as dx
    from dxmclib_gb300 import _capi as A
    from dxmclib_gb300.workloads import ct_helical
    wl = ct_helical(nz=16, histories=2_000_000)
    src = wl.source
    dworld = dx.DeviceWorld(gpu_ctx, wl.world)
    dlut = dx.DeviceLut(gpu_ctx, dx.LutBlob(wl.world.materialMap(), dworld.max_density(), src.maxPhotonEnergyProduced()))
    job = dx.Job(gpu_ctx, dworld, dlut, src.exposures(wl.world.directionCosines()), src.spectrum(), src.heel(), None,
                 seed=9, model=1, tally_mode=tally_mode)
    n = wl.world.size()
    for mode in (A.OUTPUT_RAW, A.OUTPUT_EV_PER_HISTORY, A.OUTPUT_DOSE):
        d0, v0, e0, s0 = job.result(mode, calibration=2.5)
        pinned = (torch.full((n,), -1.0, dtype=torch.float64, pin_memory=True).numpy(),
                  torch.full((n,), -1.0, dtype=torch.float64, pin_memory=True).numpy(),
                  torch.zeros(n, dtype=torch.int32, pin_memory=True).numpy().view(np.uint32))
        d1, v1, e1, s1 = job.result(mode, calibration=2.5, out=pinned)
        assert d0.sum() > 0
        np.testing.assert_array_equal(d0, d1)
        np.testing.assert_array_equal(v0, v1)
        np.testing.assert_array_equal(e0, e1)
        assert s0["histories"] == s1["histories"] and s0["steps"] == s1["steps"]
    job.close()
    dlut.close()
    dworld.close()


def test_asynchronous_results(gpu_ctx):
    """dxmc_gpu_job_result_async + _wait: double results equal the synchronous ones
    exactly, float results are their float roundings (Result<float>), and a second
    job submitted before the first one's results are waited for changes neither."""
    import torch
    import dxmclib_gb300 as dx
    from dxmclib_gb300 import _capi as A
    from dxmclib_gb300.workloads import ct_helical
    wl = ct_helical(nz=16, histories=2_000_000)
    src = wl.source
    ex = src.exposures(wl.world.directionCosines())
    dworld = dx.DeviceWorld(gpu_ctx, wl.world)
    dlut = dx.DeviceLut(gpu_ctx, dx.LutBlob(wl.world.materialMap(), dworld.max_density(), src.maxPhotonEnergyProduced()))
    n = wl.world.size()

    def pinned(dtype):
        t = torch.float64 if dtype == np.float64 else torch.float32
        return (torch.full((n,), -1.0, dtype=t, pin_memory=True).numpy(),
                torch.full((n,), -1.0, dtype=t, pin_memory=True).numpy(),
                torch.zeros(n, dtype=torch.int32, pin_memory=True).numpy().view(np.uint32))

    jobs = [dx.Job(gpu_ctx, dworld, dlut, ex, src.spectrum(), src.heel(), None, seed=s, model=1) for s in (9, 10)]
    # queue both jobs' results before waiting for either
    out64 = jobs[0].result_async(A.OUTPUT_EV_PER_HISTORY, out=pinned(np.float64))
    out32 = jobs[1].result_async(A.OUTPUT_DOSE, calibration=2.5, out=pinned(np.float32), dtype=np.float32)
    d64, v64, e64, s64 = jobs[0].result_wait()
    d32, v32, e32, s32 = jobs[1].result_wait()
    assert d64 is out64[0] and d32 is out32[0]
    r0 = jobs[0].result(A.OUTPUT_EV_PER_HISTORY)
    r1 = jobs[1].result(A.OUTPUT_DOSE, calibration=2.5)
    assert d64.sum() > 0 and d32.sum() > 0
    np.testing.assert_array_equal(d64, r0[0])
    np.testing.assert_array_equal(v64, r0[1])
    np.testing.assert_array_equal(e64, r0[2])
    np.testing.assert_array_equal(d32, r1[0].astype(np.float32))
    np.testing.assert_array_equal(v32, r1[1].astype(np.float32))
    np.testing.assert_array_equal(e32, r1[2])
    assert s64["histories"] == r0[3]["histories"] and s64["steps"] == r0[3]["steps"]
    # one asynchronous result per job at a time
    jobs[0].result_async(A.OUTPUT_RAW)
    with pytest.raises(dx.DxmcError):
        jobs[0].result_async(A.OUTPUT_RAW)
    jobs[0].result_wait()
    # a cancelled job's asynchronous result is zeroed and reports the cancellation
    big = dx.Job(gpu_ctx, dworld, dlut, ex, src.spectrum(), src.heel(), None, seed=11, model=1)
    big.cancel()
    buf = pinned(np.float64)
    big.result_async(A.OUTPUT_EV_PER_HISTORY, out=buf)
    d, v, e, st = big.result_wait(check=False)
    assert st["status"] == A.DXMC_ERR_CANCELLED
    assert not d.any() and not v.any() and not e.any()
    for j in (*jobs, big):
        j.close()
    dlut.close()
    dworld.close()
