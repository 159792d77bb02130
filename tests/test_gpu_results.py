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
