"""Tally-precision study: the same transport scored three ways.

DXMClib accumulates energy imparted and its square per voxel in the transport
type T with atomic adds (``safeValueAdd``, ``transport.hpp:208-214``).  On the
GPU the transport runs in FP32 and the tally has three modes:

* ``TALLY_F64``      -- FP64 atomics for every deposit;
* ``TALLY_WARP_F64`` -- deposits of the lanes of a warp that hit the same voxel
  are summed in FP32 first, the partial is added to the FP64 accumulators;
* ``TALLY_F32``      -- FP32 atomics only.

Every history draws the same random numbers in every mode (per-history streams),
so the runs differ only in how the deposits are summed.  ``study`` reports, per
mode, the per-voxel relative error of the energy imparted against the FP64 run
(over voxels above 1 % of the maximum), the error of the total energy imparted,
and histories/s.
"""
from __future__ import annotations

import numpy as np

from . import _capi as A

MODES = {"fp64": A.TALLY_F64, "warp_fp32_to_fp64": A.TALLY_WARP_F64, "fp32": A.TALLY_F32}


def compare(reference: np.ndarray, other: np.ndarray, threshold: float = 0.01) -> dict:
    """Per-voxel relative error of ``other`` against ``reference`` over voxels above
    ``threshold`` of the reference maximum, and the relative error of the totals."""
    ref = np.asarray(reference, np.float64)
    oth = np.asarray(other, np.float64)
    sel = ref > threshold * ref.max()
    rel = np.abs(oth[sel] - ref[sel]) / ref[sel]
    tot_ref = float(ref.sum())
    return {"voxels": int(sel.sum()), "mean_rel_err": float(rel.mean()), "max_rel_err": float(rel.max()),
            "p99_rel_err": float(np.percentile(rel, 99)),
            "total_energy_rel_err": abs(float(oth.sum()) - tot_ref) / tot_ref}


def study(ctx, world, source, seed: int = 11, model: int = 1, repeats: int = 2) -> dict:
    """Runs the job once per tally mode (plus ``repeats`` timed runs) and compares."""
    from .api import DeviceLut, DeviceWorld, Job, LutBlob
    source.updateFromWorld(world)
    source.validate()
    dworld = DeviceWorld(ctx, world)
    dlut = DeviceLut(ctx, LutBlob.cached(world.materialMap(), dworld.max_density(), source.maxPhotonEnergyProduced()))
    ex = source.exposures(world.directionCosines())
    hist = int(np.sum(ex.n_histories))
    energy = {}
    out = {"histories": hist, "voxels": int(world.size()), "modes": {}}
    for name, mode in MODES.items():
        times = []
        for r in range(repeats + 1):
            job = Job(ctx, dworld, dlut, ex, source.spectrum(), source.heel(), source.bowtie(), seed=seed, model=model,
                      tally_mode=mode)
            if r == 0:
                e, _, _, st = job.result(A.OUTPUT_RAW, want_events=False)
                energy[name] = e
            else:
                job.wait()
                st = A.JobStats()
                A.check(ctx.lib.dxmc_gpu_job_result(job.handle, A.OUTPUT_RAW, 1.0, None, None, None, A.C.byref(st)),
                        ctx.handle, "job_result")
                st = {"job_ms": st.job_ms, "kernel_ms": st.kernel_ms}
                times.append(st["job_ms"])
            job.close()
        out["modes"][name] = {"histories_per_s": hist / (min(times) / 1e3) if times else None,
                              "job_ms": min(times) if times else None}
    for name in MODES:
        if name != "fp64":
            out["modes"][name].update(compare(energy["fp64"], energy[name]))
    dlut.close()
    dworld.close()
    return out
