"""Precision study: FP32 transport with three tally modes against FP64 everywhere.

DXMClib computes the whole transport in its template type T and accumulates
energy imparted and its square per voxel with atomic adds in T
(``Transport<T>``, ``transport.hpp:114-840``; ``safeValueAdd``, ``:208-214``).
On the GPU the transport runs in FP32 and the tally has three modes:

* ``TALLY_F64``      -- FP64 atomics for every deposit;
* ``TALLY_WARP_F64`` -- deposits of the lanes of a warp that hit the same voxel
  are summed in FP32 first, the partial is added to the FP64 accumulators;
* ``TALLY_F32``      -- FP32 atomics only;

and the reference point is the FP64-everywhere kernel (``PRECISION_FP64``:
position, direction, energy, LUT evaluation and sampling in double, FP64
tallies).  Every history draws the same random numbers in every run
(per-history streams), so:

* the three FP32-transport runs follow identical tracks and differ only in how
  the deposits are summed (``vs_fp64_tally``: summation error alone);
* against FP64 everywhere the tracks part once a rounding difference flips a
  comparison, so the difference is the transport's precision error plus the
  Monte Carlo noise of the tracks that parted (``vs_fp64_everywhere``: the
  total-energy error, per-voxel errors, and z-scores of 8 x 8 x 4-voxel block
  sums against the combined standard errors from the variance fields).

Double arithmetic runs at a small fraction of the single-precision rate, so the
FP64-everywhere comparison runs on as many histories per exposure as fit in
``fp64_seconds`` (found from a short pilot), the FP32 runs it is compared with
on exactly those histories.
"""
from __future__ import annotations

import dataclasses

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


def block_sums(values, dims, block):
    nx, ny, nz = (int(d) for d in dims)
    bx, by, bz = block
    a = np.asarray(values, np.float64).reshape(nz // bz, bz, ny // by, by, nx // bx, bx)
    return a.sum(axis=(1, 3, 5)).ravel()


def compare_blocks(ref_dose, ref_var, dose, var, dims, block=(8, 8, 4), threshold: float = 0.01) -> dict:
    """z-scores of block sums (blocks above ``threshold`` of the largest) against
    the combined standard error from both variance fields (EV_PER_HISTORY)."""
    d1, v1 = block_sums(ref_dose, dims, block), block_sums(ref_var, dims, block)
    d2, v2 = block_sums(dose, dims, block), block_sums(var, dims, block)
    mean = 0.5 * (d1 + d2)
    sel = mean > threshold * mean.max()
    z = (d2[sel] - d1[sel]) / np.sqrt(np.maximum(v1[sel], 0) + np.maximum(v2[sel], 0))
    rel = np.abs(d2[sel] - d1[sel]) / d1[sel]
    return {"blocks": int(sel.sum()), "chi2_per_block": float(np.mean(z * z)),
            "frac_within_3sigma": float(np.mean(np.abs(z) <= 3)), "max_abs_z": float(np.max(np.abs(z))),
            "mean_rel_err": float(rel.mean()), "mean_bias": float(np.sum(d2[sel] - d1[sel]) / np.sum(d1[sel]))}


def _run(ctx, dworld, dlut, ex, source, seed, model, tally_mode, precision, repeats):
    """One job with results (EV_PER_HISTORY dose, variance, stats), then ``repeats``
    timed jobs; returns (dose, variance, stats), best job ms."""
    from .api import Job
    times, first = [], None
    for r in range(repeats + 1):
        job = Job(ctx, dworld, dlut, ex, source.spectrum(), source.heel(), source.bowtie(), seed=seed, model=model,
                  tally_mode=tally_mode, precision=precision)
        if r == 0:
            d, v, _, st = job.result(A.OUTPUT_EV_PER_HISTORY, want_events=False)
            first = (d, v, st)
        else:
            job.wait()
            st = A.JobStats()
            A.check(ctx.lib.dxmc_gpu_job_result(job.handle, A.OUTPUT_RAW, 1.0, None, None, None, A.C.byref(st)),
                    ctx.handle, "job_result")
            times.append(st.job_ms)
        job.close()
    return first, (min(times) if times else first[2]["job_ms"])


def study(ctx, world, source, seed: int = 11, model: int = 1, repeats: int = 2, fp64_everywhere: bool = True,
          fp64_seconds: float = 15.0) -> dict:
    """Runs the job once per tally mode (plus ``repeats`` timed runs each) and, on a
    history count the FP64 kernel finishes in about ``fp64_seconds``, FP64
    everywhere and the three FP32 modes on identical per-history streams."""
    from .api import DeviceLut, DeviceWorld, LutBlob
    source.updateFromWorld(world)
    source.validate()
    dworld = DeviceWorld(ctx, world)
    dlut = DeviceLut(ctx, LutBlob.cached(world.materialMap(), dworld.max_density(), source.maxPhotonEnergyProduced()))
    ex = source.exposures(world.directionCosines())
    hist = int(np.sum(ex.n_histories))
    dims = world.dimensions()
    res = {}
    out = {"histories": hist, "voxels": int(world.size()), "modes": {}}
    for name, mode in MODES.items():
        res[name], ms = _run(ctx, dworld, dlut, ex, source, seed, model, mode, A.PRECISION_FP32, repeats)
        out["modes"][name] = {"histories_per_s": hist / (ms / 1e3), "job_ms": ms,
                              "steps_per_history": res[name][2]["steps"] / hist}
    for name in MODES:
        if name != "fp64":
            out["modes"][name]["vs_fp64_tally"] = compare(res["fp64"][0], res[name][0])
    if fp64_everywhere:
        hpe_full = np.asarray(ex.n_histories, np.uint64)
        # pilot: about 1/1000 of the histories
        pilot = dataclasses.replace(ex, n_histories=np.maximum(hpe_full // 1000, 1).astype(np.uint64))
        _, ms = _run(ctx, dworld, dlut, pilot, source, seed, model, A.TALLY_F64, A.PRECISION_FP64, 0)
        scale = min(1.0, max(1e-3, fp64_seconds / max(ms / 1e3, 1e-6) / 1000.0))
        ex64 = dataclasses.replace(ex, n_histories=np.maximum((hpe_full * scale).astype(np.uint64), 1))
        h64 = int(np.sum(ex64.n_histories))
        ref, ms64 = _run(ctx, dworld, dlut, ex64, source, seed, model, A.TALLY_F64, A.PRECISION_FP64, 0)
        out["fp64_everywhere"] = {"histories": h64, "histories_per_s": h64 / (ms64 / 1e3), "job_ms": ms64,
                                  "steps_per_history": ref[2]["steps"] / h64}
        for name, mode in MODES.items():
            (d, v, st), _ = _run(ctx, dworld, dlut, ex64, source, seed, model, mode, A.PRECISION_FP32, 0)
            out["modes"][name]["vs_fp64_everywhere"] = dict(
                compare(ref[0], d), histories=h64, steps_per_history=st["steps"] / h64,
                blocks=compare_blocks(ref[0], ref[1], d, v, dims))
    dlut.close()
    dworld.close()
    return out
