"""GPU test of dxmc_gpu_transport_noalloc, the entry point for callers that
cannot allocate device memory while they run (an application that hands the
library a fixed arena, a real-time loop that must not reach the allocator).

It runs a job through the regular entry point (dxmc_gpu_job_submit /
dxmc_gpu_job_result with raw output) and then twice in a row through the
no-allocation entry point with the same seed, into device buffers the test owns.
Both paths draw identical per-history random streams, so the tallies agree up
to the order of the FP64 atomic additions (rtol 1e-9) and the event counts
exactly.  This file is collected last so that a run stopping at the first
failure has already run every other test.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _job_desc(exposures, spectrum, heel, bowtie, seed, keep):
    from dxmclib_gb300 import _capi as A
    jd = A.JobDesc()
    ex = exposures.to_c()
    keep.append(ex)
    jd.exposures = ex.ctypes.data_as(C.POINTER(A.Exposure))
    jd.n_exposures = len(exposures)
    se = np.ascontiguousarray(spectrum.energies, np.float64)
    sw = np.ascontiguousarray(spectrum.weights, np.float64)
    sd = A.SpectrumDesc(len(se), se.ctypes.data_as(A.DP), sw.ctypes.data_as(A.DP))
    hw = np.ascontiguousarray(heel.weights, np.float64)
    hd = A.HeelDesc(heel.energy_start, heel.energy_step, heel.energy_size, heel.angle_size, heel.angle_start,
                    heel.angle_step, hw.ctypes.data_as(A.DP))
    ba = np.ascontiguousarray(bowtie[0], np.float64)
    bw = np.ascontiguousarray(bowtie[1], np.float64)
    bd = A.BowtieDesc(len(ba), ba.ctypes.data_as(A.DP), bw.ctypes.data_as(A.DP))
    keep += [se, sw, sd, hw, hd, ba, bw, bd]
    jd.spectrum = C.pointer(sd)
    jd.heel = C.pointer(hd)
    jd.bowtie = C.pointer(bd)
    jd.seed = seed
    jd.model = 1
    jd.tally_mode = 0
    return jd


def test_noalloc_matches_job_entry_point(gpu_ctx, golden):
    import torch
    import dxmclib_gb300 as dx
    from dxmclib_gb300 import _capi as A

    g = golden("transport_cone_m1.npz")
    dims = tuple(int(x) for x in g["dims"])
    world = dx.World()
    world.setDimensions(dims)
    world.setSpacing(tuple(g["spacing"]))
    world.setDensityArray(g["density"])
    world.setMaterialIndexArray(g["material"])
    for n in g["names"]:
        world.addMaterialToMap(dx.Material(str(n)))
    assert world.isValid()
    src = dx.IsotropicSource()
    src.setPosition((0, 0, -500))
    src.setCollimationAngles(-0.12, 0.12, -0.1, 0.1)
    src.setSpecter(g["spec_weights"], g["spec_energies"])
    src.setTotalExposures(16)
    src.setHistoriesPerExposure(50_000)
    exposures = src.exposures()
    spectrum = src.spectrum()
    tube = dx.Tube(100.0)
    tube.setAlFiltration(2.5)
    heel = dx.HeelFilter(tube, 0.24).table()
    bowtie = (np.linspace(-0.2, 0.2, 21), 1.0 + 2.0 * np.linspace(-0.2, 0.2, 21) ** 2)

    ctx = gpu_ctx
    dworld = dx.DeviceWorld(ctx, world)
    blob = dx.LutBlob(world.materialMap(), dworld.max_density(), src.maxPhotonEnergyProduced())
    dlut = dx.DeviceLut(ctx, blob)
    seed = 4242

    job = dx.Job(ctx, dworld, dlut, exposures, spectrum, heel, bowtie, seed=seed, model=1, tally_mode=0)
    e_ref, e2_ref, nev_ref, stats_ref = job.result(A.OUTPUT_RAW)
    job.close()
    n = world.size()
    assert e_ref.sum() > 0

    keep = []
    jd = _job_desc(exposures, spectrum, heel, bowtie, seed, keep)
    tally = torch.full((2 * n,), -1.0, dtype=torch.float64, device="cuda")
    nev = torch.full((n,), 7, dtype=torch.int32, device="cuda")

    def noalloc(desc, dw, with_stats=True):
        st = A.JobStats() if with_stats else None
        rc = ctx.lib.dxmc_gpu_transport_noalloc(ctx.handle, dw.handle, dlut.handle, C.byref(desc),
                                                C.c_void_p(tally.data_ptr()), C.c_void_p(nev.data_ptr()),
                                                C.byref(st) if with_stats else None)
        A.check(rc, ctx.handle, "dxmc_gpu_transport_noalloc")
        torch.cuda.synchronize()
        return st, tally.cpu().numpy(), nev.cpu().numpy().view(np.uint32)

    def same(t, nv, e, e2, ne, label):
        np.testing.assert_allclose(t[0::2], e, rtol=1e-9, atol=1e-12 * e.max(), err_msg=label)
        np.testing.assert_allclose(t[1::2], e2, rtol=1e-9, atol=1e-12 * e2.max(), err_msg=label)
        np.testing.assert_array_equal(nv, ne, err_msg=label)

    for call in range(2):  # two calls in a row share (and must clear) the static scratch
        st, t, nv = noalloc(jd, dworld)
        assert st.histories == stats_ref["histories"] == int(np.sum(exposures.n_histories)), call
        assert st.steps == stats_ref["steps"] and st.deposits == stats_ref["deposits"], call
        same(t, nv, e_ref, e2_ref, nev_ref, f"call {call}")

    # without a stats pointer the call still reads the device counters (a rejection-cap
    # overflow is reported through the return code) and gives the same tallies
    _, t, nv = noalloc(jd, dworld, with_stats=False)
    same(t, nv, e_ref, e2_ref, nev_ref, "stats = NULL")

    # the reference's global majorant, both entry points
    jd.tracking = A.TRACKING_GLOBAL
    job = dx.Job(ctx, dworld, dlut, exposures, spectrum, heel, bowtie, seed=seed, model=1, tally_mode=0,
                 tracking=A.TRACKING_GLOBAL)
    eg, e2g, neg, stg = job.result(A.OUTPUT_RAW)
    job.close()
    st, t, nv = noalloc(jd, dworld)
    assert st.steps == stg["steps"] and st.deposits == stg["deposits"]
    same(t, nv, eg, e2g, neg, "global majorant")
    assert st.steps > stats_ref["steps"]  # the local grid really was in use above

    # local majorants on a world whose grid was built by dxmc_gpu_world_prepare (no job
    # has run on it): the no-allocation call tracks with that grid, as a regular job does
    dworld2 = dx.DeviceWorld(ctx, world)
    dworld2.prepare(dlut)
    jd.tracking = A.TRACKING_LOCAL
    st, t, nv = noalloc(jd, dworld2)
    job = dx.Job(ctx, dworld2, dlut, exposures, spectrum, heel, bowtie, seed=seed, model=1, tally_mode=0,
                 tracking=A.TRACKING_LOCAL)
    el, e2l, nel, stl = job.result(A.OUTPUT_RAW)
    job.close()
    assert st.steps == stl["steps"] == stats_ref["steps"] and st.deposits == stl["deposits"]
    same(t, nv, el, e2l, nel, "local majorant after prepare")
    dworld2.close()
    jd.tracking = A.TRACKING_DEFAULT

    # a heel table whose size overflows 32 bits is rejected before any device work
    huge = A.HeelDesc(heel.energy_start, heel.energy_step, 65536, 65536, heel.angle_start, heel.angle_step,
                      jd.heel.contents.weights)
    jd_huge = _job_desc(exposures, spectrum, heel, bowtie, seed, keep)
    jd_huge.heel = C.pointer(huge)
    rc = ctx.lib.dxmc_gpu_transport_noalloc(ctx.handle, dworld.handle, dlut.handle, C.byref(jd_huge),
                                            C.c_void_p(tally.data_ptr()), C.c_void_p(nev.data_ptr()), None)
    assert rc == A.DXMC_ERR_INVALID
    assert b"maximum" in ctx.lib.dxmc_gpu_last_error(ctx.handle)
    handle = C.c_void_p()
    rc = ctx.lib.dxmc_gpu_job_submit(ctx.handle, dworld.handle, dlut.handle, C.byref(jd_huge), C.byref(handle))
    assert rc == A.DXMC_ERR_INVALID and not handle.value
    assert b"maximum" in ctx.lib.dxmc_gpu_last_error(ctx.handle)

    # jobs beyond the stated maximum are rejected with a clear message, before any device work
    big = dx.ExposureTable.build(np.zeros((8193, 3)), np.tile([1, 0, 0, 0, 1, 0], (8193, 1)), (0, 0, 0, 0), 1.0, 1, 60.0)
    jd_big = _job_desc(big, spectrum, heel, bowtie, seed, keep)
    rc = ctx.lib.dxmc_gpu_transport_noalloc(ctx.handle, dworld.handle, dlut.handle, C.byref(jd_big),
                                            C.c_void_p(tally.data_ptr()), C.c_void_p(nev.data_ptr()), None)
    assert rc == A.DXMC_ERR_INVALID
    assert b"maximum" in ctx.lib.dxmc_gpu_last_error(ctx.handle)

    # a bow-tie profile without a positive mean weight is rejected by both entry points
    jd_bt = _job_desc(exposures, spectrum, heel, (bowtie[0], np.zeros(len(bowtie[0]))), seed, keep)
    rc = ctx.lib.dxmc_gpu_transport_noalloc(ctx.handle, dworld.handle, dlut.handle, C.byref(jd_bt),
                                            C.c_void_p(tally.data_ptr()), C.c_void_p(nev.data_ptr()), None)
    assert rc == A.DXMC_ERR_INVALID
    assert b"bow-tie" in ctx.lib.dxmc_gpu_last_error(ctx.handle)
    rc = ctx.lib.dxmc_gpu_job_submit(ctx.handle, dworld.handle, dlut.handle, C.byref(jd_bt), C.byref(handle))
    assert rc == A.DXMC_ERR_INVALID and not handle.value
    dlut.close()
    dworld.close()
