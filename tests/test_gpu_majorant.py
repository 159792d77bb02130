"""GPU tests of local-majorant Woodcock tracking.

The grid of a (world, LUT) pair must bound the attenuation: for every cell
holding (1 / s, R), each voxel within the distance R of the cell attenuates less
than s times the global majorant at every energy of the LUT.  The check below
recomputes that from the host LUT (double precision) with an exact distance
transform at voxel resolution.  Tracking with the grid must then sample the
same process as the reference's global majorant: dose, variance and totals of
both modes agree within the statistical criteria of tests/parity.py, with far
fewer Woodcock steps per history.
"""
from __future__ import annotations

import numpy as np
import pytest

from parity import assert_parity, compare_sparse

pytestmark = pytest.mark.gpu


def _phantom():
    from dxmclib_gb300.workloads import ct_world
    # the CT body phantom at 4 x 4 x 5 mm voxels (air, soft tissue, lung, bone)
    return ct_world(nz=24, nx=104, ny=104, spacing=(4.0, 4.0, 5.0), seed=7)


def _voxel_scales(world, blob, e_lo, e_hi):
    """Per voxel, the largest ratio of its attenuation to the global majorant over
    the energies [e_lo, e_hi] (measurement voxels count as 1)."""
    energies = np.exp(np.linspace(np.log(e_lo), np.log(e_hi), 400))
    inv = np.array([blob.max_attenuation_inverse(e) for e in energies])
    r = np.array([max(blob.attenuation(m, e).sum() * i for e, i in zip(energies, inv))
                  for m in range(len(world.materialMap()))])
    s = world.densityArray().astype(np.float64) * r[world.materialIndexArray()]
    if world.measurementMapArray() is not None:
        s[world.measurementMapArray() != 0] = 1.0
    d = world.dimensions()
    return s.reshape(d[2], d[1], d[0])


def _check_grid_bounds(dworld, dlut, world, blob, expect_air=True, expect_mid=True):
    """Every cell's (1 / s, R) per band bounds the attenuation of every voxel within
    R, and every voxel outside the body box lies within the majorant of every cell
    marked outside it."""
    from scipy import ndimage
    shift, edges, box, cells = dworld.majorant(dlut)
    assert cells.shape[3] == len(edges) + 1 >= 4 and np.all(np.diff(edges) > 0)
    bounds = [1.0, *edges, blob.info()["max_energy"]]
    sp = np.array(world.spacing())[::-1]  # (z, y, x) mm
    b = [1 << int(shift[2]), 1 << int(shift[1]), 1 << int(shift[0])]
    d = world.dimensions()
    zc, yc, xc = np.meshgrid(*[(np.arange(d[i]) + 0.5) * world.spacing()[i] for i in (2, 1, 0)], indexing="ij")
    lower = [-0.5 * d[i] * world.spacing()[i] + world.origin()[i] for i in range(3)]
    pos = [xc + lower[0], yc + lower[1], zc + lower[2]]
    checked = 0
    for band in range(cells.shape[3]):
        scale = _voxel_scales(world, blob, bounds[band] * 1.0001, bounds[band + 1] * 0.9999)
        s_cell = 1.0 / cells[..., band, 0].astype(np.float64)
        R_signed = cells[..., band, 1].astype(np.float64)
        R_cell = np.abs(R_signed)
        assert np.all(s_cell <= 1.0 + 1e-6)
        marked = R_signed < 0
        if marked.any():
            out_box = np.zeros(scale.shape, bool)
            for a in range(3):
                out_box |= (pos[a] < box[a]) | (pos[a] > box[3 + a])
            assert scale[out_box].max() <= s_cell[marked].min() * (1.0 + 1e-4), (band, scale[out_box].max(), s_cell[marked].min())
        if expect_air:
            # air cells far from the body get small scales and long flights
            assert (s_cell < 0.01).mean() > 0.05, np.unique(s_cell)
            assert np.nanmax(np.where(s_cell < 0.01, R_cell, np.nan)) > 30.0
            assert marked.any() and (~marked).any()
        if expect_mid:  # some cells get a level well below the global majorant
            assert np.any((s_cell > 0.05) & (s_cell < 0.7)), np.unique(s_cell)
        for s in np.unique(s_cell[np.isfinite(R_cell)]):
            hot = scale > s * (1.0 + 1e-4)
            if not hot.any():
                continue
            # exact gap between voxel boxes: distance transform to the hot set dilated by one voxel
            near = ndimage.binary_dilation(hot, structure=np.ones((3, 3, 3), bool))
            gap = np.where(near, 0.0, ndimage.distance_transform_edt(~near, sampling=sp))
            pad = [(0, (-gap.shape[i]) % b[i]) for i in range(3)]
            g = np.pad(gap, pad, constant_values=np.inf)
            cell_gap = g.reshape(g.shape[0] // b[0], b[0], g.shape[1] // b[1], b[1], g.shape[2] // b[2], b[2]).min(axis=(1, 3, 5))
            sel = (s_cell == s) & np.isfinite(R_cell)
            bad = sel & (R_cell > cell_gap + 1e-3)
            assert not bad.any(), (band, s, int(bad.sum()), R_cell[bad][:5], cell_gap[bad][:5])
            checked += int(sel.sum())
    assert checked > 0


def test_majorant_grid_bounds_attenuation(gpu_ctx):
    import dxmclib_gb300 as dx
    world = _phantom()
    dworld = dx.DeviceWorld(gpu_ctx, world)
    dlut = dx.DeviceLut(gpu_ctx, dx.LutBlob.from_world(world, 120.0))
    dworld.prepare(dlut)
    _check_grid_bounds(dworld, dlut, world, dx.LutBlob.from_world(world, 120.0))
    dlut.close()
    dworld.close()


def _continuous_world(n=48, distinct=None, seed=3, dims=None, spacing=3.0):
    """Soft tissue and bone with densities from a smooth field: ``distinct`` density
    values (compact layout, many levels per band) or all different (8-byte layout);
    ``dims`` (x, y, z) for a non-cubic grid."""
    import dxmclib_gb300 as dx
    rng = np.random.default_rng(seed)
    nx, ny, nz = dims or (n, n, n)
    z, y, x = np.meshgrid(np.linspace(-1, 1, nz), np.linspace(-1, 1, ny), np.linspace(-1, 1, nx), indexing="ij")
    field = 0.05 + 1.9 * np.clip(0.5 + 0.5 * np.sin(3 * x + rng.uniform(0, 3)) * np.cos(2 * y) * np.cos(z), 0, 1)
    if distinct:
        field = np.round(field * distinct / 2.0) * 2.0 / distinct + 0.001
    mat = (field > 1.3).astype(np.uint8)
    w = dx.World()
    w.setDimensions((nx, ny, nz))
    w.setSpacing((spacing, spacing, spacing))
    w.setDensityArray(field.astype(np.float32).ravel())
    w.setMaterialIndexArray(mat.ravel())
    w.addMaterialToMap(dx.Material("Tissue, Soft (ICRP)"))
    w.addMaterialToMap(dx.Material("Bone, Cortical (ICRP)"))
    assert w.isValid()
    return w


@pytest.mark.parametrize("dims", [(12, 400, 12), (12, 12, 400)])
def test_grid_bounds_on_long_axes(gpu_ctx, dims):
    """The y pass of the distance transform reads tiles of the grid from shared
    memory where a line of cells fits; longer lines (here 400 cells of 6 mm
    along y) take the global-memory kernel, as the z pass does.  Both must bound
    the attenuation, with safe lengths of many cells along the long axis."""
    import dxmclib_gb300 as dx
    # a rod of low-density tissue with a bone slab across the long axis: cells far
    # from the slab get low scales with safe lengths of many cells along that axis
    nx, ny, nz = dims
    axis = 1 if ny > nz else 0  # axis of the (z, y, x) array along the rod
    mat = np.zeros((nz, ny, nx), np.uint8)
    sl = [slice(None)] * 3
    sl[axis] = slice(180, 200)
    mat[tuple(sl)] = 1
    dens = np.where(mat == 1, 1.92, 0.3).astype(np.float32)
    world = dx.World()
    world.setDimensions(dims)
    world.setSpacing((6.0, 6.0, 6.0))
    world.setDensityArray(dens.ravel())
    world.setMaterialIndexArray(mat.ravel())
    world.addMaterialToMap(dx.Material("Tissue, Soft (ICRP)"))
    world.addMaterialToMap(dx.Material("Bone, Cortical (ICRP)"))
    assert world.isValid()
    blob = dx.LutBlob.from_world(world, 90.0)
    dworld = dx.DeviceWorld(gpu_ctx, world)
    dlut = dx.DeviceLut(gpu_ctx, blob)
    dworld.prepare(dlut)
    shift, _, _, cells = dworld.majorant(dlut)
    assert max(cells.shape[:3]) == 400 and list(shift) == [0, 0, 0]
    R = np.abs(cells[..., 1])
    assert np.nanmax(np.where(np.isfinite(R), R, np.nan)) > 100 * 6.0  # safe lengths of 100+ cells
    _check_grid_bounds(dworld, dlut, world, blob, expect_air=False, expect_mid=False)
    dlut.close()
    dworld.close()


@pytest.mark.parametrize("distinct", [120, None])
def test_many_levels_grid_bounds_and_parity(gpu_ctx, distinct):
    """Worlds with many density values (120 in the compact layout, all different in
    the 8-byte layout) have many majorant levels per band; the grid keeps at most
    12 distance transforms per band and must still bound the attenuation, and both
    tracking modes must agree."""
    import dxmclib_gb300 as dx
    from dxmclib_gb300 import _capi as A
    world = _continuous_world(distinct=distinct)
    dworld = dx.DeviceWorld(gpu_ctx, world)
    blob = dx.LutBlob.from_world(world, 90.0)
    dlut = dx.DeviceLut(gpu_ctx, blob)
    dworld.prepare(dlut)
    _check_grid_bounds(dworld, dlut, world, blob, expect_air=False)
    src = dx.DXSource()
    src.tube().setVoltage(90)
    src.tube().setAlFiltration(3.0)
    src.setFieldSize((150, 150))
    src.setHistoriesPerExposure(2_000_000)
    src.setTotalExposures(2)
    ex = src.exposures(world.directionCosines())
    out = {}
    for mode in (A.TRACKING_GLOBAL, A.TRACKING_LOCAL):
        job = dx.Job(gpu_ctx, dworld, dlut, ex, src.spectrum(), src.heel(), None, seed=41 + mode, model=1, tracking=mode)
        out[mode] = job.result(A.OUTPUT_EV_PER_HISTORY)
        job.close()
    dg, vg = out[A.TRACKING_GLOBAL][:2]
    dl, vl, _, sl = out[A.TRACKING_LOCAL]
    ref = dict(idx=np.arange(dg.size), dose=dg, var=vg, total=np.array([dg.sum()]))
    assert_parity(compare_sparse(ref, dl, vl), f"many levels ({distinct}), local vs global")
    assert sl["steps"] < out[A.TRACKING_GLOBAL][3]["steps"]
    dlut.close()
    dworld.close()


@pytest.mark.parametrize("distinct", [120, None])
def test_grid_does_not_depend_on_the_grouping_of_levels(gpu_ctx, distinct):
    """The distance transforms of a build's (band, level) pairs run in groups
    sized by the scratch memory the context's budget leaves; a context whose
    budget leaves room for one or three pairs at a time builds the same grid,
    bit for bit, as one that runs them all together."""
    import dxmclib_gb300 as dx
    world = _continuous_world(distinct=distinct)
    blob = dx.LutBlob.from_world(world, 90.0)
    _, m0 = gpu_ctx.memory()
    dworld = dx.DeviceWorld(gpu_ctx, world)
    dlut = dx.DeviceLut(gpu_ctx, blob)
    _, m1 = gpu_ctx.memory()
    dworld.prepare(dlut)
    _, m2 = gpu_ctx.memory()
    ref = dworld.majorant(dlut)
    dlut.close()
    dworld.close()
    shift, edges, box, cells = ref
    ncell, bands = int(np.prod(cells.shape[:3])), cells.shape[3]
    # the build holds the grid, two level bytes and a cost float per cell and band,
    # and two scratch floats per cell for each pair of a group
    held = (m1 - m0) + (m2 - m1) + ncell * bands * 6
    for per_group in (1, 3):
        ctx = dx.GpuContext(memory_budget=held + 8 * ncell * per_group + 4 * ncell)
        try:
            w = dx.DeviceWorld(ctx, world)
            lut = dx.DeviceLut(ctx, blob)
            w.prepare(lut)
            got = w.majorant(lut)
            for a, b in zip(ref, got):
                np.testing.assert_array_equal(a, b, err_msg=f"{per_group} pairs per group")
            lut.close()
            w.close()
        finally:
            ctx.close()


@pytest.mark.parametrize("model,layout", [(1, 0), (2, 0), (1, 1)])
def test_local_tracking_matches_global(gpu_ctx, model, layout):
    """Both tracking modes on the compact (palette) and the 8-byte voxel layout;
    the 8-byte layout has no body box (its levels are not known on the host)."""
    import dxmclib_gb300 as dx
    from dxmclib_gb300 import _capi as A
    from dxmclib_gb300.workloads import ct_source
    world = _phantom()
    src = ct_source(world, 4_000_000)
    dworld = dx.DeviceWorld(gpu_ctx, world, layout=layout)
    dlut = dx.DeviceLut(gpu_ctx, dx.LutBlob.from_world(world, src.maxPhotonEnergyProduced()))
    ex = src.exposures(world.directionCosines())
    out = {}
    for mode in (A.TRACKING_GLOBAL, A.TRACKING_LOCAL):
        job = dx.Job(gpu_ctx, dworld, dlut, ex, src.spectrum(), src.heel(), None, seed=11 + mode, model=model,
                     tracking=mode)
        out[mode] = job.result(A.OUTPUT_EV_PER_HISTORY)
        job.close()
    dg, vg, _, sg = out[A.TRACKING_GLOBAL]
    dl, vl, _, sl = out[A.TRACKING_LOCAL]
    assert sg["histories"] == sl["histories"]
    ref = dict(idx=np.arange(dg.size), dose=dg, var=vg, total=np.array([dg.sum()]))
    assert_parity(compare_sparse(ref, dl, vl), f"local vs global tracking, model {model}, layout {layout}")
    # the same process with fewer steps
    assert sl["steps"] < 0.75 * sg["steps"], (sl["steps"], sg["steps"])
    dlut.close()
    dworld.close()


def test_forced_scoring_keeps_global_majorant(gpu_ctx):
    """Measurement voxels (forced photoelectric scoring) count as scale 1, so the
    cells around them keep the global majorant and the forced estimator sees the
    reference's step density: both tracking modes give the same scored dose."""
    import dxmclib_gb300 as dx
    from dxmclib_gb300 import _capi as A
    from dxmclib_gb300.workloads import ct_source
    world = _phantom()
    d = world.dimensions()
    meas = np.zeros((d[2], d[1], d[0]), np.uint8)
    meas[8:16, 40:64, 40:64] = 1
    world.setMeasurementMapArray(meas.ravel())
    assert world.isValid()
    # the measured region's total must agree within 0.5 %: 2e7 histories put its
    # standard error near 0.15 %
    src = ct_source(world, 20_000_000)
    dworld = dx.DeviceWorld(gpu_ctx, world)
    dlut = dx.DeviceLut(gpu_ctx, dx.LutBlob.from_world(world, src.maxPhotonEnergyProduced()))
    dworld.prepare(dlut)
    shift, _, _, cells = dworld.majorant(dlut)
    b = [1 << int(shift[2]), 1 << int(shift[1]), 1 << int(shift[0])]
    # cells holding a measurement voxel track with the global majorant in every band
    m = np.pad(meas, [(0, (-meas.shape[i]) % b[i]) for i in range(3)])
    mc = m.reshape(m.shape[0] // b[0], b[0], m.shape[1] // b[1], b[1], m.shape[2] // b[2], b[2]).max(axis=(1, 3, 5))
    assert np.all(cells[mc > 0][..., 0] == 1.0) and np.all(np.isposinf(cells[mc > 0][..., 1]))
    ex = src.exposures(world.directionCosines())
    runs = []
    for seed, mode in ((21, A.TRACKING_GLOBAL), (22, A.TRACKING_GLOBAL), (23, A.TRACKING_LOCAL)):
        job = dx.Job(gpu_ctx, dworld, dlut, ex, src.spectrum(), src.heel(), None, seed=seed, model=1, tracking=mode)
        runs.append(job.result(A.OUTPUT_EV_PER_HISTORY)[:2])
        job.close()
    sel = meas.ravel() > 0
    ref = dict(idx=np.flatnonzero(sel), dose=runs[0][0][sel], var=runs[0][1][sel], total=np.array([runs[0][0][sel].sum()]))

    def against_ref(d, v):
        d_in = np.zeros_like(d)
        d_in[sel] = d[sel]
        return compare_sparse(ref, d_in, v)

    # forced scoring deposits at every step in a measured voxel, so the per-event
    # variance field under-states the spread even between two global runs: that
    # pair's chi2/dof sets the bound for the local run
    same = against_ref(*runs[1])
    assert_parity(same, "forced scoring, global vs global", correlated=True, max_chi2=1.6)
    assert_parity(against_ref(*runs[2]), "forced scoring, local vs global", correlated=True,
                  max_chi2=max(1.2, same["chi2"]) * 1.1)
    dlut.close()
    dworld.close()


def test_majorant_grids_per_world_are_evicted_and_accounted(gpu_ctx):
    """A world keeps the grids of up to four LUTs; a fifth LUT evicts the least
    recently used one (after the context's queued work), jobs on any of them stay
    correct, and freeing the world returns every grid's bytes to the budget."""
    import dxmclib_gb300 as dx
    from dxmclib_gb300 import _capi as A
    from dxmclib_gb300.workloads import ct_source
    world = _phantom()
    src = ct_source(world, 200_000)
    ex = src.exposures(world.directionCosines())
    _, before = gpu_ctx.memory()
    dworld = dx.DeviceWorld(gpu_ctx, world)
    _, with_world = gpu_ctx.memory()
    luts = [dx.DeviceLut(gpu_ctx, dx.LutBlob.from_world(world, e)) for e in (120.0, 121.0, 122.0, 123.0, 124.0)]
    _, with_luts = gpu_ctx.memory()
    totals = []
    for i, dlut in enumerate(luts):
        dworld.prepare(dlut)
        job = dx.Job(gpu_ctx, dworld, dlut, ex, src.spectrum(), src.heel(), None, seed=5, model=1)
        d, _, _, st = job.result(A.OUTPUT_RAW, want_events=False)
        assert st["histories"] == int(np.sum(ex.n_histories)) and d.sum() > 0
        totals.append(d.sum() / st["histories"])
        job.close()
    _, with_grids = gpu_ctx.memory()
    grid_bytes = (with_grids - with_luts) / 4  # four grids stay
    assert grid_bytes > 0
    # the first LUT's grid was evicted: reading it back fails, the last one's succeeds
    with pytest.raises(A.DxmcError) as e:
        dworld.majorant(luts[0])
    assert e.value.status == A.DXMC_ERR_STATE
    dworld.majorant(luts[-1])
    # a job on the evicted pair rebuilds its grid
    job = dx.Job(gpu_ctx, dworld, luts[0], ex, src.spectrum(), src.heel(), None, seed=5, model=1)
    d, _, _, st = job.result(A.OUTPUT_RAW, want_events=False)
    job.close()
    np.testing.assert_allclose(d.sum() / st["histories"], totals[0], rtol=1e-9)  # same seed, same grid
    dworld.close()
    _, after_world = gpu_ctx.memory()
    assert after_world == with_luts - (with_world - before)
    for dlut in luts:
        dlut.close()
    _, after = gpu_ctx.memory()
    assert after == before


@pytest.mark.parametrize("mode", ["concurrent", "persistent"])
def test_batch_keeps_the_grids_of_all_its_entries(gpu_ctx, mode):
    """A batch whose entries use one world with more LUTs than a world caches
    grids for: no entry's grid is evicted before the batch has launched, so every
    entry equals its job run alone; the next grid built outside the batch trims
    the cache back to four grids, and freeing the world returns every grid's bytes."""
    import dxmclib_gb300 as dx
    from dxmclib_gb300 import _capi as A
    from dxmclib_gb300.workloads import ct_source
    world = _phantom()
    src = ct_source(world, 150_000)
    ex = src.exposures(world.directionCosines())
    _, before = gpu_ctx.memory()
    dworld = dx.DeviceWorld(gpu_ctx, world)
    _, with_world = gpu_ctx.memory()
    luts = [dx.DeviceLut(gpu_ctx, dx.LutBlob.from_world(world, e)) for e in (120.0, 121.0, 122.0, 123.0, 124.0, 125.0)]
    extra = dx.DeviceLut(gpu_ctx, dx.LutBlob.from_world(world, 126.0))
    _, with_luts = gpu_ctx.memory()
    alone = []
    for dlut in luts:  # leaves the grids of the last four LUTs cached
        job = dx.Job(gpu_ctx, dworld, dlut, ex, src.spectrum(), src.heel(), None, seed=5, model=1)
        alone.append(job.result(A.OUTPUT_RAW))
        job.close()
    _, four = gpu_ctx.memory()
    grid_bytes = (four - with_luts) // 4
    assert grid_bytes > 0 and four == with_luts + 4 * grid_bytes
    batch = dx.Batch(gpu_ctx, [dx.BatchEntry(dworld, dlut, ex, src.spectrum(), src.heel(), None, 5, 1) for dlut in luts],
                     mode=dx.Batch.CONCURRENT if mode == "concurrent" else dx.Batch.PERSISTENT)
    assert batch.wait() == A.DXMC_OK
    for i, (e_a, e2_a, nev_a, st_a) in enumerate(alone):
        e_b, e2_b, nev_b, st_b = batch.jobs[i].result(A.OUTPUT_RAW)
        assert st_b["histories"] == st_a["histories"] and st_b["steps"] == st_a["steps"], i
        np.testing.assert_allclose(e_b, e_a, rtol=1e-9, atol=1e-12 * e_a.max(), err_msg=str(i))
        np.testing.assert_array_equal(nev_b, nev_a, err_msg=str(i))
    batch.close()
    for dlut in luts:  # two grids rebuilt, none evicted inside the batch
        dworld.majorant(dlut)
    # (the batch engines' buffers stay allocated: compare differences from here on)
    _, six = gpu_ctx.memory()
    dworld.prepare(extra)
    _, trimmed = gpu_ctx.memory()
    assert six - trimmed == 2 * grid_bytes  # three evicted, one built
    with pytest.raises(A.DxmcError):
        dworld.majorant(luts[0])
    dworld.majorant(extra)
    dworld.close()
    _, after_world = gpu_ctx.memory()
    assert trimmed - after_world == (with_world - before) + 4 * grid_bytes
    for dlut in luts + [extra]:
        dlut.close()
    _, after = gpu_ctx.memory()
    assert after_world - after == with_luts - with_world
