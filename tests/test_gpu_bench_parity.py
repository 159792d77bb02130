"""GPU parity on the benchmark's own configurations and in DOSE output mode.

* The headline CT helical workload: 512 x 512 x 200 voxels of 0.8 x 0.8 x 2.5
  mm (the seeded body phantom), 120 kVp helical scan with the reference's own
  exposure, spectrum and heel tables, run in the default mode of this library
  (compact palette voxels, local-majorant tracking) against DXMClib's
  Transport<double> (transport.hpp:135-202) on the same inputs.
* A DXSource beam (source.hpp:379-677) on a 128^3 phantom of the batched
  radiography configuration.
* DOSE output mode (energyImpartedToDose, transport.hpp:796-816): keV/kg, and
  mGy through the DX dose-area-product calibration (source.hpp:552-568).

At 2e7 histories a 512 x 512 x 200 grid holds less than one deposit per body
voxel, so both sides are compared as block sums (8 x 8 x 4 voxels for CT, 4 x 4
x 4 for DX, 2 x 2 x 2 for the DOSE case) with the variance fields summed over
each block.  The reference's variance field sums squared deposits per event
(transport.hpp:601-629), which understates the spread of a block that one
history deposits in several times; the fixture carries chi2/dof of two
independent reference runs compared the same way, and that same-method value
replaces the default chi2/dof bound.  The GPU runs twice the reference's
histories.
"""
from __future__ import annotations

import numpy as np
import pytest

from parity import MAX_CHI2, assert_parity, block_sums, compare_sparse

pytestmark = pytest.mark.gpu


def _tables(g, scale=2):
    import dxmclib_gb300 as dx
    ex = g["exposures"]
    table = dx.ExposureTable(ex[:, 0:3].copy(), ex[:, 3:9].copy(), ex[:, 9:12].copy(), ex[:, 12:16].copy(),
                             ex[:, 16].copy(), (ex[:, 17] * scale).astype(np.uint64), np.zeros(len(ex)))
    spec = dx.Spectrum(g["spec_energies"], g["spec_weights"])
    hm = g["heel_meta"]
    heel = dx.HeelTable(hm[1], hm[2], int(hm[3]), hm[4], hm[5], int(hm[6]), g["heel_weights"]) if hm[0] > 0 else None
    return table, spec, heel


def _job(ctx, world, table, spec, heel, max_energy, seed, output, calibration=1.0):
    import dxmclib_gb300 as dx
    dworld = dx.DeviceWorld(ctx, world)
    blob = dx.LutBlob(world.materialMap(), dworld.max_density(), max_energy)
    dlut = dx.DeviceLut(ctx, blob)
    job = dx.Job(ctx, dworld, dlut, table, spec, heel, None, seed=seed, model=1)
    dose, var, nev, stats = job.result(output, calibration=calibration)
    assert stats["histories"] == int(np.sum(table.n_histories))
    assert stats["rejection_overflows"] == 0
    job.close()
    dlut.close()
    dworld.close()
    return dose, var, nev, stats


def _max_chi2(g):
    # chi2/dof of the reference against an independent reference run (same blocks)
    return max(MAX_CHI2, float(g["same_method"][0]))


def test_ct_helical_benchmark_configuration_matches_reference(gpu_ctx, golden):
    from dxmclib_gb300 import _capi as A
    from dxmclib_gb300.workloads import ct_world
    g = golden("bench_ct_helical.npz")
    dims, block = tuple(int(x) for x in g["dims"]), tuple(int(x) for x in g["block"])
    world = ct_world(int(dims[2]), seed=int(g["phantom_seed"]))
    assert tuple(world.dimensions()) == dims and np.allclose(world.spacing(), g["spacing"])
    table, spec, heel = _tables(g)
    dose, var, nev, stats = _job(gpu_ctx, world, table, spec, heel, float(g["max_energy"]), 2026,
                                    A.OUTPUT_EV_PER_HISTORY)
    s = compare_sparse(g, block_sums(dose, dims, block), block_sums(var, dims, block))
    assert_parity(s, "ct helical 512x512x200 (8x8x4 blocks)", max_chi2=_max_chi2(g))
    # events per history agree with the reference (a count, not a dose)
    ev_ratio = (nev.sum() / stats["histories"]) / (float(g["total_events"][0]) / float(g["histories"]))
    assert abs(ev_ratio - 1) < 0.01, ev_ratio


def test_dx_benchmark_configuration_matches_reference(gpu_ctx, golden):
    import dxmclib_gb300 as dx
    from dxmclib_gb300 import _capi as A
    from dxmclib_gb300.workloads import DX_MATERIALS
    g = golden("bench_dx.npz")
    dims, block = tuple(int(x) for x in g["dims"]), tuple(int(x) for x in g["block"])
    world = dx.World()
    world.setDimensions(dims)
    world.setSpacing(tuple(g["spacing"]))
    world.setDensityArray(g["density"])
    world.setMaterialIndexArray(g["material"])
    for n in DX_MATERIALS:
        world.addMaterialToMap(dx.Material(n))
    assert world.isValid()
    table, spec, heel = _tables(g)
    dose, var, nev, stats = _job(gpu_ctx, world, table, spec, heel, float(g["max_energy"]), 2027,
                                    A.OUTPUT_EV_PER_HISTORY)
    s = compare_sparse(g, block_sums(dose, dims, block), block_sums(var, dims, block))
    assert_parity(s, "dx 128^3 (4x4x4 blocks)", max_chi2=_max_chi2(g))


@pytest.mark.parametrize("mode", ["kevkg", "mgy"])
def test_dose_output_mode_matches_reference(gpu_ctx, golden, mode):
    """DOSE mode tallies the energy imparted per voxel mass (keV/kg) without
    normalising by the histories, and the variance as the squared-deposit sum
    times the same factor squared; with the DX source's calibration factor the
    unit is mGy.  Both sides are divided by the history count (dose / N,
    variance / N^2) so that runs of different length compare."""
    import dxmclib_gb300 as dx
    from dxmclib_gb300 import _capi as A
    from dxmclib_gb300.workloads import DX_MATERIALS
    g = golden("transport_dose_dx.npz")
    dims, block = tuple(int(x) for x in g["dims"]), tuple(int(x) for x in g["block"])
    world = dx.World()
    world.setDimensions(dims)
    world.setSpacing(tuple(g["spacing"]))
    world.setDensityArray(g["density"])
    world.setMaterialIndexArray(g["material"])
    for n in DX_MATERIALS:
        world.addMaterialToMap(dx.Material(n))
    table, spec, heel = _tables(g)
    n_ref = float(g["histories"])
    # the reference's factor is DAP / (N_ref * sum E w mu_en); the GPU run has twice the
    # histories, so its factor for the same DAP is half
    cal = float(g["calibration"]) * n_ref / float(np.sum(table.n_histories)) if mode == "mgy" else 1.0
    dose, var, nev, stats = _job(gpu_ctx, world, table, spec, heel, float(g["max_energy"]), 2028, A.OUTPUT_DOSE,
                                    calibration=cal)
    n_gpu = float(stats["histories"])
    ref = {k[len(mode) + 1:]: v for k, v in g.items() if k.startswith(mode + "_")}
    if mode == "mgy":  # mGy for the same dose-area product: independent of the history count
        ref_n = ref
        d_gpu, v_gpu = block_sums(dose, dims, block), block_sums(var, dims, block)
    else:  # keV/kg summed over histories: per history on both sides
        ref_n = dict(ref, dose=ref["dose"] / n_ref, var=ref["var"] / n_ref ** 2, total=ref["total"] / n_ref)
        d_gpu, v_gpu = block_sums(dose, dims, block) / n_gpu, block_sums(var, dims, block) / n_gpu ** 2
    s = compare_sparse(ref_n, d_gpu, v_gpu)
    assert_parity(s, f"dose mode {mode} (2x2x2 blocks)")


def _ct_dual_world(g):
    import dxmclib_gb300 as dx
    world = dx.World()
    world.setDimensions(tuple(int(x) for x in g["dims"]))
    world.setSpacing(tuple(float(x) for x in g["spacing"]))
    world.setDensityArray(g["density"])
    world.setMaterialIndexArray(g["material"])
    for n in g["names"]:
        world.addMaterialToMap(dx.Material(str(n)))
    assert world.isValid()
    return world


def test_dual_source_ct_matches_reference(gpu_ctx, golden):
    """A dual-source helical scan (CTSpiralDualSource, source.hpp:1488-1600: tubes
    of 140 and 80 kV taking turns, each with its own spectrum, heel table,
    distance, field of view and start angle) through the Python Transport, which
    runs one job per tube and normalises their summed tallies, against the
    reference's Transport<double> (2 x 2 x 2-voxel blocks)."""
    import dxmclib_gb300 as dx
    from dxmclib_gb300 import _capi as A
    g = golden("transport_ct_dual_m1.npz")
    world = _ct_dual_world(g)
    src = dx.CTSpiralDualSource()
    src.setPitch(1.0)
    src.tubeB().setVoltage(80)
    src.tubeB().setAlFiltration(6.0)
    src.setTubeAmas(100)
    src.setTubeBmas(250)
    src.setSourceDetectorDistanceB(1050)
    src.setFieldOfViewB(330)
    src.setStartAngleDegB(90)
    src.tube().setVoltage(140)
    src.tube().setAlFiltration(2.5)
    src.setPosition((0, 0, -20))
    src.setSourceDetectorDistance(1190)
    src.setCollimation(40)
    src.setFieldOfView(500)
    src.setStartAngleDeg(0)
    src.setExposureAngleStepDeg(2.0)
    src.setScanLenght(40)
    src.setHistoriesPerExposure(int(g["exposures"][0, 17]) * 2)
    ex = src.exposures(world.directionCosines()).as_matrix()
    ref_ex = g["exposures"].copy()
    ref_ex[:, 17] *= 2
    np.testing.assert_allclose(ex, ref_ex, rtol=0, atol=1e-9)
    tr = dx.Transport(gpu_ctx)
    tr.setOutputMode(dx.Transport.EV_PER_HISTORY)
    tr.setSeed(2031)
    res = tr(world, src)
    assert res.numberOfHistories == int(np.sum(ref_ex[:, 17]))
    dims, block = tuple(int(x) for x in g["dims"]), tuple(int(x) for x in g["block"])
    ref = {"idx": g["r_idx"], "dose": g["r_dose"], "var": g["r_var"], "total": g["r_total"]}
    s = compare_sparse(ref, block_sums(res.dose, dims, block), block_sums(res.variance, dims, block))
    assert_parity(s, "dual-source ct spiral (2x2x2 blocks)", max_chi2=_max_chi2(g))


def test_ct_bowtie_matches_reference(gpu_ctx, golden):
    """A CT helical scan through a bow-tie filter (CTSpiralSource::setBowTieFilter,
    source.hpp:821; BowTieFilter, beamfilters.hpp:65-197) through the Python
    Transport against the reference's Transport<double> of the same scan (2 x 2 x
    2-voxel blocks).  The filter's table is given unsorted and with a negative
    angle, so the product's table build (|angle|, sort, mean-1 weights) is tested
    along with the device's interpolation in the fan angle."""
    import dxmclib_gb300 as dx
    g = golden("transport_ct_bowtie_m1.npz")
    world = _ct_dual_world(g)
    src = dx.CTSpiralSource()
    src.setPitch(1.0)
    src.tube().setVoltage(120)
    src.tube().setAlFiltration(2.5)
    src.setPosition((0, 0, -20))
    src.setSourceDetectorDistance(1190)
    src.setCollimation(40)
    src.setFieldOfView(500)
    src.setStartAngleDeg(0)
    src.setExposureAngleStepDeg(1.0)
    src.setScanLenght(40)
    src.setBowTieFilter(g["bowtie_angles"], g["bowtie_weights"])
    src.setHistoriesPerExposure(int(g["exposures"][0, 17]) * 2)
    ex = src.exposures(world.directionCosines()).as_matrix()
    ref_ex = g["exposures"].copy()
    ref_ex[:, 17] *= 2
    np.testing.assert_allclose(ex, ref_ex, rtol=0, atol=1e-9)
    tr = dx.Transport(gpu_ctx)
    tr.setOutputMode(dx.Transport.EV_PER_HISTORY)
    tr.setSeed(2047)
    res = tr(world, src)
    assert res.numberOfHistories == int(np.sum(ref_ex[:, 17]))
    dims, block = tuple(int(x) for x in g["dims"]), tuple(int(x) for x in g["block"])
    ref = {"idx": g["r_idx"], "dose": g["r_dose"], "var": g["r_var"], "total": g["r_total"]}
    s = compare_sparse(ref, block_sums(res.dose, dims, block), block_sums(res.variance, dims, block))
    assert_parity(s, "ct spiral with bow-tie (2x2x2 blocks)", max_chi2=_max_chi2(g))


def test_ct_family_calibration_matches_reference(gpu_ctx, golden):
    """Source::getCalibrationValue of a dual-source spiral (CTAxialDualSource copy,
    both tubes in the CTDI run) and of a topogram (an axial copy stepping one
    collimation, source.hpp:1679-1701) as GPU jobs, against the reference's own
    CTDI runs of 1e8 histories; the tolerance of the single-tube calibration
    test, 2 %."""
    import dxmclib_gb300 as dx
    g = golden("ct_family_calibration_m1.npz")
    tr = dx.Transport(gpu_ctx)
    dual = dx.CTSpiralDualSource()
    dual.setPitch(1.2)
    dual.tubeB().setVoltage(80)
    dual.tubeB().setAlFiltration(6.0)
    dual.setTubeAmas(100)
    dual.setTubeBmas(250)
    dual.setSourceDetectorDistanceB(1050)
    dual.setFieldOfViewB(330)
    dual.setStartAngleDegB(90)
    dual.tube().setVoltage(140)
    dual.tube().setAlFiltration(2.5)
    dual.setCollimation(40)
    dual.setScanLenght(100)
    dual.setHistoriesPerExposure(1000)
    f = dual.getCalibrationValue(1, transport=tr)
    print(f"[calibration] dual-source spiral: {f:.6e} vs reference {float(g['spiral_dual']):.6e}")
    assert abs(f / float(g["spiral_dual"]) - 1.0) < 0.02
    topo = dx.CTTopogramSource()
    topo.tube().setVoltage(120)
    topo.tube().setAlFiltration(2.5)
    topo.setCollimation(10)
    topo.setScanLenght(300)
    topo.setHistoriesPerExposure(10000)
    f = topo.getCalibrationValue(1, transport=tr)
    print(f"[calibration] topogram: {f:.6e} vs reference {float(g['topogram']):.6e}")
    assert abs(f / float(g["topogram"]) - 1.0) < 0.02
