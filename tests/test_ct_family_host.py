"""CPU tests of the CT source family of the Python mirror against the reference:
axial (a step other than the collimation, gantry tilt), spiral and axial
dual-source (tube B, tube currents, its own distance, field of view and start
angle) and topogram (source.hpp:1192-1702).  The fixtures hold the reference's
Source::getExposure tables after alignToDirectionCosines, and the spectrum and
heel tables its exposures 0 (tube A) and 1 (tube B) sample with
(tests/golden/make_golden.py, step ct_family)."""
from __future__ import annotations

import numpy as np
import pytest


def _common(s, kvp, al, position, sdd, coll, fov, tilt, start, hpe, heel=True):
    s.tube().setVoltage(kvp)
    s.tube().setAlFiltration(al)
    s.setPosition(position)
    s.setSourceDetectorDistance(sdd)
    s.setCollimation(coll)
    s.setFieldOfView(fov)
    s.setGantryTiltAngleDeg(tilt)
    s.setStartAngleDeg(start)
    s.setModelHeelEffect(heel)
    s.setHistoriesPerExposure(hpe)


def _tube_b(s, kvp, al, cu, mas_a, mas_b, sdd_b, fov_b, start_b):
    s.tubeB().setVoltage(kvp)
    s.tubeB().setAlFiltration(al)
    if cu > 0:
        s.tubeB().setCuFiltration(cu)
    s.setTubeAmas(mas_a)
    s.setTubeBmas(mas_b)
    s.setSourceDetectorDistanceB(sdd_b)
    s.setFieldOfViewB(fov_b)
    s.setStartAngleDegB(start_b)


def ct_family_sources():
    """The sources of make_golden.ct_family_cases, set up through the mirror's API."""
    import dxmclib_gb300 as dx
    axial = dx.CTAxialSource()
    axial.setStep(25)
    _common(axial, 100, 3.0, (0, 0, -20), 1100, 20, 450, 5.0, 15, 100)
    axial.setExposureAngleStepDeg(3.0)
    axial.setScanLenght(50)

    sdual = dx.CTSpiralDualSource()
    sdual.setPitch(1.2)
    _tube_b(sdual, 80, 6.0, 0.1, 120, 200, 1000, 330, 100)
    _common(sdual, 140, 2.5, (0, 0, -30), 1190, 40, 500, 0.0, 10, 100)
    sdual.setExposureAngleStepDeg(2.0)
    sdual.setScanLenght(60)

    adual = dx.CTAxialDualSource()
    adual.setStep(30)
    _tube_b(adual, 100, 4.0, 0.0, 200, 100, 1190, 260, 95)
    _common(adual, 120, 2.5, (0, 0, 0), 1190, 20, 500, 8.0, 0, 100, heel=False)
    adual.setExposureAngleStepDeg(5.0)
    adual.setScanLenght(60)

    topo = dx.CTTopogramSource()
    _common(topo, 120, 2.5, (0, 0, -30), 1190, 10, 500, 0.0, 30, 100)
    topo.setScanLenght(300)
    return {"ctaxial": axial, "ctspiral_dual": sdual, "ctaxial_dual": adual, "cttopogram": topo}


@pytest.mark.parametrize("name", ["ctaxial", "ctspiral_dual", "ctaxial_dual", "cttopogram"])
def test_ct_family_exposures_match_reference(lib, golden, name):
    src = ct_family_sources()[name]
    g = golden(f"source_{name}.npz")
    ex = src.exposures().as_matrix()
    assert ex.shape == g["exposures"].shape
    np.testing.assert_allclose(ex, g["exposures"], rtol=0, atol=1e-9)
    assert src.maxPhotonEnergyProduced() == pytest.approx(float(g["max_energy"]))
    assert src.totalExposures() == len(g["exposures"])


def _check_heel(table, g, prefix):
    meta = g[f"{prefix}heel_meta"]
    if table is None:
        assert meta[0] == 0
        return
    assert meta[0] == 1
    assert (table.energy_start, table.energy_step, table.energy_size, table.angle_size) == \
        (meta[1], meta[2], int(meta[3]), int(meta[6]))
    assert table.angle_start == pytest.approx(meta[4], rel=1e-12)
    assert table.angle_step == pytest.approx(meta[5], rel=1e-12)
    np.testing.assert_allclose(table.weights, g[f"{prefix}heel_weights"], rtol=1e-12, atol=1e-14)


@pytest.mark.parametrize("name", ["ctspiral_dual", "ctaxial_dual"])
def test_dual_source_beams_match_reference(lib, golden, name):
    """Each tube's beam: its exposures (every other one), spectrum and heel table
    (CTDualSource::updateSpecterDistribution builds both heel tables whatever
    modelHeelEffect says, source.hpp:1150-1175), and the tube weights in the
    exposures (mAs times the unnormalised spectrum, normalised to a mean of one)."""
    from dxmclib_gb300 import _capi as A

    def _alias_table(weights):
        w = np.ascontiguousarray(weights, np.float64)
        p = np.zeros(len(w))
        a = np.zeros(len(w), np.uint64)
        assert lib.dxmc_alias_table(w.ctypes.data_as(A.DP), len(w), p.ctypes.data_as(A.DP), a.ctypes.data_as(A.U64P)) == 0
        return p, a

    src = ct_family_sources()[name]
    g = golden(f"source_{name}.npz")
    beams = src.beams()
    assert len(beams) == 2
    ex = g["exposures"]
    for k, b in enumerate(beams):
        np.testing.assert_allclose(b.exposures.as_matrix(), ex[k::2], rtol=0, atol=1e-9)
        _check_heel(b.heel, g, f"x{k}_")
        probs, alias = _alias_table(b.spectrum.weights)
        np.testing.assert_allclose(probs, g[f"x{k}_spec_probs"], rtol=1e-12, atol=1e-300)
        np.testing.assert_array_equal(alias, g[f"x{k}_spec_alias"])
    np.testing.assert_array_equal(beams[1].spectrum.energies, g["x1_tube_b_energies"])
    np.testing.assert_allclose(beams[1].spectrum.weights, g["x1_tube_b_weights"], rtol=1e-12, atol=1e-300)
    wa, wb = src.tubeWeights()
    np.testing.assert_allclose(ex[0::2, 16], wa, rtol=1e-12)
    np.testing.assert_allclose(ex[1::2, 16], wb, rtol=1e-12)
    assert wa + wb == pytest.approx(2.0)


def test_single_tube_ct_sources_have_one_beam(lib, golden):
    srcs = ct_family_sources()
    for name in ("ctaxial", "cttopogram"):
        g = golden(f"source_{name}.npz")
        (b,) = srcs[name].beams()
        _check_heel(b.heel, g, "x0_")
        np.testing.assert_allclose(b.exposures.as_matrix(), g["exposures"], rtol=0, atol=1e-9)


def test_cbct_and_isotropic_ct_exposures_match_reference(lib, golden):
    """CBCTSource (source.hpp:679-782: the tube at half the source-detector distance,
    rotating about the second direction cosine) and IsotropicCTSource
    (source.hpp:346-377: rotation about z over the exposures)."""
    import dxmclib_gb300 as dx
    cb = dx.CBCTSource()
    cb.tube().setVoltage(90)
    cb.tube().setAlFiltration(4.0)
    cb.setPosition((5, -3, 10))
    cb.setSourceDetectorDistance(600)
    cb.setFieldSize((250, 200))
    cb.setSourceAnglesDeg(20, -15)
    cb.setSpanAngleDeg(200)
    cb.setStepAngleDeg(2.5)
    cb.setModelHeelEffect(True)
    cb.setHistoriesPerExposure(100)
    iso = dx.IsotropicCTSource()
    iso.setPosition((0, -300, 20))
    iso.setDirectionCosines((1, 0, 0, 0, 0, 1))
    iso.setCollimationAngles(-0.3, 0.3, -0.05, 0.05)
    iso.setSpecter(np.linspace(1, 3, 13), np.arange(20, 81, 5.0))
    iso.setHistoriesPerExposure(100)
    iso.setTotalExposures(36)
    for name, src in (("cbct", cb), ("isotropic_ct", iso)):
        g = golden(f"source_{name}.npz")
        ex = src.exposures().as_matrix()
        assert ex.shape == g["exposures"].shape, name
        np.testing.assert_allclose(ex, g["exposures"], rtol=0, atol=1e-9, err_msg=name)
        assert src.maxPhotonEnergyProduced() == pytest.approx(float(g["max_energy"])), name
    g = golden("source_cbct.npz")
    h = cb.heel()
    meta = g["heel_meta"]
    assert (h.energy_size, h.angle_size) == (int(meta[3]), int(meta[6]))
    np.testing.assert_allclose(h.weights, g["heel_weights"], rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(cb.spectrum().weights, g["spec_weights"], rtol=1e-12, atol=1e-300)
