"""CPU tests of the dose-calibration host code: the CTDI phantom against the
reference's CTDIPhantom (world.hpp:229-390) entry by entry, the calibration
arithmetic of ctCalibration (source.hpp:943-987), and the axial calibration
exposures against the reference's own tables for the same CT spiral source."""
from __future__ import annotations

import numpy as np


def test_ctdi_phantom_matches_reference(golden):
    from dxmclib_gb300.calibration import CENTER, EAST, NORTH, SOUTH, WEST, CTDIPhantom
    g = golden("ctdi_phantom.npz")
    for d in (160, 320):
        w = CTDIPhantom(d)
        assert w.dimensions() == tuple(int(x) for x in g[f"d{d}_dims"])
        assert np.array_equal(np.bincount(w.materialIndexArray(), minlength=3), g[f"d{d}_material_counts"])
        assert np.array_equal(np.unique(w._density64), g[f"d{d}_densities"])
        holes = g[f"d{d}_holes"].astype(np.uint64)
        off = 0
        for pos, count in zip((CENTER, WEST, EAST, SOUTH, NORTH), g[f"d{d}_counts"]):
            assert np.array_equal(w.holeIndices(pos), holes[off:off + int(count)]), (d, pos)
            off += int(count)
        if d == 160:
            assert np.array_equal(w.materialIndexArray(), g["d160_material"])
            assert np.array_equal(w.measurementMapArray(), g["d160_measurement"])


def test_calibration_arithmetic():
    from dxmclib_gb300.calibration import CENTER, CTDIPhantom, calibration_histories_per_exposure, ctdi_factor
    w = CTDIPhantom(160)
    dose = np.zeros(w.size())
    dose[w.holeIndices(CENTER)] = 2.0
    for p in range(1, 5):
        dose[w.holeIndices(p)] = 4.0
    # CTDIw = (2 + 2 * 4) / 3 * 100 / 40 = 8.333..., factor = 10 / 8.333 / 0.5
    assert abs(ctdi_factor(w, dose, 40.0, 10.0, 0.5) - 10.0 / (10.0 / 3.0 * 2.5) / 0.5) < 1e-12
    assert calibration_histories_per_exposure(360, 1000) == 1000 * (100_000_000 // 360_000)
    assert calibration_histories_per_exposure(360, 10_000_000) == 10_000_000


def test_calibration_exposures_match_reference(golden):
    import dxmclib_gb300 as dx
    g = golden("ct_calibration_m1.npz")
    src = dx.CTSpiralSource()
    src.setPosition((0, 0, 0))
    src.tube().setVoltage(120.0)
    src.tube().setAlFiltration(2.5)
    src.setCollimation(40.0)
    src.setPitch(1.0)
    src.setScanLenght(100.0)
    src.setExposureAngleStepDeg(1.0)
    src.setFieldOfView(500.0)
    src.setSourceDetectorDistance(1190.0)
    src.setHistoriesPerExposure(1000)
    assert src.exposuresPerRotatition() == int(g["exposures_per_rotation"])
    from dxmclib_gb300.calibration import calibration_histories_per_exposure
    hpe = calibration_histories_per_exposure(src.exposuresPerRotatition(), src.historiesPerExposure())
    assert hpe == int(g["calibration_hpe"])
    ours = src.calibration_exposures(hpe).as_matrix()
    ref = g["exposures"]
    assert ours.shape == ref.shape
    np.testing.assert_allclose(ours[:, :17], ref[:, :17], atol=1e-9)
    assert np.array_equal(ours[:, 17], ref[:, 17])


class _SpectrumTube:
    """Stands in for a Tube with a given (energy, normalised weight) table."""

    def __init__(self, energies, weights):
        self.e, self.w = np.asarray(energies, np.float64), np.asarray(weights, np.float64)

    def getEnergy(self):
        return list(self.e)

    def getSpecter(self, energies=None, normalize=True):
        return list(self.w)

    def voltage(self):
        return float(self.e.max())


def test_dx_dap_calibration_matches_reference(golden):
    """DXSource::getCalibrationValue (source.hpp:552-568) on the reference's own spectrum:
    DAP / (N * sum_E E w(E) mu_en,air(E)), with mu_en from the physics model as the
    reference's Material::getMassEnergyAbsorbtion (material.cpp:56-59) gives it."""
    import dxmclib_gb300 as dx
    g = golden("transport_dose_dx.npz")
    src = dx.DXSource()
    src._tube = _SpectrumTube(g["spec_energies"], g["spec_weights"])
    src.setTotalExposures(8)
    src.setHistoriesPerExposure(int(g["histories"]) // 8)
    assert abs(src.getCalibrationValue(1) / float(g["calibration"]) - 1.0) < 1e-12


def test_ct_benchmark_exposures_match_reference(golden):
    """The exposure table of the benchmark's CT helical workload (workloads.ct_source)
    is the reference's CTSpiralSource table for the same settings."""
    from dxmclib_gb300.workloads import ct_source, ct_world
    g = golden("bench_ct_helical.npz")
    world = ct_world(int(g["dims"][2]), seed=int(g["phantom_seed"]))
    src = ct_source(world, int(g["histories"]))
    ours = src.exposures(world.directionCosines()).as_matrix()
    ref = g["exposures"]
    assert ours.shape == ref.shape
    np.testing.assert_allclose(ours[:, :17], ref[:, :17], atol=1e-9)
    assert np.array_equal(ours[:, 17], ref[:, 17])
    # and the same spectrum and heel table: the benchmark runs the reference's workload
    spec = src.spectrum()
    np.testing.assert_array_equal(spec.energies, g["spec_energies"])
    np.testing.assert_allclose(spec.weights, g["spec_weights"], rtol=1e-12)
    np.testing.assert_allclose(src.heel().weights, g["heel_weights"], rtol=1e-12, atol=1e-14)
