"""CPU tests of the host arithmetic of multi-beam transport (dual-source CT): the
per-beam seeds and the reference's normalisation of summed raw tallies
(Transport::normalizeScoring and energyImpartedToDose, transport.hpp:780-816)."""
from __future__ import annotations

import numpy as np
import pytest


def test_beam_seeds():
    from dxmclib_gb300.api import beam_seed
    assert beam_seed(12345, 0) == 12345
    seeds = {beam_seed(12345, k) for k in range(4)}
    assert len(seeds) == 4 and all(0 <= s < 1 << 64 for s in seeds)
    assert beam_seed((1 << 64) - 1, 1) == ((1 << 64) - 1 + 0x9E3779B97F4A7C15) % (1 << 64)


def test_normalize_scoring_matches_the_reference_formula():
    from dxmclib_gb300.api import normalize_scoring
    rng = np.random.default_rng(5)
    e = rng.uniform(0, 100, 50)
    e2 = e * e * rng.uniform(1, 3, 50)
    n = 1_000_000
    d, v = normalize_scoring(e, e2, n)
    np.testing.assert_allclose(d, e * 1e3 / n, rtol=1e-15)
    np.testing.assert_allclose(v, (e2 * 1e6 / n - (e * 1e3 / n) ** 2) / (n - 1), rtol=1e-12)


def test_energy_imparted_to_dose_skips_empty_voxels():
    import dxmclib_gb300 as dx
    from dxmclib_gb300.api import energy_imparted_to_dose
    w = dx.World()
    w.setDimensions((2, 2, 1))
    w.setSpacing((2.0, 2.0, 5.0))
    w.setDensityArray(np.array([1.0, 0.0, 2.0, 0.5], np.float32))
    w.setMaterialIndexArray(np.zeros(4, np.uint8))
    w.addMaterialToMap(dx.Material("Water, Liquid"))
    e = np.array([10.0, 7.0, 4.0, 1.0])
    e2 = e * e
    dose, var = energy_imparted_to_dose(w, e, e2, calibration=3.0)
    mass = np.array([1.0, 0.0, 2.0, 0.5]) * (2 * 2 * 5 / 1000.0) * 0.001
    expect = np.where(mass > 0, e * 3.0 / np.where(mass > 0, mass, 1), 0.0)
    np.testing.assert_allclose(dose, expect, rtol=1e-12)
    assert dose[1] == 0 and var[1] == 0
    np.testing.assert_allclose(var[[0, 2, 3]], (e2 * (3.0 / np.where(mass > 0, mass, 1)) ** 2)[[0, 2, 3]], rtol=1e-12)


def test_single_tube_sources_have_one_beam():
    import dxmclib_gb300 as dx
    p = dx.PencilSource()
    p.setTotalExposures(3)
    (b,) = p.beams()
    assert len(b.exposures) == 3 and b.spectrum is None and b.heel is None
