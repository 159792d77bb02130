"""CPU tests: the host-side tables of the GPU path against the reference.

Golden fixtures come from DXMClib itself (tests/golden/make_golden.py runs the
reference headers compiled unmodified with the project Material backend).
"""
from __future__ import annotations

import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parents[1]


def _materials(names):
    from dxmclib_gb300 import Material
    return [Material(str(n)) for n in names]


@pytest.mark.parametrize("max_energy", [60, 120])
def test_lut_tables_match_reference(lib, golden, max_energy):
    """AttenuationLut<double>::generate (attenuationlut.hpp:64-96) table by table."""
    from dxmclib_gb300 import LutBlob
    g = golden(f"lut_4mat_{max_energy}kev.npz")
    mats = _materials(g["names"])
    md = np.zeros(len(mats))
    np.maximum.at(md, g["material"].astype(np.int64), g["density"].astype(np.float64))
    blob = LutBlob(mats, md, float(g["max_energy"]))
    info = blob.info()
    meta = g["meta"]
    assert info["n_energy"] == int(meta[0])
    assert info["linear_index"] == int(meta[1])
    assert info["linear_step"] == pytest.approx(meta[2], rel=1e-14)
    assert info["linear_energy"] == pytest.approx(meta[3], rel=1e-14)
    assert info["min_energy"] == meta[4] and info["max_energy"] == meta[5]
    np.testing.assert_array_equal(info["x"], g["x"])
    np.testing.assert_allclose(info["coef"], g["coef"], rtol=0, atol=1e-9)
    np.testing.assert_allclose(info["maxcoef"], g["maxcoef"], rtol=0, atol=1e-9)
    # RITA form-factor and Compton scatter-factor tables: bit-exact
    np.testing.assert_array_equal(info["rita"], g["rita"])
    np.testing.assert_array_equal(info["spline"], g["spline"])
    np.testing.assert_allclose(info["shells"], g["shells"], rtol=1e-12, atol=1e-15)
    # public lookups on a dense energy grid
    E, q = g["energies"], g["q"]
    for m in range(len(mats)):
        att = np.array([blob.attenuation(m, e) for e in E])
        np.testing.assert_allclose(att, g["att"][m], rtol=1e-12)
        sf = np.array([blob.scatter_factor(m, x) for x in q])
        np.testing.assert_allclose(sf, g["sf"][m], rtol=1e-12, atol=1e-15)
    mi = np.array([blob.max_attenuation_inverse(e) for e in E])
    np.testing.assert_allclose(mi, g["maxinv"], rtol=1e-12)


def test_alias_tables_match_reference(lib, golden):
    """RandomDistribution::generateTable (dxmcrandom.hpp:229-274)."""
    from dxmclib_gb300 import _capi as A
    g = golden("alias.npz")
    k = 0
    while f"w{k}" in g:
        w = np.ascontiguousarray(g[f"w{k}"])
        p = np.zeros(len(w))
        a = np.zeros(len(w), np.uint64)
        assert lib.dxmc_alias_table(w.ctypes.data_as(A.DP), len(w), p.ctypes.data_as(A.DP), a.ctypes.data_as(A.U64P)) == 0
        np.testing.assert_array_equal(p, g[f"p{k}"])
        np.testing.assert_array_equal(a, g[f"a{k}"])
        k += 1
    assert k >= 4


def test_alias_table_distribution(lib):
    """Sampling the alias table reproduces the weights (statistical check of the table)."""
    from dxmclib_gb300 import _capi as A
    rng = np.random.default_rng(0)
    w = rng.uniform(0, 1, 40)
    p = np.zeros(40)
    a = np.zeros(40, np.uint64)
    lib.dxmc_alias_table(w.ctypes.data_as(A.DP), 40, p.ctypes.data_as(A.DP), a.ctypes.data_as(A.U64P))
    implied = p.copy()
    for k in range(40):
        implied[a[k]] += 1 - p[k]
    np.testing.assert_allclose(implied / 40, w / w.sum(), rtol=1e-12)


def _splitmix64(x):
    """SplitMix64 (Steele, Lea and Flood, OOPSLA 2014), restated in Python: returns
    (new counter, output)."""
    m = (1 << 64) - 1
    x = (x + 0x9E3779B97F4A7C15) & m
    z = x
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & m
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & m
    return x, z ^ (z >> 31)


def test_stream_seed_known_answers(lib):
    """The per-history stream state (SplitMix64 from the counter mix(seed) ^ history,
    two outputs, lowest bit of the last word set) against a Python restatement, for
    seeds and history ids across the 64-bit range; and neighbouring histories share
    no state word (an earlier seeding, seed ^ history * gamma, let history h's
    second word equal history h + 1's first for many seeds)."""
    from dxmclib_gb300 import _capi as A
    # SplitMix64 itself: its first two outputs from counter 0
    x, a = _splitmix64(0)
    x, b = _splitmix64(x)
    assert (a, b) == (0xE220A8397B1DCDAF, 0x6E789E6AA1B965F4)
    for seed in (0, 1, 11, 2026, 0xFFFFFFFFFFFFFFFF, 0x123456789ABCDEF0):
        words = set()
        for h in (0, 1, 2, 3, 255, 256, 1 << 32, (1 << 64) - 1):
            _, key = _splitmix64(seed)
            x = key ^ h
            x, a = _splitmix64(x)
            x, b = _splitmix64(x)
            want = [a & 0xFFFFFFFF, a >> 32, b & 0xFFFFFFFF, (b >> 32) | 1]
            o = np.zeros(4, np.uint32)
            assert lib.dxmc_stream_seed(seed, h, o.ctypes.data_as(A.U32P)) == 0
            assert o.tolist() == want, (seed, h)
            assert not words & {a, b}, (seed, h)
            words |= {a, b}


def _dx_source():
    import dxmclib_gb300 as dx
    s = dx.DXSource()
    s.tube().setVoltage(80)
    s.tube().setAlFiltration(3.0)
    s.setPosition((10, 5, -20))
    s.setSourceDetectorDistance(1000)
    s.setFieldSize((200, 150))
    s.setTubeRotationDeg(0)
    s.setSourceAnglesDeg(15, -10)
    s.setModelHeelEffect(True)
    s.setHistoriesPerExposure(800)
    s.setTotalExposures(2)
    return s


def _ct_source(tilt=False):
    import dxmclib_gb300 as dx
    s = dx.CTSpiralSource()
    if not tilt:
        s.tube().setVoltage(120)
        s.tube().setAlFiltration(2.5)
        s.setPosition((0, 0, -30))
        s.setSourceDetectorDistance(1190)
        s.setCollimation(40)
        s.setFieldOfView(500)
        s.setGantryTiltAngleDeg(0)
        s.setStartAngleDeg(0)
        s.setExposureAngleStepDeg(1.0)
        s.setPitch(1.0)
        s.setScanLenght(80)
    else:
        s.tube().setVoltage(100)
        s.tube().setAlFiltration(7.0)
        s.setPitch(1.5)
        s.setPosition((0, 0, 0))
        s.setSourceDetectorDistance(1000)
        s.setCollimation(20)
        s.setFieldOfView(400)
        s.setGantryTiltAngleDeg(12.0)
        s.setStartAngleDeg(30)
        s.setExposureAngleStepDeg(2.0)
        s.setScanLenght(40)
    s.setHistoriesPerExposure(100)
    return s


def test_source_exposure_tables_match_reference(lib, golden):
    """Source::getExposure + Exposure::alignToDirectionCosines for the host sources (source.hpp)."""
    import dxmclib_gb300 as dx
    pen = dx.PencilSource()
    pen.setPosition((3, -2, -300))
    pen.setDirectionCosines((1, 0, 0, 0, 1, 0))
    pen.setPhotonEnergy(60.0)
    pen.setHistoriesPerExposure(1000)
    pen.setTotalExposures(3)
    iso = dx.IsotropicSource()
    iso.setPosition((0, 0, -400))
    iso.setDirectionCosines((1, 0, 0, 0, 1, 0))
    iso.setCollimationAngles(-0.2, 0.2, -0.1, 0.15)
    iso.setSpecter(np.linspace(1, 3, 13), np.arange(20, 81, 5.0))
    iso.setHistoriesPerExposure(500)
    iso.setTotalExposures(2)
    cases = {"pencil": pen, "isotropic": iso, "dx": _dx_source(), "ctspiral": _ct_source(False),
             "ctspiral_tilt": _ct_source(True)}
    for name, src in cases.items():
        g = golden(f"source_{name}.npz")
        ex = src.exposures().as_matrix()
        assert ex.shape == g["exposures"].shape, name
        np.testing.assert_allclose(ex, g["exposures"], rtol=0, atol=1e-9, err_msg=name)
        assert src.maxPhotonEnergyProduced() == pytest.approx(g["max_energy"]), name


def test_heel_table_layout_matches_reference(lib, golden):
    """HeelFilter grid (beamfilters.hpp:455-505): energy bins and angular span."""
    g = golden("source_dx.npz")
    h = _dx_source().heel()
    meta = g["heel_meta"]
    assert meta[0] == 1
    assert (h.energy_start, h.energy_step, h.energy_size) == (meta[1], meta[2], int(meta[3]))
    assert h.angle_start == pytest.approx(meta[4], rel=1e-12)
    assert h.angle_step == pytest.approx(meta[5], rel=1e-12)
    assert h.angle_size == int(meta[6])
    # weights are normalised to mean 1 per energy bin, like the reference's
    w = h.weights.reshape(h.energy_size, h.angle_size)
    np.testing.assert_allclose(w.mean(axis=1), 1.0, rtol=1e-12)
    gw = g["heel_weights"].reshape(int(meta[3]), int(meta[6]))
    np.testing.assert_allclose(gw.mean(axis=1), 1.0, rtol=1e-12)


def test_tube_spectra_match_reference(lib, golden):
    """Tube::getSpecter (tube.hpp:191-261: thick-target Bethe-Heitler bremsstrahlung
    over the tabulated tungsten electron fluence, K lines, filtration, normalised)
    and the HeelFilter weight table (beamfilters.hpp:455-505) against the
    reference's, at 70-120 kV with Al and Cu filtration and two anode angles."""
    import dxmclib_gb300 as dx
    g = golden("tube_spectra.npz")
    for k in range(int(g["n"])):
        kvp, al, cu, anode = g[f"case{k}"]
        src = dx.DXSource()
        src.tube().setVoltage(kvp)
        src.tube().setAnodeAngleDeg(anode)
        src.tube().setAlFiltration(al)
        if cu > 0:
            src.tube().setCuFiltration(cu)
        src.setFieldSize((300, 200))
        src.setSourceDetectorDistance(1000)
        e = src.tube().getEnergy()
        np.testing.assert_array_equal(e, g[f"energies{k}"])
        np.testing.assert_allclose(src.tube().getSpecter(e), g[f"weights{k}"], rtol=1e-12, atol=1e-300, err_msg=str(kvp))
        h = src.heel()
        meta = g[f"heel_meta{k}"]
        assert (h.energy_start, h.energy_step, h.energy_size, h.angle_size) == (meta[1], meta[2], int(meta[3]), int(meta[6]))
        assert h.angle_start == pytest.approx(meta[4], rel=1e-12) and h.angle_step == pytest.approx(meta[5], rel=1e-12)
        np.testing.assert_allclose(h.weights, g[f"heel_weights{k}"], rtol=1e-12, atol=1e-14, err_msg=f"heel {kvp}")


def test_tube_spectrum_is_physical(lib):
    import dxmclib_gb300 as dx
    t = dx.Tube(120)
    t.setAlFiltration(2.5)
    e = t.getEnergy()
    s = t.getSpecter(e)
    assert e[0] == 1 and e[-1] == 120 and len(e) == 120
    assert s.sum() == pytest.approx(1.0)
    mean = float((e * s).sum())
    assert 45 < mean < 70
    assert s[:10].sum() < 1e-6  # filtered away
    t2 = dx.Tube(120)
    t2.setAlFiltration(6.0)
    assert float((e * t2.getSpecter(e)).sum()) > mean  # more filtration hardens the beam


def test_capi_exports_every_declared_symbol(lib):
    header = (REPO / "include" / "dxmc_gpu.h").read_text()
    names = set(re.findall(r"^\s*(?:const\s+)?\w+[\s\*]+(dxmc_\w+)\s*\(", header, re.MULTILINE))
    assert len(names) >= 25
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing
    assert lib.dxmc_gpu_abi_version() == 3


def test_bowtie_table_matches_reference(lib, golden):
    """The table jobs sample bow-tie weights from (dxmc_bowtie_table) equals the
    reference's BowTieFilter<double> table (beamfilters.hpp:102-130: |angle|,
    sorted, weights over their mean), given unsorted and with a negative angle."""
    from dxmclib_gb300 import _capi as A
    g = golden("bowtie.npz")
    a = np.ascontiguousarray(g["angles"], np.float64)
    w = np.ascontiguousarray(g["weights"], np.float64)
    ta, tw = np.zeros(len(a)), np.zeros(len(a))
    assert lib.dxmc_bowtie_table(a.ctypes.data_as(A.DP), w.ctypes.data_as(A.DP), len(a), ta.ctypes.data_as(A.DP),
                                 tw.ctypes.data_as(A.DP)) == A.DXMC_OK
    np.testing.assert_array_equal(ta, g["table_angles"])
    np.testing.assert_allclose(tw, g["table_weights"], rtol=1e-15, atol=0)
    # sampleIntensityWeight (beamfilters.hpp:150-190): clamped at both ends, linear
    # between the bracketing nodes; the device's binary search brackets the same pair
    q = np.abs(g["queries"])
    expect = np.interp(q, ta, tw)
    np.testing.assert_allclose(g["query_weights"], expect, rtol=1e-13, atol=0)
    zeros = np.zeros(3)
    assert lib.dxmc_bowtie_table(a.ctypes.data_as(A.DP), zeros.ctypes.data_as(A.DP), 3, ta.ctypes.data_as(A.DP),
                                 tw.ctypes.data_as(A.DP)) == A.DXMC_ERR_INVALID
    assert lib.dxmc_bowtie_table(a.ctypes.data_as(A.DP), w.ctypes.data_as(A.DP), 0, ta.ctypes.data_as(A.DP),
                                 tw.ctypes.data_as(A.DP)) == A.DXMC_ERR_INVALID
    # beyond DXMC_MAX_BOWTIE_POINTS (1 << 20): rejected before anything is read
    assert lib.dxmc_bowtie_table(a.ctypes.data_as(A.DP), w.ctypes.data_as(A.DP), (1 << 20) + 1,
                                 ta.ctypes.data_as(A.DP), tw.ctypes.data_as(A.DP)) == A.DXMC_ERR_INVALID


def test_invalid_inputs_are_rejected(lib):
    from dxmclib_gb300 import _capi as A
    prov = A.MaterialProvider()
    assert lib.dxmc_physics_material(b"NotAMaterial42", -1.0, C.byref(prov)) == A.DXMC_ERR_INVALID
    assert lib.dxmc_physics_material(b"H2O", -1.0, C.byref(prov)) == A.DXMC_ERR_INVALID  # formula without density
    # counts the number parser throws on (out of double range, a lone point): a status, not an
    # exception across the C ABI
    for bad_formula in (b"H" + b"9" * 400 + b"O", b"H.O", b"H2O."):
        assert lib.dxmc_physics_material(bad_formula, 1.0, C.byref(prov)) == A.DXMC_ERR_INVALID, bad_formula
    assert lib.dxmc_physics_material(b"H2O", 1.0, C.byref(prov)) == A.DXMC_OK
    blob = C.c_void_p()
    md = np.array([1.0])
    assert lib.dxmc_lut_build_max_density(C.byref(prov), 0, md.ctypes.data_as(A.DP), 60.0, C.byref(blob)) == A.DXMC_ERR_INVALID
    assert lib.dxmc_lut_build_max_density(C.byref(prov), 1, md.ctypes.data_as(A.DP), -5.0, C.byref(blob)) == A.DXMC_ERR_INVALID
    lib.dxmc_physics_material_free(C.byref(prov))


def test_invariant_division_is_exact(lib):
    """The kernels map a history id to its exposure with a multiply-high and two
    shifts instead of a division (udiv_magic / udiv_apply); it must equal n / d
    for every 32-bit n and divisor."""
    from dxmclib_gb300 import _capi as A
    rng = np.random.default_rng(11)
    n = np.concatenate([rng.integers(0, 2 ** 32, 200_000, dtype=np.uint64),
                        np.array([0, 1, 2, 3, 2 ** 31 - 1, 2 ** 31, 2 ** 32 - 2, 2 ** 32 - 1], np.uint64)]).astype(np.uint32)
    divisors = [1, 2, 3, 5, 7, 10, 22223, 65535, 65536, 65537, 2 ** 31 - 1, 2 ** 31, 2 ** 31 + 1, 2 ** 32 - 1]
    divisors += [int(d) for d in rng.integers(2, 2 ** 32, 40, dtype=np.uint64)]
    out = np.zeros_like(n)
    for d in divisors:
        assert lib.dxmc_udiv_invariant(n.ctypes.data_as(A.U32P), len(n), d, out.ctypes.data_as(A.U32P)) == 0
        np.testing.assert_array_equal(out, n // np.uint32(d), err_msg=str(d))
        # the multiples of d and their neighbours, where rounding would show
        k = (n[:1000].astype(np.uint64) % (2 ** 32 // d + 1)) * d
        m = np.concatenate([k, k + 1, np.where(k > 0, k - 1, 0)])
        m = m[m < 2 ** 32].astype(np.uint32)
        o2 = np.zeros_like(m)
        assert lib.dxmc_udiv_invariant(m.ctypes.data_as(A.U32P), len(m), d, o2.ctypes.data_as(A.U32P)) == 0
        np.testing.assert_array_equal(o2, m // np.uint32(d), err_msg=str(d))
