"""CPU tests: the oracle port (oracle/port, a C++ restatement of DXMClib's
transport) against the reference's own results (golden fixtures), so the
port can stand in for the reference where the reference cannot be built."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

from parity import assert_parity, compare_sparse

REPO = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(REPO / "oracle" / "port"))
import binding as port  # noqa: E402


def _lut(names, material, density, max_energy):
    import dxmclib_gb300 as dx
    mats = [dx.Material(str(n)) for n in names]
    md = np.zeros(len(mats))
    np.maximum.at(md, np.asarray(material, np.int64).ravel(), np.asarray(density, np.float64).ravel())
    return dx.LutBlob(mats, md, max_energy).info()


def _pencil_exposures(histories):
    import dxmclib_gb300 as dx
    s = dx.PencilSource()
    s.setPosition((0, 0, -200))
    s.setPhotonEnergy(60.0)
    s.setTotalExposures(10)
    s.setHistoriesPerExposure(histories // 10)
    m = s.exposures().as_matrix()
    m[:, 18] = 60.0
    return m


@pytest.mark.parametrize("model", [0, 1, 2])
def test_port_pencil_matches_reference(lib, golden, model):
    g = golden(f"transport_pencil_m{model}.npz")
    n = 64
    mat = np.zeros(n ** 3, np.uint8)
    dens = np.ones(n ** 3)
    info = _lut(["Water, Liquid"], mat, dens, 60.0)
    N = int(g["histories"])
    e, e2, nev, secs, steps = port.transport(info, (n, n, n), (2, 2, 2), dens, mat, _pencil_exposures(N), model=model,
                                             seed=17 + model)
    d, v = port.ev_per_history(e, e2, N)
    assert_parity(compare_sparse(g, d, v), f"port pencil m{model}")


def test_port_cone_matches_reference(lib, golden):
    import dxmclib_gb300 as dx
    g = golden("transport_cone_m1.npz")
    dims = tuple(int(x) for x in g["dims"])
    info = _lut(g["names"], g["material"], g["density"], float(g["spec_energies"].max()))
    src = dx.IsotropicSource()
    src.setPosition((0, 0, -500))
    src.setCollimationAngles(-0.12, 0.12, -0.1, 0.1)
    src.setSpecter(g["spec_weights"], g["spec_energies"])
    src.setTotalExposures(8)
    N = int(g["histories"])
    src.setHistoriesPerExposure(N // 8)
    e, e2, nev, secs, steps = port.transport(info, dims, tuple(g["spacing"]), g["density"], g["material"],
                                             src.exposures().as_matrix(), model=1, seed=5,
                                             spectrum=(g["spec_energies"], g["spec_weights"]))
    d, v = port.ev_per_history(e, e2, N)
    assert_parity(compare_sparse(g, d, v), "port cone m1")


def test_port_ct_matches_reference(lib, golden):
    g = golden("transport_ct_m1.npz")
    dims = tuple(int(x) for x in g["dims"])
    info = _lut(g["names"], g["material"], g["density"], float(g["max_energy"]))
    hm = g["heel_meta"]
    heel = dict(energy_start=hm[1], energy_step=hm[2], energy_size=hm[3], angle_start=hm[4], angle_step=hm[5],
                angle_size=hm[6], weights=g["heel_weights"])
    e, e2, nev, secs, steps = port.transport(info, dims, tuple(g["spacing"]), g["density"], g["material"],
                                             g["exposures"], model=1, seed=9,
                                             spectrum=(g["spec_energies"], g["spec_weights"]), heel=heel)
    d, v = port.ev_per_history(e, e2, int(g["histories"]))
    assert_parity(compare_sparse(g, d, v), "port ct")


def test_port_ct_bowtie_matches_reference(lib, golden):
    """A CT helical scan through a bow-tie filter (BowTieFilter, beamfilters.hpp:65-197:
    |angle|, sorted, weights normalised to mean 1, interpolated in the fan angle)
    against the reference's own transport of the same scan, as 2 x 2 x 2 block sums."""
    from parity import block_sums
    g = golden("transport_ct_bowtie_m1.npz")
    dims = tuple(int(x) for x in g["dims"])
    info = _lut(g["names"], g["material"], g["density"], float(g["max_energy"]))
    hm = g["heel_meta"]
    heel = dict(energy_start=hm[1], energy_step=hm[2], energy_size=hm[3], angle_start=hm[4], angle_step=hm[5],
                angle_size=hm[6], weights=g["heel_weights"])
    e, e2, nev, secs, steps = port.transport(info, dims, tuple(g["spacing"]), g["density"], g["material"],
                                             g["exposures"], model=1, seed=13,
                                             spectrum=(g["spec_energies"], g["spec_weights"]), heel=heel,
                                             bowtie=(g["bowtie_angles"], g["bowtie_weights"]))
    d, v = port.ev_per_history(e, e2, int(g["histories"]))
    block = tuple(int(x) for x in g["block"])
    ref = {"idx": g["r_idx"], "dose": g["r_dose"], "var": g["r_var"], "total": g["r_total"]}
    s = compare_sparse(ref, block_sums(d, dims, block), block_sums(v, dims, block))
    assert_parity(s, "port ct bow-tie (2x2x2 blocks)", max_chi2=max(1.2, float(g["same_method"][0])))


def test_port_forced_matches_reference(lib, golden):
    import dxmclib_gb300 as dx
    g = golden("transport_forced_m1.npz")
    dims = tuple(int(x) for x in g["dims"])
    n = int(np.prod(dims))
    mat = np.zeros(n, np.uint8)
    dens = np.ones(n)
    info = _lut(["Water, Liquid"], mat, dens, 50.0)
    src = dx.IsotropicSource()
    src.setPosition((0, 0, -300))
    src.setCollimationAngles(-0.05, 0.05, -0.05, 0.05)
    src.setSpecter([1.0], [50.0])
    src.setTotalExposures(8)
    N = int(g["histories"])
    src.setHistoriesPerExposure(N // 8)
    e, e2, nev, secs, steps = port.transport(info, dims, tuple(g["spacing"]), dens, mat, src.exposures().as_matrix(),
                                             model=1, seed=3, spectrum=([50.0], [1.0]), measurement=g["measurement"])
    d, v = port.ev_per_history(e, e2, N)
    assert_parity(compare_sparse(g, d, v), "port forced", correlated=True)


def _cone_setup(n, histories_per_exposure):
    import dxmclib_gb300 as dx
    world = dx.World()
    world.setDimensions((n, n, n))
    world.setSpacing((2.0, 2.0, 2.0))
    world.setDensityArray(np.ones(n ** 3, np.float32))
    world.setMaterialIndexArray(np.zeros(n ** 3, np.uint8))
    world.addMaterialToMap(dx.Material("Water, Liquid"))
    assert world.isValid()
    src = dx.IsotropicSource()
    src.setPosition((0, 0, -200))
    src.setCollimationAngles(-0.08, 0.08, -0.08, 0.08)
    src.setSpecter([1.0], [60.0])
    src.setTotalExposures(20)
    src.setHistoriesPerExposure(histories_per_exposure)
    blob = dx.LutBlob(world.materialMap(), [1.0], 60.0)
    return world, src, blob


def test_port_normalized_direction_mode():
    """The normalised physics mode (unit scattering axis in peturb; no reference
    counterpart) changes the transport: the reference's shrinking directions keep
    scattered photons in a water cube longer, so it imparts about 0.8 % more
    energy than the normalised mode (1e6 histories per run, about 0.1 % noise)."""
    n = 32
    world, src, blob = _cone_setup(n, 50_000)
    sp = src.spectrum()
    tot = {}
    for norm in (False, True):
        e, _, _, _, _ = port.transport(blob.info(), (n, n, n), (2.0,) * 3, np.ones(n ** 3), np.zeros(n ** 3, np.uint8),
                                       src.exposures().as_matrix(), model=1, seed=3,
                                       spectrum=(sp.energies, sp.weights), normalized_direction=norm)
        tot[norm] = e.sum() / 1e6
    assert 0.003 < tot[False] / tot[True] - 1.0 < 0.015, tot


@pytest.mark.parametrize("precision", ["double", "float"])
def test_port_ct_benchmark_configuration_matches_reference(golden, precision):
    """The port on the headline CT helical workload (512 x 512 x 200, the reference's
    own exposure, spectrum, heel and LUT tables from the fixture; no product code),
    in both precisions, against Transport<double> as 8 x 8 x 4 block sums.  This is
    the configuration and the code path bench.py's CPU legs time."""
    from parity import block_sums
    from dxmclib_gb300.workloads import ct_phantom_arrays
    g = golden("bench_ct_helical.npz")
    dims, block = tuple(int(x) for x in g["dims"]), tuple(int(x) for x in g["block"])
    mat, dens = ct_phantom_arrays(*dims, spacing=tuple(g["spacing"]), seed=int(g["phantom_seed"]))
    hm = g["heel_meta"]
    heel = dict(energy_start=hm[1], energy_step=hm[2], energy_size=hm[3], angle_start=hm[4], angle_step=hm[5],
                angle_size=hm[6], weights=g["heel_weights"])
    ex = g["exposures"].copy()
    ex[:, 17] = ex[:, 17] // 2
    n = int(ex[:, 17].sum())
    e, e2, nev, secs, steps = port.transport(port.lut_from_fixture(g), dims, tuple(g["spacing"]), dens, mat, ex,
                                             model=1, seed=5, spectrum=(g["spec_energies"], g["spec_weights"]),
                                             heel=heel, precision=precision)
    d, v = port.ev_per_history(e, e2, n)
    s = compare_sparse(g, block_sums(d, dims, block), block_sums(v, dims, block))
    assert_parity(s, f"port {precision} ct helical 512x512x200", max_chi2=max(1.2, float(g["same_method"][0])))


def test_port_dx_benchmark_configuration_matches_reference(lib, golden):
    """The port on the batched-radiography phantom (128^3, a DXSource beam with the
    reference's own exposure, spectrum and heel tables) against Transport<double>
    as 4 x 4 x 4 block sums, at half the reference's histories."""
    from parity import block_sums
    from dxmclib_gb300.workloads import DX_MATERIALS
    g = golden("bench_dx.npz")
    dims, block = tuple(int(x) for x in g["dims"]), tuple(int(x) for x in g["block"])
    info = _lut(DX_MATERIALS, g["material"], g["density"], float(g["max_energy"]))
    hm = g["heel_meta"]
    heel = dict(energy_start=hm[1], energy_step=hm[2], energy_size=hm[3], angle_start=hm[4], angle_step=hm[5],
                angle_size=hm[6], weights=g["heel_weights"])
    ex = g["exposures"].copy()
    ex[:, 17] = ex[:, 17] // 2
    n = int(ex[:, 17].sum())
    e, e2, nev, secs, steps = port.transport(info, dims, tuple(g["spacing"]), g["density"], g["material"], ex,
                                             model=1, seed=21, spectrum=(g["spec_energies"], g["spec_weights"]),
                                             heel=heel)
    d, v = port.ev_per_history(e, e2, n)
    s = compare_sparse(g, block_sums(d, dims, block), block_sums(v, dims, block))
    assert_parity(s, "port dx 128^3 (4x4x4 blocks)", max_chi2=max(1.2, float(g["same_method"][0])))
