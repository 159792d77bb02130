"""Generate the golden fixtures in tests/golden/ from the reference itself.

Runs DXMClib (headers compiled unmodified from the reference checkout, plus
the project Material backend; see oracle/Makefile) through
tests/golden/ref_binding.py and stores, as small .npz files:

* lut_*.npz         AttenuationLut<double> tables and public lookups for a
                    4-material world (attenuationlut.hpp, attenuationinterpolator.hpp);
* alias.npz         SpecterDistribution alias tables (dxmcrandom.hpp:229-274);
* source_*.npz      Source::getExposure tables, spectrum and heel tables for
                    Pencil / Isotropic / DX / CT spiral sources (source.hpp);
* transport_*.npz   Transport<double> tallies in EV_PER_HISTORY mode for the
                    pencil-beam and heterogeneous cone-beam cases, stored
                    for voxels above 0.2 % of the maximum dose plus depth and
                    lateral profiles and the total energy imparted;
* interactions_*.npz histograms of the reference interaction samplers;
* ctdi_phantom.npz  CTDIPhantom arrays and hole lists (world.hpp:229-390);
* ct_calibration_m1.npz the reference's CT calibration factor and the tables of
                    the axial copy it runs (source.hpp:925-988);
* bench_ct_helical.npz Transport<double> on the 512 x 512 x 200 CT helical
                    workload (the benchmark's headline configuration), as block
                    sums of 8 x 8 x 4 voxels, with the reference's exposure,
                    spectrum and heel tables, its LUT tables for the phantom and
                    the statistics of a second, independent reference run
                    against the first (the per-event variance estimator's
                    over-dispersion at this block size);
* bench_dx.npz      the same for a DXSource beam on a 128^3 phantom of the
                    batched-radiography configuration (4 x 4 x 4 blocks);
* tube_spectra.npz  Tube::getSpecter spectra and HeelFilter weights at 70-120 kV
                    with Al / Cu filtration and two anode angles;
* transport_dose_dx.npz Transport<double> in DOSE mode (mGy through the DX
                    dose-area-product calibration, and keV/kg without it) on a
                    64^3 DX phantom, 2 x 2 x 2 block sums, with the factor;
* bowtie.npz        BowTieFilter<double>'s normalised table and
                    sampleIntensityWeight at query angles (beamfilters.hpp:65-197);
* transport_ct_bowtie_m1.npz Transport<double> of a CT helical scan through a
                    bow-tie filter (2 x 2 x 2 block sums, two independent runs).

Usage:  make -C oracle REF=<reference checkout> && python tests/golden/make_golden.py [--quick]
The generator needs the reference checkout and is not run by the test suite.
"""
from __future__ import annotations

import argparse
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))
import ref_binding as R  # noqa: E402

MATERIALS4 = ["Water, Liquid", "Bone, Cortical (ICRP)", "Tissue, Soft (ICRP)", "Air, Dry (near sea level)"]


def hetero_world(n=48, spacing=4.0, seed=7):
    """Seeded heterogeneous phantom: soft-tissue box with bone and lung-density inclusions in air."""
    rng = np.random.default_rng(seed)
    z, y, x = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    c = (n - 1) / 2
    mat = np.full((n, n, n), 3, np.uint8)  # air
    body = ((x - c) / (0.42 * n)) ** 2 + ((y - c) / (0.32 * n)) ** 2 <= 1.0
    mat[body] = 2
    dens = np.where(mat == 3, 0.0012, 1.03).astype(np.float64)
    for _ in range(6):
        cx, cy, cz = rng.uniform(0.3 * n, 0.7 * n, 3)
        r = rng.uniform(0.05 * n, 0.12 * n)
        sph = (x - cx) ** 2 + (y - cy) ** 2 + (z - cz) ** 2 <= r * r
        sph &= body
        m = int(rng.integers(0, 2))
        mat[sph] = m
        dens[sph] = rng.uniform(0.2, 2.0)
    return mat.ravel(), dens.ravel()


def sparse_tally(dose, var, nev, dims, frac=0.002):
    d3 = dose.reshape(dims[2], dims[1], dims[0])
    keep = np.nonzero(dose > frac * dose.max())[0].astype(np.uint32)
    return dict(
        idx=keep, dose=dose[keep], var=var[keep], nev=nev[keep].astype(np.uint32),
        depth=d3.sum(axis=(1, 2)), lateral_x=d3.sum(axis=(0, 1)), lateral_y=d3.sum(axis=(0, 2)),
        total=np.array([dose.sum()]), total_events=np.array([nev.sum()], np.float64),
    )


def gen_lut(out: Path):
    n = 16
    rng = np.random.default_rng(1)
    mat = rng.integers(0, 4, n ** 3).astype(np.uint8)
    dens = (np.array([1.0, 1.92, 1.03, 0.0012])[mat] * rng.uniform(0.5, 1.5, n ** 3)).astype(np.float32)
    w = R.WorldArgs((n, n, n), (1, 1, 1), dens.astype(np.float64), mat, MATERIALS4)
    for maxE in (60.0, 120.0):
        E = np.concatenate([np.linspace(1.0, maxE, 600), np.geomspace(1.0, maxE, 200)])
        q = np.linspace(0, 12, 200)
        t = R.lut_dump(w, maxE, E, q)
        np.savez_compressed(out / f"lut_4mat_{int(maxE)}kev.npz", material=mat, density=dens, energies=E, q=q,
                            names=np.array(MATERIALS4), max_energy=maxE, **t)


def gen_alias(out: Path):
    rng = np.random.default_rng(3)
    cases = {}
    for k, n in enumerate([1, 2, 7, 60, 150]):
        w = rng.uniform(0, 1, n) ** 3
        if n > 3:
            w[rng.integers(0, n, 2)] = 0.0
        p, a = R.alias_table(w)
        cases[f"w{k}"] = w
        cases[f"p{k}"] = p
        cases[f"a{k}"] = a
    np.savez_compressed(out / "alias.npz", **cases)


def gen_sources(out: Path):
    n = 32
    w = R.WorldArgs((n, n, n), (4, 4, 4), np.ones(n ** 3), np.zeros(n ** 3, np.uint8), ["Water, Liquid"])
    cases = {
        "pencil": R.SourceArgs(R.PENCIL, position=(3, -2, -300), cosines=(1, 0, 0, 0, 1, 0), energy=60.0,
                               histories_per_exposure=1000, total_exposures=3),
        "isotropic": R.SourceArgs(R.ISOTROPIC, position=(0, 0, -400), cosines=(1, 0, 0, 0, 1, 0),
                                  collimation=(-0.2, 0.2, -0.1, 0.15), spec_energies=np.arange(20, 81, 5.0),
                                  spec_weights=np.linspace(1, 3, 13), histories_per_exposure=500, total_exposures=2),
        "dx": R.SourceArgs(R.DX, position=(10, 5, -20), kvp=80, al_mm=3.0, field_size=(200, 150), sdd=1000,
                           source_angles_deg=(15, -10), tube_rotation_deg=0, heel=1, histories_per_exposure=800,
                           total_exposures=2),
        "ctspiral": R.SourceArgs(R.CTSPIRAL, position=(0, 0, -30), kvp=120, al_mm=2.5, ct_collimation=40, pitch=1.0,
                                 scan_length=80, angle_step_deg=1.0, start_angle_deg=0, fov=500, sdd=1190,
                                 tilt_deg=0.0, heel=1, histories_per_exposure=100),
        "ctspiral_tilt": R.SourceArgs(R.CTSPIRAL, position=(0, 0, 0), kvp=100, al_mm=7.0, ct_collimation=20, pitch=1.5,
                                      scan_length=40, angle_step_deg=2.0, start_angle_deg=30, fov=400, sdd=1000,
                                      tilt_deg=12.0, heel=0, histories_per_exposure=100),
    }
    for name, s in cases.items():
        t = R.source_tables(s, w)
        np.savez_compressed(out / f"source_{name}.npz", **t)


def gen_transport(out: Path, quick: bool):
    scale = 0.1 if quick else 1.0
    # pencil 60 keV in a 64^3 water cube of 2 mm voxels (the small pencil-beam workload)
    n = 64
    dims = (n, n, n)
    w = R.WorldArgs(dims, (2.0, 2.0, 2.0), np.ones(n ** 3), np.zeros(n ** 3, np.uint8), ["Water, Liquid"])
    for model in (0, 1, 2):
        hist = int(2e6 * scale)
        s = R.SourceArgs(R.PENCIL, position=(0, 0, -200), cosines=(1, 0, 0, 0, 1, 0), energy=60.0,
                         histories_per_exposure=hist // 10, total_exposures=10)
        t0 = time.time()
        dose, var, nev, N, st = R.transport(w, s, model=model)
        print(f"pencil model {model}: {N} histories {st:.2f} s ({N / st:.3g} hist/s)", flush=True)
        np.savez_compressed(out / f"transport_pencil_m{model}.npz", dims=np.array(dims), spacing=np.array([2.0] * 3),
                            histories=N, seconds=st, **sparse_tally(dose, var, nev, dims))
    # heterogeneous cone beam with a spectrum
    mat, dens = hetero_world()
    n = 48
    dims = (n, n, n)
    w = R.WorldArgs(dims, (4.0, 4.0, 4.0), dens, mat, MATERIALS4)
    spec_e = np.arange(20.0, 101.0, 1.0)
    spec_w = np.exp(-0.5 * ((spec_e - 55) / 15) ** 2) + 0.2
    for model in (1, 2):
        hist = int(4e6 * scale)
        s = R.SourceArgs(R.ISOTROPIC, position=(0, 0, -500), cosines=(1, 0, 0, 0, 1, 0),
                         collimation=(-0.12, 0.12, -0.1, 0.1), spec_energies=spec_e, spec_weights=spec_w,
                         histories_per_exposure=hist // 8, total_exposures=8)
        dose, var, nev, N, st = R.transport(w, s, model=model)
        print(f"cone model {model}: {N} histories {st:.2f} s ({N / st:.3g} hist/s)", flush=True)
        np.savez_compressed(out / f"transport_cone_m{model}.npz", dims=np.array(dims), spacing=np.array([4.0] * 3),
                            material=mat, density=dens.astype(np.float32), names=np.array(MATERIALS4),
                            spec_energies=spec_e, spec_weights=spec_w, histories=N, seconds=st,
                            **sparse_tally(dose, var, nev, dims))
    # forced-interaction (measurement map) case: water slab with a measured cylinder
    n = 40
    dims = (n, n, n)
    z, y, x = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    meas = (((x - 20) ** 2 + (y - 20) ** 2) <= 16).astype(np.uint8).ravel()
    w = R.WorldArgs(dims, (2.0, 2.0, 2.0), np.ones(n ** 3), np.zeros(n ** 3, np.uint8), ["Water, Liquid"],
                    measurement=meas)
    hist = int(2e6 * scale)
    s = R.SourceArgs(R.ISOTROPIC, position=(0, 0, -300), cosines=(1, 0, 0, 0, 1, 0),
                     collimation=(-0.05, 0.05, -0.05, 0.05), spec_energies=np.array([50.0]),
                     spec_weights=np.array([1.0]), histories_per_exposure=hist // 8, total_exposures=8)
    dose, var, nev, N, st = R.transport(w, s, model=1)
    print(f"forced: {N} histories {st:.2f} s", flush=True)
    np.savez_compressed(out / "transport_forced_m1.npz", dims=np.array(dims), spacing=np.array([2.0] * 3),
                        measurement=meas, histories=N, seconds=st, **sparse_tally(dose, var, nev, dims))


def gen_ct(out: Path, quick: bool):
    """Reference CT-spiral run on a small phantom; the fixture carries the reference's
    own exposure, spectrum and heel tables so the GPU run consumes identical inputs."""
    mat, dens = hetero_world(n=48, spacing=4.0, seed=11)
    n = 48
    dims = (n, n, n)
    w = R.WorldArgs(dims, (4.0, 4.0, 4.0), dens, mat, MATERIALS4)
    hpe = 2000 if quick else 12000
    s = R.SourceArgs(R.CTSPIRAL, position=(0, 0, -20), kvp=120, al_mm=2.5, ct_collimation=40, pitch=1.0,
                     scan_length=40, angle_step_deg=1.0, start_angle_deg=0, fov=500, sdd=1190, heel=1,
                     histories_per_exposure=hpe)
    tabs = R.source_tables(s, w)
    dose, var, nev, N, st = R.transport(w, s, model=1)
    print(f"ct: {N} histories {st:.2f} s", flush=True)
    np.savez_compressed(out / "transport_ct_m1.npz", dims=np.array(dims), spacing=np.array([4.0] * 3), material=mat,
                        density=dens.astype(np.float32), names=np.array(MATERIALS4), histories=N, seconds=st,
                        exposures=tabs["exposures"], spec_energies=tabs["spec_energies"],
                        spec_weights=tabs["spec_weights"], heel_meta=tabs["heel_meta"],
                        heel_weights=tabs.get("heel_weights", np.zeros(0)), max_energy=tabs["max_energy"],
                        **sparse_tally(dose, var, nev, dims))


def block_tally(dose, var, nev, dims, block, frac=0.002):
    """Block sums (dose, variance, events) of a tally, kept for blocks above frac of
    the largest block (dims x-fastest as the world, block in voxels per axis)."""
    nx, ny, nz = dims
    bx, by, bz = block

    def bs(a):
        return a.reshape(nz // bz, bz, ny // by, by, nx // bx, bx).sum(axis=(1, 3, 5)).ravel()

    d, v, n = bs(dose), bs(var), bs(nev.astype(np.float64))
    keep = np.nonzero(d > frac * d.max())[0].astype(np.uint32)
    return dict(idx=keep, dose=d[keep], var=v[keep], nev=n[keep], total=np.array([dose.sum()]),
                total_events=np.array([nev.sum()], np.float64)), (d, v)


def same_method_stats(a, b):
    """parity.compare_sparse of two independent reference runs (block sums)."""
    sys.path.insert(0, str(HERE.parent))
    from parity import compare_sparse
    ref = dict(idx=np.arange(len(a[0])), dose=a[0], var=a[1], total=np.array([a[0].sum()]))
    st = compare_sparse(ref, b[0], b[1])
    return np.array([st["chi2"], st["n_voxels"], st["beyond_3sigma"], st["max_abs_z"], st["total_ratio"],
                     st["mean_bias"]])


def gen_bench_ct(out: Path, quick: bool):
    """The headline CT helical workload (512 x 512 x 200, 0.8 x 0.8 x 2.5 mm, seeded body
    phantom; 120 kVp, 2.5 mm Al, 40 mm collimation, pitch 1, 1 degree steps, heel) run
    twice by the reference at 2e7 histories each."""
    sys.path.insert(0, str(HERE.parents[1]))
    from dxmclib_gb300.workloads import CT_MATERIALS, ct_phantom_arrays
    dims, spacing, block = (512, 512, 200), (0.8, 0.8, 2.5), (8, 8, 4)
    mat, dens = ct_phantom_arrays()
    names = [n for n, _ in CT_MATERIALS]
    w = R.WorldArgs(dims, spacing, dens.astype(np.float64), mat, names,
                    material_densities=[d for _, d in CT_MATERIALS])
    hist = int(2e6 if quick else 2e7)
    length = dims[2] * spacing[2]
    s = R.SourceArgs(R.CTSPIRAL, position=(0, 0, -length / 2), kvp=120, al_mm=2.5, ct_collimation=40, pitch=1.0,
                     scan_length=length, angle_step_deg=1.0, start_angle_deg=0, fov=500, sdd=1190, heel=1,
                     histories_per_exposure=1)
    n_exp = len(R.source_tables(s, w)["exposures"])
    s.desc.histories_per_exposure = -(-hist // n_exp)
    tabs = R.source_tables(s, w)
    md = np.zeros(len(names))
    np.maximum.at(md, mat.astype(np.int64), dens.astype(np.float64))
    lut = R.lut_dump(R.WorldArgs((4, 1, 1), (1, 1, 1), md, np.arange(4, dtype=np.uint8), names), tabs["max_energy"],
                     np.array([10.0]), np.array([1.0]))
    runs = []
    for k in range(2):
        dose, var, nev, N, st, _ = R.transport_ex(w, s, model=1)
        print(f"bench ct run {k}: {N} histories {st:.2f} s ({N / st:.3g} hist/s)", flush=True)
        runs.append((block_tally(dose, var, nev, dims, block), N, st))
        del dose, var, nev
    (tally, full_a), N, st = runs[0]
    stats = same_method_stats(full_a, runs[1][0][1])
    print(f"bench ct: reference vs reference chi2/n {stats[0]:.3f} over {int(stats[1])} blocks", flush=True)
    np.savez_compressed(out / "bench_ct_helical.npz", dims=np.array(dims), spacing=np.array(spacing),
                        block=np.array(block), phantom_seed=20261203, names=np.array(names),
                        material_densities=np.array([d for _, d in CT_MATERIALS]), histories=N, seconds=st,
                        exposures=tabs["exposures"], spec_energies=tabs["spec_energies"],
                        spec_weights=tabs["spec_weights"], heel_meta=tabs["heel_meta"],
                        heel_weights=tabs.get("heel_weights", np.zeros(0)), max_energy=tabs["max_energy"],
                        max_density=md, lut_x=lut["x"], lut_coef=lut["coef"], lut_maxcoef=lut["maxcoef"],
                        lut_rita=lut["rita"], lut_spline=lut["spline"], lut_shells=lut["shells"], lut_meta=lut["meta"],
                        same_method=stats, **tally)


def gen_bench_dx(out: Path, quick: bool):
    """A DXSource beam (80 kVp, 3 mm Al, 200 mm field at SDD 1000 mm, angled, heel) on a
    128^3 phantom of the batched-radiography configuration, two reference runs."""
    sys.path.insert(0, str(HERE.parents[1]))
    from dxmclib_gb300.workloads import DX_MATERIALS, dx_phantom_arrays
    n = 128
    dims, spacing, block = (n, n, n), (2.0, 2.0, 2.0), (4, 4, 4)
    mat, dens = dx_phantom_arrays(n, np.random.default_rng(20261204))
    w = R.WorldArgs(dims, spacing, dens.astype(np.float64), mat, DX_MATERIALS)
    hist = int(1e6 if quick else 1e7)
    s = R.SourceArgs(R.DX, position=(0, 0, 0), cosines=(-1, 0, 0, 0, 0, 1), kvp=80, al_mm=3.0, field_size=(200, 200),
                     sdd=1000, source_angles_deg=(15, -10), tube_rotation_deg=0, heel=1,
                     histories_per_exposure=hist // 8, total_exposures=8)
    tabs = R.source_tables(s, w)
    runs = []
    for k in range(2):
        dose, var, nev, N, st, _ = R.transport_ex(w, s, model=1)
        print(f"bench dx run {k}: {N} histories {st:.2f} s", flush=True)
        runs.append((block_tally(dose, var, nev, dims, block), N, st))
    (tally, full_a), N, st = runs[0]
    stats = same_method_stats(full_a, runs[1][0][1])
    print(f"bench dx: reference vs reference chi2/n {stats[0]:.3f} over {int(stats[1])} blocks", flush=True)
    np.savez_compressed(out / "bench_dx.npz", dims=np.array(dims), spacing=np.array(spacing), block=np.array(block),
                        phantom_seed=20261204, material=mat, density=dens.astype(np.float32),
                        names=np.array(DX_MATERIALS), histories=N, seconds=st, exposures=tabs["exposures"],
                        spec_energies=tabs["spec_energies"], spec_weights=tabs["spec_weights"],
                        heel_meta=tabs["heel_meta"], heel_weights=tabs.get("heel_weights", np.zeros(0)),
                        max_energy=tabs["max_energy"], same_method=stats, **tally)


def gen_dose(out: Path, quick: bool):
    """DOSE output mode (transport.hpp:186-195, 796-816): a DX beam on a 64^3 phantom,
    once with the source's dose-area-product calibration (mGy) and once without (keV/kg)."""
    sys.path.insert(0, str(HERE.parents[1]))
    from dxmclib_gb300.workloads import DX_MATERIALS, dx_phantom_arrays
    n = 64
    dims, spacing, block = (n, n, n), (4.0, 4.0, 4.0), (2, 2, 2)
    mat, dens = dx_phantom_arrays(n, np.random.default_rng(7))
    w = R.WorldArgs(dims, spacing, dens.astype(np.float64), mat, DX_MATERIALS)
    hist = int(4e5 if quick else 4e6)
    s = R.SourceArgs(R.DX, position=(0, 0, 0), cosines=(-1, 0, 0, 0, 0, 1), kvp=70, al_mm=3.0, field_size=(150, 150),
                     sdd=1000, source_angles_deg=(0, 0), tube_rotation_deg=0, heel=1,
                     histories_per_exposure=hist // 8, total_exposures=8)
    tabs = R.source_tables(s, w)
    cal = R.calibration_value(w, s, model=1)
    res = {}
    for label, use_cal in (("mgy", True), ("kevkg", False)):
        dose, var, nev, N, st, units = R.transport_ex(w, s, model=1, output_mode=1, use_calibration=use_cal)
        assert units == (2 if use_cal else 1), units
        t, _ = block_tally(dose, var, nev, dims, block)
        res.update({f"{label}_{k}": v for k, v in t.items()})
        print(f"dose {label}: {N} histories, total {dose.sum():.6g}", flush=True)
    np.savez_compressed(out / "transport_dose_dx.npz", dims=np.array(dims), spacing=np.array(spacing),
                        block=np.array(block), material=mat, density=dens.astype(np.float32),
                        names=np.array(DX_MATERIALS), histories=N, calibration=cal, exposures=tabs["exposures"],
                        spec_energies=tabs["spec_energies"], spec_weights=tabs["spec_weights"],
                        heel_meta=tabs["heel_meta"], heel_weights=tabs.get("heel_weights", np.zeros(0)),
                        max_energy=tabs["max_energy"], **res)


def gen_tubes(out: Path):
    """Tube<double>::getSpecter (tube.hpp:191-261) and HeelFilter<double> weights
    (beamfilters.hpp:455-505), read through DX sources of the reference, at the
    voltages and filtrations of the benchmark configurations."""
    w = R.WorldArgs((8, 8, 8), (1, 1, 1), np.ones(512), np.zeros(512, np.uint8), ["Water, Liquid"])
    res = {}
    cases = [(70, 3.0, 0.0, 12.0), (80, 3.0, 0.0, 12.0), (90, 3.0, 0.1, 12.0), (120, 2.5, 0.0, 12.0), (100, 2.0, 0.0, 8.0)]
    for k, (kvp, al, cu, anode) in enumerate(cases):
        s = R.SourceArgs(R.DX, kvp=kvp, al_mm=al, cu_mm=cu, anode_angle_deg=anode, field_size=(300, 200), sdd=1000,
                         heel=1, histories_per_exposure=10, total_exposures=1)
        t = R.source_tables(s, w)
        res[f"case{k}"] = np.array([kvp, al, cu, anode])
        res[f"energies{k}"] = t["spec_energies"]
        res[f"weights{k}"] = t["spec_weights"]
        res[f"heel_meta{k}"] = t["heel_meta"]
        res[f"heel_weights{k}"] = t["heel_weights"]
    np.savez_compressed(out / "tube_spectra.npz", n=len(cases), **res)


def gen_interactions(out: Path, quick: bool):
    n = 8
    w = R.WorldArgs((n, n, n), (1, 1, 1), np.ones(n ** 3) * 1.92, np.zeros(n ** 3, np.uint8),
                    ["Bone, Cortical (ICRP)"])
    N = int(4e5 if quick else 2e6)
    res = {}
    for model in (0, 1, 2):
        for kind, name in ((1, "compton"), (2, "rayleigh"), (0, "photo")):
            for energy in (20.0, 60.0):
                hc, he, sums = R.interactions(w, 120.0, model, kind, energy, N, nbins=100, seed=model * 10 + kind)
                key = f"m{model}_{name}_{int(energy)}"
                res[key + "_cos"] = hc
                res[key + "_e"] = he
                res[key + "_sums"] = sums
    np.savez_compressed(out / "interactions_bone.npz", n=N, **res)


def gen_ctdi(out: Path, quick: bool):
    """CTDIPhantom<double> (world.hpp:229-390) arrays and hole lists, and the reference's
    CT calibration factor (source.hpp:925-988) with the exact exposure, spectrum and
    heel tables of the axial copy it runs, so the GPU calibration consumes the same inputs."""
    phantoms = {}
    for d in (160, 320):
        dims, dens, mat, meas, counts, holes = R.ctdi_phantom(d)
        phantoms[f"d{d}_dims"] = np.array(dims)
        phantoms[f"d{d}_counts"] = np.array(counts)
        phantoms[f"d{d}_holes"] = holes.astype(np.uint32)
        phantoms[f"d{d}_material_counts"] = np.bincount(mat, minlength=3)
        phantoms[f"d{d}_densities"] = np.unique(dens)
        if d == 160:
            phantoms["d160_material"] = mat
            phantoms["d160_measurement"] = meas
    np.savez_compressed(out / "ctdi_phantom.npz", **phantoms)
    hpe = 1000
    s = R.SourceArgs(R.CTSPIRAL, position=(0, 0, 0), kvp=120, al_mm=2.5, ct_collimation=40, pitch=1.0,
                     scan_length=100, angle_step_deg=1.0, start_angle_deg=0, fov=500, sdd=1190, heel=1,
                     histories_per_exposure=hpe)
    t = time.time()
    factor, meta = R.ct_calibration(s, model=1, ctdivol=1.0, diameter=320)
    seconds = time.time() - t
    print(f"ct calibration: factor {factor:.6e}, {meta[0] * meta[1]:.3e} histories, {seconds:.1f} s", flush=True)
    cal = R.SourceArgs(R.CT_CALIBRATION, position=(0, 0, 0), kvp=120, al_mm=2.5, ct_collimation=40, pitch=1.0,
                       scan_length=100, angle_step_deg=1.0, start_angle_deg=0, fov=500, sdd=1190, heel=1,
                       histories_per_exposure=int(meta[1]))
    dims, dens, mat, meas, counts, holes = R.ctdi_phantom(320)
    w = R.WorldArgs(dims, (1.0, 1.0, 2.5), dens, mat, ["Air, Dry (near sea level)", "Air, Dry (near sea level)",
                                                       "Polymethyl Methacralate (Lucite, Perspex)"], measurement=meas)
    tabs = R.source_tables(cal, w)
    np.savez_compressed(out / "ct_calibration_m1.npz", factor=factor, exposures_per_rotation=meta[0],
                        calibration_hpe=meta[1], mean_weight=meta[2], seconds=seconds, ctdivol=1.0, diameter=320,
                        collimation=40.0, pitch=1.0, exposures=tabs["exposures"], spec_energies=tabs["spec_energies"],
                        spec_weights=tabs["spec_weights"], heel_meta=tabs["heel_meta"],
                        heel_weights=tabs.get("heel_weights", np.zeros(0)), max_energy=tabs["max_energy"])


def ct_family_cases():
    """The CT sources beyond the single-tube spiral: axial (with a step other than the
    collimation), spiral and axial dual-source (tube B, tube currents, its own
    distance, field of view and start angle) and topogram."""
    return {
        "ctaxial": R.SourceArgs(R.CTAXIAL, position=(0, 0, -20), kvp=100, al_mm=3.0, ct_collimation=20,
                                scan_length=50, angle_step_deg=3.0, start_angle_deg=15, fov=450, sdd=1100,
                                tilt_deg=5.0, heel=1, histories_per_exposure=100, axial_step=25),
        "ctspiral_dual": R.SourceArgs(R.CTSPIRAL_DUAL, position=(0, 0, -30), kvp=140, al_mm=2.5, ct_collimation=40,
                                      pitch=1.2, scan_length=60, angle_step_deg=2.0, start_angle_deg=10, fov=500,
                                      sdd=1190, tilt_deg=0.0, heel=1, histories_per_exposure=100, kvp_b=80,
                                      al_mm_b=6.0, cu_mm_b=0.1, mas_a=120, mas_b=200, sdd_b=1000, fov_b=330,
                                      start_angle_b_deg=100),
        "ctaxial_dual": R.SourceArgs(R.CTAXIAL_DUAL, position=(0, 0, 0), kvp=120, al_mm=2.5, ct_collimation=20,
                                     scan_length=60, angle_step_deg=5.0, start_angle_deg=0, fov=500, sdd=1190,
                                     tilt_deg=8.0, heel=0, histories_per_exposure=100, axial_step=30, kvp_b=100,
                                     al_mm_b=4.0, mas_a=200, mas_b=100, sdd_b=1190, fov_b=260, start_angle_b_deg=95),
        "cttopogram": R.SourceArgs(R.CTTOPOGRAM, position=(0, 0, -30), kvp=120, al_mm=2.5, ct_collimation=10,
                                   scan_length=300, start_angle_deg=30, fov=500, sdd=1190, tilt_deg=0.0, heel=1,
                                   histories_per_exposure=100),
    }


def gen_ct_family(out: Path, quick: bool):
    """Exposure tables and the per-tube spectrum / heel tables of the CT family
    (source.hpp:1192-1702), a dual-source transport (Transport<double>, block sums)
    and the calibration factors of a spiral dual source and a topogram
    (Source::getCalibrationValue: the reference's own CTDI run, 1e8 histories)."""
    n = 32
    w = R.WorldArgs((n, n, n), (4, 4, 4), np.ones(n ** 3), np.zeros(n ** 3, np.uint8), ["Water, Liquid"])
    for name, s in ct_family_cases().items():
        t = R.source_tables(s, w)
        for k in (0, 1):
            e = R.exposure_tables(s, w, k)
            for key, v in e.items():
                t[f"x{k}_{key}"] = v
        np.savez_compressed(out / f"source_{name}.npz", **t)
    # dual-source helical scan of the heterogeneous phantom
    mat, dens = hetero_world(n=48, spacing=4.0, seed=11)
    dims = (48, 48, 48)
    wt = R.WorldArgs(dims, (4.0, 4.0, 4.0), dens, mat, MATERIALS4)
    hpe = 400 if quick else 2400
    s = R.SourceArgs(R.CTSPIRAL_DUAL, position=(0, 0, -20), kvp=140, al_mm=2.5, ct_collimation=40, pitch=1.0,
                     scan_length=40, angle_step_deg=2.0, start_angle_deg=0, fov=500, sdd=1190, heel=1,
                     histories_per_exposure=hpe, kvp_b=80, al_mm_b=6.0, mas_a=100, mas_b=250, sdd_b=1050, fov_b=330,
                     start_angle_b_deg=90)
    tabs = R.source_tables(s, wt)
    beams = [R.exposure_tables(s, wt, k) for k in (0, 1)]
    runs = []
    for k in range(2):
        dose, var, nev, N, st = R.transport(wt, s, model=1)
        print(f"ct dual run {k}: {N} histories {st:.2f} s", flush=True)
        runs.append(block_tally(dose, var, nev, dims, (2, 2, 2)))
    extra = {f"x{k}_{key}": v for k in (0, 1) for key, v in beams[k].items()}
    np.savez_compressed(out / "transport_ct_dual_m1.npz", dims=np.array(dims), spacing=np.array([4.0] * 3),
                        material=mat, density=dens.astype(np.float32), names=np.array(MATERIALS4), histories=N,
                        block=np.array([2, 2, 2]), exposures=tabs["exposures"], spec_energies=tabs["spec_energies"],
                        spec_weights=tabs["spec_weights"], heel_meta=tabs["heel_meta"],
                        heel_weights=tabs.get("heel_weights", np.zeros(0)), max_energy=tabs["max_energy"],
                        same_method=same_method_stats(runs[0][1], runs[1][1]),
                        **{f"r_{k}": v for k, v in runs[0][0].items()}, **extra)
    # calibration factors (the sources' defaults: CTDIvol 1 mGy, 320 mm phantom)
    factors = {}
    cal_cases = {
        "spiral_dual": R.SourceArgs(R.CTSPIRAL_DUAL, position=(0, 0, 0), kvp=140, al_mm=2.5, ct_collimation=40,
                                    pitch=1.2, scan_length=100, angle_step_deg=1.0, start_angle_deg=0, fov=500,
                                    sdd=1190, heel=1, histories_per_exposure=1000, kvp_b=80, al_mm_b=6.0, mas_a=100,
                                    mas_b=250, sdd_b=1050, fov_b=330, start_angle_b_deg=90),
        "topogram": R.SourceArgs(R.CTTOPOGRAM, position=(0, 0, 0), kvp=120, al_mm=2.5, ct_collimation=10,
                                 scan_length=300, start_angle_deg=0, fov=500, sdd=1190, heel=1,
                                 histories_per_exposure=10000),
    }
    for name, s in cal_cases.items():
        if quick:
            break
        t = time.time()
        factors[name] = R.calibration_value(w, s, model=1)
        print(f"calibration {name}: {factors[name]:.6e} ({time.time() - t:.1f} s)", flush=True)
    np.savez_compressed(out / "ct_family_calibration_m1.npz", ctdivol=1.0, diameter=320,
                        **{k: np.array(v) for k, v in factors.items()})


BOWTIE_ANGLES = np.array([0.2, 0.0, -0.06, 0.03, 0.1, 0.45, 0.15, 0.3, 0.25, 0.35, 0.4])


def bowtie_weights(angles):
    """A CT body bow-tie's fluence profile: 1 on the axis falling to about 0.15 at the
    edge of a 500 mm field of view."""
    a = np.abs(np.asarray(angles, np.float64))
    return 0.15 + 0.85 * np.exp(-(a / 0.18) ** 2)


def gen_bowtie(out: Path, quick: bool):
    """BowTieFilter<double> (unsorted, one negative angle: |angle|, sort, mean-1
    normalisation) and a CT helical scan through it (CTSpiralSource with
    setBowTieFilter, source.hpp:821; the weight enters Exposure::sampleParticle)."""
    w_raw = bowtie_weights(BOWTIE_ANGLES)
    queries = np.concatenate([np.linspace(-0.5, 0.5, 201), np.abs(BOWTIE_ANGLES), -np.abs(BOWTIE_ANGLES)])
    ta, tw, qw = R.bowtie(BOWTIE_ANGLES, w_raw, queries)
    np.savez_compressed(out / "bowtie.npz", angles=BOWTIE_ANGLES, weights=w_raw, queries=queries, table_angles=ta,
                        table_weights=tw, query_weights=qw)
    mat, dens = hetero_world(n=48, spacing=4.0, seed=11)
    dims = (48, 48, 48)
    wt = R.WorldArgs(dims, (4.0, 4.0, 4.0), dens, mat, MATERIALS4)
    hpe = 4000 if quick else 24000
    s = R.SourceArgs(R.CTSPIRAL, position=(0, 0, -20), kvp=120, al_mm=2.5, ct_collimation=40, pitch=1.0,
                     scan_length=40, angle_step_deg=1.0, start_angle_deg=0, fov=500, sdd=1190, heel=1,
                     histories_per_exposure=hpe, bowtie=(BOWTIE_ANGLES, w_raw))
    tabs = R.source_tables(s, wt)
    runs = []
    for k in range(2):
        dose, var, nev, N, st = R.transport(wt, s, model=1)
        print(f"ct bowtie run {k}: {N} histories {st:.2f} s", flush=True)
        runs.append(block_tally(dose, var, nev, dims, (2, 2, 2)))
    np.savez_compressed(out / "transport_ct_bowtie_m1.npz", dims=np.array(dims), spacing=np.array([4.0] * 3),
                        material=mat, density=dens.astype(np.float32), names=np.array(MATERIALS4), histories=N,
                        block=np.array([2, 2, 2]), exposures=tabs["exposures"], spec_energies=tabs["spec_energies"],
                        spec_weights=tabs["spec_weights"], heel_meta=tabs["heel_meta"],
                        heel_weights=tabs.get("heel_weights", np.zeros(0)), max_energy=tabs["max_energy"],
                        bowtie_angles=BOWTIE_ANGLES, bowtie_weights=w_raw,
                        same_method=same_method_stats(runs[0][1], runs[1][1]),
                        **{f"r_{k}": v for k, v in runs[0][0].items()})


def gen_more_sources(out: Path):
    """Exposure, spectrum and heel tables of the cone-beam CT source (CBCTSource,
    source.hpp:679-782) and the rotating isotropic source (IsotropicCTSource,
    source.hpp:346-377)."""
    n = 32
    w = R.WorldArgs((n, n, n), (4, 4, 4), np.ones(n ** 3), np.zeros(n ** 3, np.uint8), ["Water, Liquid"])
    cases = {
        "cbct": R.SourceArgs(R.CBCT, position=(5, -3, 10), kvp=90, al_mm=4.0, field_size=(250, 200), sdd=600,
                             source_angles_deg=(20, -15), span_deg=200, step_deg=2.5, heel=1,
                             histories_per_exposure=100),
        "isotropic_ct": R.SourceArgs(R.ISOTROPIC_CT, position=(0, -300, 20), cosines=(1, 0, 0, 0, 0, 1),
                                     collimation=(-0.3, 0.3, -0.05, 0.05), spec_energies=np.arange(20, 81, 5.0),
                                     spec_weights=np.linspace(1, 3, 13), histories_per_exposure=100,
                                     total_exposures=36),
    }
    for name, src in cases.items():
        np.savez_compressed(out / f"source_{name}.npz", **R.source_tables(src, w))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--quick", action="store_true")
    ap.add_argument("--only", default="")
    a = ap.parse_args()
    if not R.available():
        raise SystemExit("oracle/_ref/libdxmc_ref.so missing: run `make -C oracle REF=<reference checkout>` first")
    out = HERE
    steps = dict(lut=lambda: gen_lut(out), alias=lambda: gen_alias(out), sources=lambda: gen_sources(out),
                 transport=lambda: gen_transport(out, a.quick), ct=lambda: gen_ct(out, a.quick),
                 interactions=lambda: gen_interactions(out, a.quick), ctdi=lambda: gen_ctdi(out, a.quick),
                 bench_ct=lambda: gen_bench_ct(out, a.quick), bench_dx=lambda: gen_bench_dx(out, a.quick),
                 dose=lambda: gen_dose(out, a.quick), tubes=lambda: gen_tubes(out),
                 ct_family=lambda: gen_ct_family(out, a.quick), more_sources=lambda: gen_more_sources(out),
                 bowtie=lambda: gen_bowtie(out, a.quick))
    for name, fn in steps.items():
        if a.only and name not in a.only.split(","):
            continue
        t = time.time()
        fn()
        print(f"{name}: {time.time() - t:.1f} s", flush=True)


if __name__ == "__main__":
    main()
