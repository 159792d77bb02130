"""Seeded synthetic workloads with the shapes of the benchmark configurations.

There are no public datasets on this path: the phantoms below are generated
from fixed seeds with the sizes, spacings, materials and densities of the
benchmark configurations (pencil beam on a 64^3 water cube; CT helical on a
512 x 512 x 200 body phantom; batched DX on uneven grids).
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from .api import CTSpiralSource, DXSource, Material, PencilSource, World

AIR, SOFT, LUNG, BONE = 0, 1, 2, 3
CT_MATERIALS = [("Air, Dry (near sea level)", 0.001205), ("Tissue, Soft (ICRP)", 1.03),
                ("Lung Tissue (ICRU-44)", 0.26), ("Bone, Cortical (ICRP)", 1.92)]


@dataclass
class Workload:
    name: str
    world: World
    source: object
    histories: int


def pencil_water(n: int = 64, spacing_mm: float = 2.0, energy: float = 60.0, histories: int = 1_000_000,
                 exposures: int = 10) -> Workload:
    """60 keV pencil beam along +z into the centre of an all-water cube (configuration 1)."""
    w = World()
    w.setDimensions((n, n, n))
    w.setSpacing((spacing_mm,) * 3)
    w.setDensityArray(np.ones(n ** 3, np.float32))
    w.setMaterialIndexArray(np.zeros(n ** 3, np.uint8))
    w.addMaterialToMap(Material("Water, Liquid"))
    src = PencilSource()
    src.setPosition((0, 0, -(n * spacing_mm)))
    src.setDirectionCosines((1, 0, 0, 0, 1, 0))
    src.setPhotonEnergy(energy)
    src.setTotalExposures(exposures)
    src.setHistoriesPerExposure(max(histories // exposures, 1))
    return Workload(f"pencil_water_{n}^3", w, src, exposures * max(histories // exposures, 1))


def ct_phantom_arrays(nx: int = 512, ny: int = 512, nz: int = 200, spacing=(0.8, 0.8, 2.5), seed: int = 20261203):
    """Body phantom: elliptic soft-tissue cylinder (semi-axes 160 x 120 mm) in air,
    two lung ellipsoids and 30 bone spheres (radius 5-20 mm) placed from the seed."""
    rng = np.random.default_rng(seed)
    sx, sy, sz = spacing
    x = (np.arange(nx) - (nx - 1) / 2) * sx
    y = (np.arange(ny) - (ny - 1) / 2) * sy
    z = (np.arange(nz) - (nz - 1) / 2) * sz
    X, Y = np.meshgrid(x, y, indexing="xy")  # (ny, nx)
    body2d = (X / 160.0) ** 2 + (Y / 120.0) ** 2 <= 1.0
    lungs = [(-75.0, -5.0, 0.0, 55.0, 70.0, 0.42 * nz * sz), (75.0, -5.0, 0.0, 55.0, 70.0, 0.42 * nz * sz)]
    spheres = []
    while len(spheres) < 30:
        cx, cy = rng.uniform(-160, 160), rng.uniform(-120, 120)
        if (cx / 160.0) ** 2 + (cy / 120.0) ** 2 > 0.8:
            continue
        cz = rng.uniform(z[0], z[-1])
        r = rng.uniform(5.0, 20.0)
        spheres.append((cx, cy, cz, r))
    mat = np.empty((nz, ny, nx), np.uint8)
    dens = np.empty((nz, ny, nx), np.float32)
    d_of = np.array([d for _, d in CT_MATERIALS], np.float32)
    for k in range(nz):
        m = np.where(body2d, SOFT, AIR).astype(np.uint8)
        for (cx, cy, cz, ax, ay, az) in lungs:
            t = 1.0 - ((z[k] - cz) / az) ** 2
            if t > 0:
                m[(((X - cx) / ax) ** 2 + ((Y - cy) / ay) ** 2 <= t) & body2d] = LUNG
        for (cx, cy, cz, r) in spheres:
            dz = z[k] - cz
            if abs(dz) < r:
                rr = r * r - dz * dz
                m[((X - cx) ** 2 + (Y - cy) ** 2 <= rr) & body2d] = BONE
        mat[k] = m
        dens[k] = d_of[m]
    return mat.ravel(), dens.ravel()


def ct_world(nz: int = 200, seed: int = 20261203, nx: int = 512, ny: int = 512, spacing=(0.8, 0.8, 2.5)) -> World:
    """The body phantom as a World (four materials: air, soft tissue, lung, bone)."""
    mat, dens = ct_phantom_arrays(nx, ny, nz, spacing, seed)
    w = World()
    w.setDimensions((nx, ny, nz))
    w.setSpacing(spacing)
    w.setDensityArray(dens)
    w.setMaterialIndexArray(mat)
    for name, d in CT_MATERIALS:
        w.addMaterialToMap(Material(name, density=d))
    return w


def ct_source(world: World, histories: int) -> CTSpiralSource:
    """120 kVp, 2.5 mm Al, 40 mm collimation, pitch 1, 1 degree steps over the phantom length."""
    length = world.dimensions()[2] * world.spacing()[2]
    src = CTSpiralSource()
    src.tube().setVoltage(120.0)
    src.tube().setAlFiltration(2.5)
    src.setCollimation(40.0)
    src.setPitch(1.0)
    src.setPosition((0.0, 0.0, -length / 2))
    src.setScanLenght(length)
    src.setExposureAngleStepDeg(1.0)
    src.setModelHeelEffect(True)
    n_exp = src.totalExposures()
    src.setHistoriesPerExposure(max(int(math.ceil(histories / n_exp)), 1))
    return src


def ct_helical(nz: int = 200, histories: int = 100_000_000, seed: int = 20261203) -> Workload:
    """CT helical on the 512 x 512 x nz body phantom: 120 kVp, 2.5 mm Al, 40 mm
    collimation, pitch 1, 1 degree steps over the phantom length (configuration 2)."""
    w = ct_world(nz, seed)
    src = ct_source(w, histories)
    return Workload(f"ct_helical_512x512x{nz}", w, src, src.totalExposures() * src.historiesPerExposure())


DX_MATERIALS = ["Tissue, Soft (ICRP)", "Bone, Cortical (ICRP)", "Lung Tissue (ICRU-44)"]


def dx_phantom_arrays(n: int, rng):
    """Material ids and densities of an n^3 soft-tissue grid with 3-8 random
    ellipsoid inclusions of the three DX materials at densities uniform in
    [0.2, 2.0] (numpy only; x fastest)."""
    mat = np.zeros((n, n, n), np.uint8)
    dens = np.full((n, n, n), 1.0, np.float32)
    zz, yy, xx = np.ogrid[:n, :n, :n]
    for _ in range(int(rng.integers(3, 9))):
        c = rng.uniform(0.2 * n, 0.8 * n, 3)
        a = rng.uniform(0.05 * n, 0.25 * n, 3)
        m = int(rng.integers(0, 3))
        sel = ((xx - c[0]) / a[0]) ** 2 + ((yy - c[1]) / a[1]) ** 2 + ((zz - c[2]) / a[2]) ** 2 <= 1
        mat[sel] = m
        dens[sel] = rng.uniform(0.2, 2.0)
    return mat.ravel(), dens.ravel()


def dx_world(n: int, spacing_mm: float, rng) -> World:
    """n^3 grid of soft tissue with 3-8 random ellipsoid inclusions of the three
    materials at densities uniform in [0.2, 2.0]."""
    mat, dens = dx_phantom_arrays(n, rng)
    w = World()
    w.setDimensions((n, n, n))
    w.setSpacing((spacing_mm,) * 3)
    w.setDensityArray(dens)
    w.setMaterialIndexArray(mat)
    for name in DX_MATERIALS:
        w.addMaterialToMap(Material(name))
    return w


def dx_source(rng, histories: int, kvp: float = None) -> DXSource:
    """70-90 kVp with 3 mm Al, 100-300 mm square field at the default SDD, 8 exposures."""
    src = DXSource()
    src.tube().setVoltage(float(rng.uniform(70, 90)) if kvp is None else float(kvp))
    src.tube().setAlFiltration(3.0)
    fs = float(rng.uniform(100, 300))
    src.setFieldSize((fs, fs))
    src.setSourceAnglesDeg(float(rng.uniform(-30, 30)), float(rng.uniform(-20, 20)))
    src.setTotalExposures(8)
    src.setHistoriesPerExposure(max(histories // 8, 1))
    return src


def dx_batch(n_jobs: int = 64, seed: int = 20261204, histories_range=(1_000_000, 10_000_000)):
    """Uneven DX jobs: grids 64^3 - 256^3 at 1-4 mm with ellipsoid inclusions of three
    materials (densities 0.2-2.0), 70-90 kVp with 3 mm Al, 100-300 mm fields at SDD 1000 mm."""
    rng = np.random.default_rng(seed)
    jobs = []
    for j in range(n_jobs):
        n = int(rng.choice([64, 96, 128, 160, 192, 224, 256]))
        sp = float(rng.uniform(1.0, 4.0))
        w = dx_world(n, sp, rng)
        src = dx_source(rng, 8)
        h = int(np.exp(rng.uniform(np.log(histories_range[0]), np.log(histories_range[1]))))
        src.setHistoriesPerExposure(max(h // 8, 1))
        jobs.append(Workload(f"dx_{j}_{n}^3", w, src, 8 * max(h // 8, 1)))
    return jobs


@dataclass
class StreamJob:
    arrival: float      # seconds after the start of the stream
    kind: str           # "pencil", "dx" or "ct"
    world_key: str
    world: World
    source: object
    histories: int
    seed: int


def serving_stream(n_jobs: int = 64, rate_per_s: float = 200.0, seed: int = 20261205,
                   histories_range=(1_000_000, 100_000_000), ct_slices=(100, 200, 400), dx_sizes=(128, 192, 256)):
    """Mixed dose requests with Poisson arrivals (configuration 4): 40 % pencil beams on
    the 64^3 water cube, 40 % DX on 128^3-256^3 phantoms, 20 % CT helical on
    512 x 512 x (100-400) phantoms; histories log-uniform in ``histories_range``.
    The phantoms come from a small seeded pool (one per grid size), as a clinic
    serves repeated requests on the same patient models."""
    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1.0 / rate_per_s, n_jobs)) if rate_per_s > 0 else np.zeros(n_jobs)
    worlds = {}

    def world(kind, size):
        key = f"{kind}_{size}"
        if key not in worlds:
            if kind == "pencil":
                worlds[key] = pencil_water(size).world
            elif kind == "dx":
                worlds[key] = dx_world(size, 400.0 / size, np.random.default_rng(seed + size))
            else:
                worlds[key] = ct_world(size, seed=20261203)
        return key, worlds[key]

    out = []
    lo, hi = histories_range
    for j in range(n_jobs):
        u = rng.uniform()
        h = int(math.exp(rng.uniform(math.log(lo), math.log(hi))))
        if u < 0.4:
            key, w = world("pencil", 64)
            src = PencilSource()
            src.setPosition((0, 0, -128.0))
            src.setDirectionCosines((1, 0, 0, 0, 1, 0))
            src.setPhotonEnergy(60.0)
            src.setTotalExposures(10)
            src.setHistoriesPerExposure(max(h // 10, 1))
            kind = "pencil"
        elif u < 0.8:
            key, w = world("dx", int(rng.choice(dx_sizes)))
            src = dx_source(rng, h, kvp=float(rng.choice([70.0, 80.0, 90.0])))
            kind = "dx"
        else:
            key, w = world("ct", int(rng.choice(ct_slices)))
            src = ct_source(w, h)
            kind = "ct"
        n_hist = int(np.sum(src.exposures(w.directionCosines()).n_histories)) if kind == "ct" else None
        out.append(StreamJob(float(arrivals[j]), kind, key, w, src, n_hist or h, int(rng.integers(1, 2**31))))
    return out
