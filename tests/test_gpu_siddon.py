"""GPU test of the Siddon traversal (dxmc_gpu_radiological_path) against the CPU
restatement in oracle/siddon.py on a heterogeneous grid, for both voxel
layouts: rays from outside in every direction, rays along the grid axes through
voxel faces and edges, and rays starting inside.  The kernel accumulates in
FP32 (compensated) with the FP32 LUT: relative tolerance 1e-4."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

sys.path.insert(0, str(Path(__file__).resolve().parents[1] / "oracle"))
import siddon  # noqa: E402

pytestmark = pytest.mark.gpu


def _rays(lo, hi, rng, n=3000):
    center = (lo + hi) / 2
    rays = []
    for _ in range(n // 2):  # from a sphere outside towards a random point of the box
        u = rng.normal(size=3)
        o = center + 200.0 * u / np.linalg.norm(u)
        t = rng.uniform(lo, hi)
        rays.append([*o, *(t - o), rng.uniform(20, 120)])
    for _ in range(n // 4):  # along an axis, through faces and edges of voxels
        k = rng.integers(3)
        o = rng.uniform(lo, hi)
        o = np.round(o)  # many land on voxel boundary planes
        o[k] = lo[k] - 10 if rng.uniform() < 0.5 else hi[k] + 10
        d = np.zeros(3)
        d[k] = 1.0 if o[k] < lo[k] else -1.0
        rays.append([*o, *d, 60.0])
    for _ in range(n - len(rays)):  # from inside, any direction
        o = rng.uniform(lo, hi)
        d = rng.normal(size=3)
        rays.append([*o, *d, rng.uniform(20, 120)])
    return np.array(rays, np.float32)


@pytest.mark.parametrize("layout", [0, 1])
def test_radiological_path_matches_cpu(gpu_ctx, layout):
    import dxmclib_gb300 as dx
    rng = np.random.default_rng(17 + layout)
    dims, sp, origin = (24, 20, 16), (2.0, 2.5, 3.0), (1.0, -2.0, 3.0)
    n = int(np.prod(dims))
    mat = rng.integers(0, 3, n).astype(np.uint8)
    dens = np.array([1.0, 1.92, 0.0012], np.float32)[mat] * rng.choice([1.0, 1.5, 0.5], n).astype(np.float32)
    world = dx.World()
    world.setDimensions(dims)
    world.setSpacing(sp)
    world.setOrigin(origin)
    world.setDensityArray(dens)
    world.setMaterialIndexArray(mat)
    for name in ("Water, Liquid", "Bone, Cortical (ICRP)", "Air, Dry (near sea level)"):
        world.addMaterialToMap(dx.Material(name))
    assert world.isValid()
    dworld = dx.DeviceWorld(gpu_ctx, world, layout=layout)
    blob = dx.LutBlob(world.materialMap(), dworld.max_density(), 150.0)
    dlut = dx.DeviceLut(gpu_ctx, blob)
    ext = np.array(world.matrixExtent()).reshape(3, 2)
    lo, hi = ext[:, 0], ext[:, 1]
    rays = _rays(lo, hi, rng)
    gpu = dworld.radiological_path(dlut, rays)
    cpu = siddon.radiological_path(dims, sp, lo, dens, mat, lambda m, e: float(np.sum(blob.attenuation(m, e))),
                                   rays.astype(np.float64))
    assert np.count_nonzero(cpu) > len(rays) * 0.9
    np.testing.assert_allclose(gpu, cpu, rtol=1e-4, atol=1e-6 * cpu.max())
    dlut.close()
    dworld.close()


def test_palette_indices_of_every_voxel(gpu_ctx):
    """The compact layout's palette index of every voxel, read through rays along
    x through the centre of every (y, z) row: equal to the 8-byte layout's and the
    CPU restatement's, on a grid whose voxel count leaves a tail after the
    4-voxel groups of the palette kernels (105 voxels)."""
    import dxmclib_gb300 as dx
    rng = np.random.default_rng(23)
    dims, sp = (7, 3, 5), (2.0, 3.0, 4.0)
    n = int(np.prod(dims))
    mat = rng.integers(0, 2, n).astype(np.uint8)
    dens = np.array([1.0, 1.92], np.float32)[mat] * rng.choice([0.5, 1.0, 1.25, 2.0], n).astype(np.float32)
    world = dx.World()
    world.setDimensions(dims)
    world.setSpacing(sp)
    world.setDensityArray(dens)
    world.setMaterialIndexArray(mat)
    for name in ("Water, Liquid", "Bone, Cortical (ICRP)"):
        world.addMaterialToMap(dx.Material(name))
    assert world.isValid()
    ext = np.array(world.matrixExtent()).reshape(3, 2)
    lo, hi = ext[:, 0], ext[:, 1]
    rays = []
    for z in range(dims[2]):
        for y in range(dims[1]):
            o = [lo[0] - 5.0, lo[1] + (y + 0.5) * sp[1], lo[2] + (z + 0.5) * sp[2]]
            rays.append([*o, 1.0, 0.0, 0.0, 60.0])
    rays = np.array(rays, np.float32)
    paths = []
    for layout in (0, 1):
        dworld = dx.DeviceWorld(gpu_ctx, world, layout=layout)
        blob = dx.LutBlob(world.materialMap(), dworld.max_density(), 150.0)
        dlut = dx.DeviceLut(gpu_ctx, blob)
        paths.append(dworld.radiological_path(dlut, rays))
        dlut.close()
        dworld.close()
    cpu = siddon.radiological_path(dims, sp, lo, dens, mat, lambda m, e: float(np.sum(blob.attenuation(m, e))),
                                   rays.astype(np.float64))
    assert np.all(cpu > 0)
    np.testing.assert_allclose(paths[0], paths[1], rtol=1e-6)  # a wrong index changes a voxel by >= 25 %
    np.testing.assert_allclose(paths[0], cpu, rtol=1e-4)
