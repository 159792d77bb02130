"""Dose calibration: the CTDI phantom and the CT calibration run on the GPU.

DXMClib converts a CT simulation to mGy with a second transport run
(``CTBaseSource::ctCalibration``, ``source.hpp:925-988``): the source is copied
into an axial source that scans one collimation at the centre of a PMMA CTDI
phantom (``CTDIPhantom``, ``world.hpp:229-390``) whose five air holes form a
measurement map (forced photoelectric scoring, ``transport.hpp:523-581``); the
mean dose in the centre and peripheral holes gives the weighted CTDI, and the
factor maps it to the source's CTDIvol.  Here the phantom is restated on the
host (pinned entry by entry against the reference) and the calibration run is
an ordinary GPU job.
"""
from __future__ import annotations

import math
from typing import List

import numpy as np

from . import _capi as A
from .api import Material, World

CENTER, WEST, EAST, SOUTH, NORTH = range(5)


def circle_indices_2d(dim, spacing, center, radius) -> np.ndarray:
    """Indices i + j * dim[0] of the in-plane voxels whose centre offset lies within
    ``radius`` of ``center`` (``CTDIPhantom::circleIndices2D``, world.hpp:363-390),
    in the reference's order (i outer, j inner)."""
    f0 = int((center[0] - radius) / spacing[0])
    f1 = int((center[0] + radius) / spacing[0]) + 1
    f2 = int((center[1] - radius) / spacing[1])
    f3 = int((center[1] + radius) / spacing[1]) + 1
    i0, i1 = max(f0, 0), min(f1, int(dim[0]))
    j0, j1 = max(f2, 0), min(f3, int(dim[1]))
    if i1 <= i0 or j1 <= j0:
        return np.zeros(0, np.uint64)
    i = np.arange(i0, i1, dtype=np.float64)[:, None]
    j = np.arange(j0, j1, dtype=np.float64)[None, :]
    px = center[0] - i * spacing[0] + spacing[0] / 2
    py = center[1] - j * spacing[1] + spacing[1] / 2
    inside = px * px + py * py <= radius * radius
    ii, jj = np.nonzero(inside)
    return ((ii + i0) + (jj + j0) * int(dim[0])).astype(np.uint64)


class CTDIPhantom(World):
    """PMMA CTDI phantom of the given diameter (mm): 1 x 1 x 2.5 mm voxels, 60 slices,
    five air holes of 13.1 mm diameter (centre and 13 mm inside the rim) measured
    over the central 100 mm (world.hpp:262-355).  Materials: 0 air around the
    phantom, 1 air in the holes, 2 PMMA."""

    HOLE_DIAMETER = 13.1
    HOLE_DISPLACEMENT = 13.0

    def __init__(self, diameter: int = 320):
        super().__init__()
        diameter = int(diameter)
        sp = (1.0, 1.0, 2.5)
        self.setDirectionCosines((1, 0, 0, 0, 1, 0))
        self.setSpacing(sp)
        self.setOrigin((0, 0, 0))
        n_xy = diameter + 3 if diameter % 2 == 0 else diameter + 2  # odd in-plane dimensions
        dim = (n_xy, n_xy, 60)
        self.setDimensions(dim)
        air = Material("Air, Dry (near sea level)")
        pmma = Material("Polymethyl Methacralate (Lucite, Perspex)")
        self.addMaterialToMap(air)
        self.addMaterialToMap(air)
        self.addMaterialToMap(pmma)
        hole_r = self.HOLE_DIAMETER / 2.0
        radii = diameter / 2.0
        fdim = (dim[0], dim[1])
        fsp = (sp[0], sp[1])
        fcenter = (dim[0] * sp[0] * 0.5, dim[1] * sp[1] * 0.5)
        d = self.HOLE_DISPLACEMENT
        offsets = [(0.0, 0.0), (0.0, radii - d), (0.0, -radii + d), (radii - d, 0.0), (-radii + d, 0.0)]
        centers = [(fcenter[0] + a, fcenter[1] + b) for a, b in offsets]
        nxy = dim[0] * dim[1]
        # the reference's internal hole order: 0 centre, 1 south, 2 north, 3 east, 4 west
        internal: List[List[np.ndarray]] = [[] for _ in range(5)]
        hole2d = [circle_indices_2d(fdim, fsp, c, hole_r) for c in centers]
        for k in range(dim[2]):
            z = sp[2] * (k - dim[2] * 0.5 + 0.5)
            if abs(z) <= 50.0:
                for h in range(5):
                    internal[h].append(hole2d[h] + np.uint64(k * nxy))
        self._holes = [np.concatenate(lst) if lst else np.zeros(0, np.uint64) for lst in internal]
        density = np.full(self.size(), self.airDensity(), np.float64)
        material = np.zeros(self.size(), np.uint8)
        body = circle_indices_2d(fdim, fsp, fcenter, radii)
        for k in range(dim[2]):
            off = np.uint64(k * nxy)
            density[body + off] = pmma.standardDensity()
            material[body + off] = 2
            for h in range(5):
                density[hole2d[h] + off] = air.standardDensity()
                material[hole2d[h] + off] = 1
        measurement = np.zeros(self.size(), np.uint8)
        for idx in self._holes:
            measurement[idx] = 1
        self.setDensityArray(density.astype(np.float32))
        self._density64 = density
        self.setMaterialIndexArray(material)
        self.setMeasurementMapArray(measurement)
        self.makeValid()

    @staticmethod
    def airDensity() -> float:
        return 0.001205  # g/cm3

    @staticmethod
    def ctdiMinHistories() -> int:
        return 100_000_000

    def holeIndices(self, position: int) -> np.ndarray:
        """Voxel indices of a hole (CENTER, WEST, EAST, SOUTH or NORTH)."""
        internal = {CENTER: 0, SOUTH: 1, NORTH: 2, EAST: 3, WEST: 4}[position]
        return self._holes[internal]


def ctdi_factor(world: CTDIPhantom, dose: np.ndarray, collimation_mm: float, ctdivol: float,
                mean_weight: float) -> float:
    """source.hpp:963-987: mean dose per hole, CTDIw = (centre + 2 periphery) / 3
    scaled to 100 mm over the collimation, factor = CTDIvol / CTDIw / mean weight."""
    measured = [float(np.mean(dose[world.holeIndices(p)])) for p in (CENTER, WEST, EAST, SOUTH, NORTH)]
    periphery = sum(measured[1:]) / 4.0
    ctdiw = (measured[0] + 2.0 * periphery) / 3.0 * 100.0 / collimation_mm
    return ctdivol / ctdiw / mean_weight


def calibration_histories_per_exposure(exposures_per_rotation: int, histories_per_exposure: int) -> int:
    """source.hpp:943-953: enough rotations of histories for at least 1e8 in total."""
    stat = CTDIPhantom.ctdiMinHistories() // (exposures_per_rotation * histories_per_exposure)
    return histories_per_exposure * max(int(stat), 1)


def run_ctdi(ctx, world: CTDIPhantom, exposures, spectrum, heel, bowtie, model: int, seed: int = 0x5EED):
    """One calibration run on the GPU: dose (keV/kg, uncalibrated) per voxel."""
    from .api import Beam
    dose, var, stats = _run_beams(ctx, world, [Beam(exposures, spectrum, heel, bowtie)], model, seed)
    return dose, var, stats


def run_ctdi_beams(ctx, world: CTDIPhantom, beams, model: int, seed: int = 0x5EED) -> np.ndarray:
    """The calibration run of a source whose tubes take turns (dual-source CT): one
    GPU job per beam, each with its own spectrum, heel and bow-tie tables and its
    own random streams.  DOSE output (keV/kg) is linear in the energy imparted, so
    the beams' doses add."""
    return _run_beams(ctx, world, beams, model, seed)[0]


def _run_beams(ctx, world, beams, model, seed):
    from .api import DeviceLut, DeviceWorld, Job, LutBlob, beam_seed
    dworld = DeviceWorld(ctx, world)
    dose = var = None
    stats = {"histories": 0}
    try:
        emax = max(float(np.max(b.spectrum.energies)) if b.spectrum is not None else float(np.max(b.exposures.mono_energy))
                   for b in beams)
        dlut = DeviceLut(ctx, LutBlob.cached(world.materialMap(), dworld.max_density(), emax))
        try:
            for k, b in enumerate(beams):
                job = Job(ctx, dworld, dlut, b.exposures, b.spectrum, b.heel, b.bowtie, seed=beam_seed(seed, k),
                          model=model)
                d, v, _, st = job.result(A.OUTPUT_DOSE, 1.0, want_events=False)
                job.close()
                dose = d if dose is None else dose + d
                var = v if var is None else var + v
                stats = {**st, "histories": stats["histories"] + st["histories"]}
        finally:
            dlut.close()
    finally:
        dworld.close()
    return dose, var, stats
