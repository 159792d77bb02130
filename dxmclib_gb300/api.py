"""Host-side mirror of DXMClib's World / Material / Source / Transport API.

The names, arguments and error behaviour follow the reference
(include/dxmc/world.hpp, material.hpp, source.hpp, transport.hpp); the work
happens in libdxmc_gpu.so through the C ABI (include/dxmc_gpu.h).  Geometry
(Source::getExposure) and spectrum generation stay on the host, as in the
reference; photon generation, transport and scoring run on the GPU.

There is no CPU fallback: every transport call goes through the CUDA kernels,
and ``Transport()`` raises if the library or a device is unavailable.
"""
from __future__ import annotations

import atexit
import ctypes as C
import math
import time
import weakref
from dataclasses import dataclass, field
from typing import List, Optional, Sequence

import numpy as np

from . import _capi as A

PI = math.pi
DEG_TO_RAD = PI / 180.0
ELECTRON_REST_MASS = 510.9989461
KEV_TO_MJ = 1.6021773e-13


class LOWENERGYCORRECTION:
    NONE = 0
    LIVERMORE = 1
    IA = 2


# ---------------------------------------------------------------------------
# vector helpers (vectormath.hpp)
# ---------------------------------------------------------------------------
def _normalize(v):
    v = np.asarray(v, dtype=np.float64)
    return v / np.sqrt(np.sum(v * v, axis=-1, keepdims=True))


def _cross(a, b):
    return np.cross(np.asarray(a, np.float64), np.asarray(b, np.float64))


def _rotate(vec, axis, angle):
    """vectormath::rotate (vectormath.hpp:83-99), vectorised over leading axes."""
    vec = np.asarray(vec, np.float64)
    axis = np.asarray(axis, np.float64)
    angle = np.asarray(angle, np.float64)
    s = np.sin(angle)[..., None]
    c = np.cos(angle)[..., None]
    midt = (1 - c) * np.sum(vec * axis, axis=-1, keepdims=True)
    out = np.empty(np.broadcast_shapes(vec.shape, axis.shape, c.shape))
    out[..., 0] = (c * vec[..., 0:1] + midt * axis[..., 0:1] + s * (axis[..., 1:2] * vec[..., 2:3] - axis[..., 2:3] * vec[..., 1:2]))[..., 0]
    out[..., 1] = (c * vec[..., 1:2] + midt * axis[..., 1:2] + s * (-axis[..., 0:1] * vec[..., 2:3] + axis[..., 2:3] * vec[..., 0:1]))[..., 0]
    out[..., 2] = (c * vec[..., 2:3] + midt * axis[..., 2:3] + s * (axis[..., 0:1] * vec[..., 1:2] - axis[..., 1:2] * vec[..., 0:1]))[..., 0]
    return out


# ---------------------------------------------------------------------------
# Material (material.hpp:60-139) backed by the project physics model
# ---------------------------------------------------------------------------
class Material:
    def __init__(self, name_or_z="", pretty_name: str = "", density: float = -1.0):
        lib = A.load()
        self._provider = A.MaterialProvider()
        if isinstance(name_or_z, (int, np.integer)):
            rc = lib.dxmc_physics_element_material(int(name_or_z), C.byref(self._provider))
            self._name = ""
        else:
            self._name = str(name_or_z)
            rc = lib.dxmc_physics_material(self._name.encode(), float(density), C.byref(self._provider))
        self._valid = rc == A.DXMC_OK
        self._pretty = pretty_name or self._name
        if self._valid and isinstance(name_or_z, (int, np.integer)):
            self._name = f"Z{int(name_or_z)}"
        if self._valid and density > 0:
            self._provider.standard_density = float(density)

    def isValid(self) -> bool:
        return self._valid

    def name(self) -> str:
        return self._name

    def prettyName(self) -> str:
        return self._pretty or self._name

    def standardDensity(self) -> float:
        return self._provider.standard_density if self._valid else -1.0

    def setStandardDensity(self, density: float) -> None:
        if density > 0:
            self._provider.standard_density = float(density)

    def getPhotoelectricAttenuation(self, e: float) -> float:
        return self._provider.photoelectric(self._provider.user, e)

    def getComptonAttenuation(self, e: float) -> float:
        return self._provider.compton(self._provider.user, e)

    def getRayleightAttenuation(self, e: float) -> float:
        return self._provider.rayleigh(self._provider.user, e)

    def getMassEnergyAbsorbtion(self, e: float) -> float:
        """Mass energy-absorption coefficient, cm2/g (material.hpp:74)."""
        out = C.c_double(0.0)
        A.check(A.load().dxmc_physics_mass_energy_absorption(C.byref(self._provider), float(e), C.byref(out)))
        return out.value

    def getTotalAttenuation(self, e: float) -> float:
        return self.getPhotoelectricAttenuation(e) + self.getComptonAttenuation(e) + self.getRayleightAttenuation(e)

    @property
    def provider(self) -> A.MaterialProvider:
        if not self._valid:
            raise ValueError("invalid material")
        return self._provider

    def __del__(self):
        try:
            if self._valid and A._lib is not None:
                A._lib.dxmc_physics_material_free(C.byref(self._provider))
        except Exception:
            pass


# ---------------------------------------------------------------------------
# World (world.hpp:37-227)
# ---------------------------------------------------------------------------
class World:
    def __init__(self):
        self._dims = (0, 0, 0)
        self._spacing = (1.0, 1.0, 1.0)
        self._origin = (0.0, 0.0, 0.0)
        self._cosines = (1.0, 0.0, 0.0, 0.0, 1.0, 0.0)
        self._density: Optional[np.ndarray] = None
        self._material: Optional[np.ndarray] = None
        self._measurement: Optional[np.ndarray] = None
        self._measurement_given = False  # False: validate() made the all-zero map
        self._materials: List[Material] = []
        self._valid = False

    def setDimensions(self, dims):
        self._dims = tuple(int(d) for d in dims)
        self._valid = False

    def setSpacing(self, spacing):
        self._spacing = tuple(float(s) for s in spacing)
        self._valid = False

    def setOrigin(self, origin):
        self._origin = tuple(float(o) for o in origin)
        self._valid = False

    def setDirectionCosines(self, cosines):
        c = np.asarray(cosines, np.float64)
        c = np.concatenate([_normalize(c[:3]), _normalize(c[3:])])
        self._cosines = tuple(c.tolist())
        self._valid = False

    def setDensityArray(self, density):
        self._density = np.ascontiguousarray(density, dtype=np.float32).ravel()
        self._valid = False

    def setMaterialIndexArray(self, material):
        self._material = np.ascontiguousarray(material, dtype=np.uint8).ravel()
        self._valid = False

    def setMeasurementMapArray(self, measurement):
        self._measurement = None if measurement is None else np.ascontiguousarray(measurement, dtype=np.uint8).ravel()
        self._measurement_given = measurement is not None
        self._valid = False

    def addMaterialToMap(self, material: Material) -> bool:
        self._valid = False
        if material.isValid():
            self._materials.append(material)
            return True
        return False

    def clearMaterialMap(self):
        self._materials = []
        self._valid = False

    def materialMap(self) -> List[Material]:
        return self._materials

    def dimensions(self):
        return self._dims

    def spacing(self):
        return self._spacing

    def origin(self):
        return self._origin

    def directionCosines(self):
        return self._cosines

    def densityArray(self):
        return self._density

    def materialIndexArray(self):
        return self._material

    def measurementMapArray(self):
        return self._measurement

    def size(self) -> int:
        return int(np.prod(self._dims))

    def matrixExtent(self):
        out = []
        for i in range(3):
            half = self._dims[i] * self._spacing[i] * 0.5
            out += [self._origin[i] - half, self._origin[i] + half]
        return tuple(out)

    def makeValid(self):
        if not self._valid:
            self._valid = self._validate()

    def isValid(self) -> bool:
        self.makeValid()
        return self._valid

    def _validate(self) -> bool:
        n = self.size()
        if n <= 0 or np.prod(self._spacing) <= 0:
            return False
        if self._density is None or self._material is None:
            return False
        if self._measurement is None:
            self._measurement = np.zeros(n, np.uint8)
        if len(self._density) != n or len(self._material) != n or len(self._measurement) != n:
            return False
        if not all(m.isValid() for m in self._materials):
            return False
        c = np.asarray(self._cosines)
        z = _cross(c[:3], c[3:])
        ortho = np.dot(z, c[:3]) + np.dot(z, c[3:]) + np.dot(c[:3], c[3:])
        if abs(ortho) > 0.001:
            return False
        return int(self._material.min()) >= 0 and int(self._material.max()) < len(self._materials)


# ---------------------------------------------------------------------------
# Exposures: Exposure<T> (exposure.hpp:36-304) flattened to a table
# ---------------------------------------------------------------------------
@dataclass
class ExposureTable:
    """Per-exposure records after alignToDirectionCosines (one row per exposure)."""
    position: np.ndarray          # (n, 3)
    cosines: np.ndarray           # (n, 6)
    beam_direction: np.ndarray    # (n, 3)
    collimation: np.ndarray       # (n, 4)
    weight: np.ndarray            # (n,)
    n_histories: np.ndarray       # (n,) uint64
    mono_energy: np.ndarray       # (n,)

    @staticmethod
    def build(position, cosines, collimation, weight, n_histories, mono_energy, world_cosines=(1, 0, 0, 0, 1, 0)):
        position = np.atleast_2d(np.asarray(position, np.float64))
        cosines = np.atleast_2d(np.asarray(cosines, np.float64))
        n = max(len(position), len(cosines))
        position = np.broadcast_to(position, (n, 3)).copy()
        cosines = np.broadcast_to(cosines, (n, 6)).copy()
        # Exposure constructor: normalizeDirectionCosines + calculateBeamDirection
        cosines[:, :3] = _normalize(cosines[:, :3])
        cosines[:, 3:] = _normalize(cosines[:, 3:])
        beam = _cross(cosines[:, :3], cosines[:, 3:])
        # alignToDirectionCosines(world basis): changeBasisInverse with b1, b2, b3 = b1 x b2
        wc = np.asarray(world_cosines, np.float64)
        b1, b2 = wc[:3], wc[3:]
        b3 = _cross(b1, b2)
        M = np.stack([b1, b2, b3])  # newVector[k] = dot(b_k, v)
        position = position @ M.T
        cx = cosines[:, :3] @ M.T
        cy = cosines[:, 3:] @ M.T
        beam = beam @ M.T
        cosines = np.concatenate([cx, cy], axis=1)
        coll = np.broadcast_to(np.asarray(collimation, np.float64), (n, 4)).copy()
        return ExposureTable(position, cosines, beam, coll,
                             np.broadcast_to(np.asarray(weight, np.float64), (n,)).copy(),
                             np.broadcast_to(np.asarray(n_histories, np.uint64), (n,)).copy(),
                             np.broadcast_to(np.asarray(mono_energy, np.float64), (n,)).copy())

    def __len__(self):
        return len(self.weight)

    def to_c(self) -> np.ndarray:
        """Packs the table in the layout of dxmc_exposure (19 eight-byte fields per record)."""
        n = len(self)
        buf = np.empty((n, 19), np.float64)
        buf[:, 0:3] = self.position
        buf[:, 3:9] = self.cosines
        buf[:, 9:12] = self.beam_direction
        buf[:, 12:16] = self.collimation
        buf[:, 16] = self.weight
        buf.view(np.uint64)[:, 17] = self.n_histories.astype(np.uint64)
        buf[:, 18] = self.mono_energy
        assert C.sizeof(A.Exposure) == 19 * 8
        return buf

    def as_matrix(self) -> np.ndarray:
        """(n, 19) rows: pos[3], cos[6], beam[3], coll[4], weight, n_histories, 0."""
        n = len(self)
        m = np.zeros((n, 19))
        m[:, 0:3] = self.position
        m[:, 3:9] = self.cosines
        m[:, 9:12] = self.beam_direction
        m[:, 12:16] = self.collimation
        m[:, 16] = self.weight
        m[:, 17] = self.n_histories
        return m


@dataclass
class Spectrum:
    energies: np.ndarray
    weights: np.ndarray


@dataclass
class HeelTable:
    energy_start: float
    energy_step: float
    energy_size: int
    angle_start: float
    angle_step: float
    angle_size: int
    weights: np.ndarray


from .tube import Tube, HeelFilter  # noqa: E402  (uses Material above)


# ---------------------------------------------------------------------------
# Sources (source.hpp)
# ---------------------------------------------------------------------------
class Source:
    def __init__(self):
        self._position = np.zeros(3)
        self._cosines = np.array([1.0, 0, 0, 0, 1.0, 0])
        self._hpe = int(1e6)

    def setPosition(self, pos):
        self._position = np.asarray(pos, np.float64).copy()

    def position(self):
        return self._position

    def setDirectionCosines(self, cos):
        c = np.asarray(cos, np.float64)
        self._cosines = np.concatenate([_normalize(c[:3]), _normalize(c[3:])])

    def directionCosines(self):
        return self._cosines

    def setHistoriesPerExposure(self, n: int):
        self._hpe = int(n)

    def historiesPerExposure(self) -> int:
        return self._hpe

    def totalExposures(self) -> int:
        raise NotImplementedError

    def maxPhotonEnergyProduced(self) -> float:
        return 150.0

    def validate(self) -> bool:
        return True

    def isValid(self) -> bool:
        return True

    def updateFromWorld(self, world: World) -> None:
        pass

    def exposures(self, world_cosines=(1, 0, 0, 0, 1, 0)) -> ExposureTable:
        raise NotImplementedError

    def _memo_exposures(self, world_cosines, build):
        """The exposure table for the source's current settings: built by ``build()``
        once and returned as a copy while no setting (or the world's cosines)
        changes.  Thousands of CT exposures cost about a millisecond to rebuild."""
        def norm(v):
            if isinstance(v, np.ndarray):
                return (v.dtype.str, v.shape, v.tobytes())
            if isinstance(v, (tuple, list)):
                return tuple(norm(x) for x in v)
            if v is None or isinstance(v, (bool, int, float, str, np.generic)):
                return v
            return ("object", id(v))
        key = (norm(tuple(np.asarray(world_cosines, np.float64).ravel())),
               tuple((k, norm(v)) for k, v in sorted(vars(self).items()) if k not in ("_exposure_memo", "_tube")))
        memo = getattr(self, "_exposure_memo", None)
        if memo is None or memo[0] != key:
            memo = (key, build())
            self._exposure_memo = memo
        t = memo[1]
        return ExposureTable(t.position.copy(), t.cosines.copy(), t.beam_direction.copy(), t.collimation.copy(),
                             t.weight.copy(), t.n_histories.copy(), t.mono_energy.copy())

    def spectrum(self) -> Optional[Spectrum]:
        return None

    def heel(self) -> Optional[HeelTable]:
        return None

    def bowtie(self):
        return None

    def getCalibrationValue(self, model=LOWENERGYCORRECTION.NONE, transport=None) -> float:
        return 1.0

    def beams(self, world_cosines=(1, 0, 0, 0, 1, 0)) -> list:
        """The source's exposures grouped by the spectrum, heel and bow-tie tables they
        sample (one group unless several tubes take turns)."""
        return [Beam(self.exposures(world_cosines), self.spectrum(), self.heel(), self.bowtie())]


class PencilSource(Source):
    """PencilSource (source.hpp:203-263)."""

    def __init__(self):
        super().__init__()
        self._energy = 100.0
        self._total = 10
        self._air_dose = 1.0

    def setPhotonEnergy(self, e: float):
        self._energy = min(max(float(e), 1.0), ELECTRON_REST_MASS)

    def photonEnergy(self):
        return self._energy

    def maxPhotonEnergyProduced(self):
        return self._energy

    def setTotalExposures(self, n: int):
        if n > 0:
            self._total = int(n)

    def totalExposures(self):
        return self._total

    def setAirDose(self, gycm2: float):
        if gycm2 > 0:
            self._air_dose = float(gycm2)

    def exposures(self, world_cosines=(1, 0, 0, 0, 1, 0)):
        n = self._total
        return ExposureTable.build(np.tile(self._position, (n, 1)), np.tile(self._cosines, (n, 1)), (0, 0, 0, 0),
                                   1.0, self._hpe, min(max(self._energy, 0.0), 500.0), world_cosines)

    def getCalibrationValue(self, model=LOWENERGYCORRECTION.NONE, transport=None):
        """source.hpp:238-246: airDose / (N * E * mu_en(air) * keV->mJ)."""
        air = Material("Air, Dry (near sea level)")
        n = self.totalExposures() * self.historiesPerExposure()
        mea = A.load() and _mass_energy_absorption(air, self._energy)
        return self._air_dose / (n * self._energy * mea * KEV_TO_MJ)


def _mass_energy_absorption(material: Material, energy: float) -> float:
    """Material::getMassEnergyAbsorbtion (material.cpp:56-59) from the physics model."""
    return material.getMassEnergyAbsorbtion(energy)


class IsotropicSource(Source):
    """IsotropicSource (source.hpp:265-350)."""

    def __init__(self):
        super().__init__()
        self._total = 1
        self._coll = np.zeros(4)
        self._spec = Spectrum(np.array([60.0]), np.array([1.0]))
        self._max_e = 60.0

    def setTotalExposures(self, n):
        self._total = int(n)

    def totalExposures(self):
        return self._total

    def setSpecter(self, weights, energies):
        e = np.asarray(energies, np.float64)
        self._max_e = float(e.max())
        self._spec = Spectrum(e, np.asarray(weights, np.float64))

    def maxPhotonEnergyProduced(self):
        return self._max_e

    def setCollimationAngles(self, x0, x1=None, y0=None, y1=None):
        if x1 is None or y0 is None:
            xr, yr = float(x0), float(x1 if x1 is not None else x0)
            x0, x1, y0, y1 = -xr / 2, xr / 2, -yr / 2, yr / 2
        self._coll = np.array([np.clip(x0, -PI / 2, PI / 2), np.clip(x1, -PI / 2, PI / 2),
                               np.clip(y0, -PI, PI), np.clip(y1, -PI, PI)])

    def collimationAngles(self):
        return self._coll

    def spectrum(self):
        return self._spec

    def exposures(self, world_cosines=(1, 0, 0, 0, 1, 0)):
        n = self._total
        return ExposureTable.build(np.tile(self._position, (n, 1)), np.tile(self._cosines, (n, 1)), self._coll,
                                   1.0, self._hpe, 0.0, world_cosines)


class IsotropicCTSource(IsotropicSource):
    """IsotropicCTSource (source.hpp:346-377): the isotropic source rotated about z
    through a full turn over its exposures."""

    def exposures(self, world_cosines=(1, 0, 0, 0, 1, 0)):
        n = self._total
        angle = (np.arange(n, dtype=np.float64) * 2 * PI) / n
        z = np.array([0.0, 0.0, 1.0])
        pos = _rotate(np.tile(self._position, (n, 1)), z, angle)
        cos = np.concatenate([_rotate(np.tile(self._cosines[:3], (n, 1)), z, angle),
                              _rotate(np.tile(self._cosines[3:], (n, 1)), z, angle)], axis=1)
        return ExposureTable.build(pos, cos, self._coll, 1.0, self._hpe, 0.0, world_cosines)


class DAPSource(Source):
    """DAPSource (source.hpp:379-632): a tube with spectrum and heel effect, a field
    at the source-detector distance and the dose-area-product calibration."""

    def __init__(self):
        super().__init__()
        self._sdd = 1000.0
        self._field = np.array([100.0, 100.0])
        self._coll = np.zeros(2)
        self._tube = Tube()
        self._tube.setAlFiltration(2.0)
        self._tube_rotation = 0.0
        self._total = 1000
        self._heel = True
        self._dap = 1.0
        self.setDirectionCosines(self._zero_cosines())
        self._update_field(self._field)

    @staticmethod
    def _zero_cosines():
        return np.array([-1.0, 0, 0, 0, 0, 1.0])

    def setDap(self, gycm2: float):
        if gycm2 > 0.0:
            self._dap = float(gycm2)

    def dap(self) -> float:
        return self._dap

    def getCalibrationValue(self, model=LOWENERGYCORRECTION.NONE, transport=None) -> float:
        """source.hpp:552-568: DAP / (N * sum_E E * w(E) * mu_en,air(E)) over the normalised spectrum."""
        air = Material("Air, Dry (near sea level)")
        e = self._tube.getEnergy()
        w = self._tube.getSpecter(e)
        out = sum(float(k) * float(wt) * _mass_energy_absorption(air, float(k)) for k, wt in zip(e, w))
        out *= self.totalExposures() * self.historiesPerExposure()
        return self._dap / out

    def tube(self) -> "Tube":
        return self._tube

    def maxPhotonEnergyProduced(self):
        return self._tube.voltage()

    def _update_field(self, fs):
        self._field = np.abs(np.asarray(fs, np.float64))
        self._coll = np.arctan(self._field * 0.5 / self._sdd) * 2.0

    def setFieldSize(self, mm):
        self._update_field(mm)

    def fieldSize(self):
        return self._field

    def setSourceDetectorDistance(self, mm):
        self._sdd = abs(float(mm))
        self._update_field(self._field)

    def collimationAngles(self):
        return self._coll

    def setCollimationAngles(self, angles):
        self._coll = np.abs(np.asarray(angles, np.float64))
        self._field = np.tan(self._coll / 2) * self._sdd * 2

    def setModelHeelEffect(self, on: bool):
        self._heel = bool(on)

    def setTubeRotationDeg(self, angle):
        self.setTubeRotation(angle * DEG_TO_RAD)

    def setTubeRotation(self, angle):
        diff = angle - self._tube_rotation
        cos = self._cosines.copy()
        beam = _cross(cos[:3], cos[3:])
        cos[:3] = _rotate(cos[:3], beam, diff)
        cos[3:] = _rotate(cos[3:], beam, diff)
        self.setDirectionCosines(cos)
        self._tube_rotation = angle

    def setSourceAnglesDeg(self, primary, secondary):
        self.setSourceAngles(primary * DEG_TO_RAD, secondary * DEG_TO_RAD)

    def setSourceAngles(self, primary, secondary):
        """source.hpp:441-466."""
        err = 1e-6
        secondary = min(max(secondary, -PI / 2 + err), PI / 2 - err)
        while primary > PI:
            primary -= PI
        while primary < -PI:
            primary += PI
        cos = self._zero_cosines()
        z = np.array([0.0, 0, 1.0])
        cos[:3] = _rotate(cos[:3], z, primary)
        cos[3:] = _rotate(cos[3:], z, primary)
        x = np.array([1.0, 0, 0])
        cos[:3] = _rotate(cos[:3], x, -secondary)
        cos[3:] = _rotate(cos[3:], x, -secondary)
        beam = _cross(cos[:3], cos[3:])
        cos[:3] = _rotate(cos[:3], beam, self._tube_rotation)
        cos[3:] = _rotate(cos[3:], beam, self._tube_rotation)
        self.setDirectionCosines(cos)

    def _collimation4(self):
        c = self._coll
        return (-c[0] / 2, c[0] / 2, -c[1] / 2, c[1] / 2)

    def spectrum(self):
        e = self._tube.getEnergy()
        return Spectrum(e, self._tube.getSpecter(e))

    def heel(self):
        if not self._heel:
            return None
        return HeelFilter(self._tube, self._coll[1]).table()


class DXSource(DAPSource):
    """DXSource (source.hpp:634-677): projection radiography, every exposure from the
    tube at the source-detector distance behind the position."""

    def setTotalExposures(self, n):
        self._total = max(int(n), 1)

    def totalExposures(self):
        return self._total

    def tubePosition(self):
        beam = _cross(self._cosines[:3], self._cosines[3:])
        return self._position - beam * self._sdd

    def exposures(self, world_cosines=(1, 0, 0, 0, 1, 0)):
        n = self._total
        return ExposureTable.build(np.tile(self.tubePosition(), (n, 1)), np.tile(self._cosines, (n, 1)),
                                   self._collimation4(), 1.0, self._hpe, 0.0, world_cosines)


class CBCTSource(DAPSource):
    """CBCTSource (source.hpp:679-782): the tube, at half the source-detector distance
    from the position, rotates about the source's second direction cosine in steps
    of ``stepAngle`` over ``spanAngle``."""

    def __init__(self):
        super().__init__()
        self._total = 180
        self._span = PI
        self._step_angle = PI / 180
        self.setSourceDetectorDistance(500.0)

    def setSpanAngle(self, a):
        self._span = max(float(a), self._step_angle)
        self._total = max(int(self._span / self._step_angle), 2)

    def setSpanAngleDeg(self, a):
        self.setSpanAngle(a * DEG_TO_RAD)

    def spanAngle(self):
        return self._span

    def spanAngleDeg(self):
        return self._span / DEG_TO_RAD

    def setStepAngle(self, a):
        self._step_angle = max(float(a), PI / 360)
        self._total = max(int(self._span / self._step_angle), 2)

    def setStepAngleDeg(self, a):
        self.setStepAngle(a * DEG_TO_RAD)

    def stepAngle(self):
        return self._step_angle

    def stepAngleDeg(self):
        return self._step_angle / DEG_TO_RAD

    def totalExposures(self):
        return self._total

    def rotationAxis(self):
        return self._cosines[3:].copy()

    def tubePosition(self):
        beam = _cross(self._cosines[:3], self._cosines[3:])
        return self._position - beam * self._sdd * 0.5

    def exposures(self, world_cosines=(1, 0, 0, 0, 1, 0)):
        n = self._total
        angle = np.arange(n, dtype=np.float64) * self._step_angle
        axis = self.rotationAxis()
        iso = _rotate(np.tile(self.tubePosition() - self._position, (n, 1)), axis, angle) + self._position
        cos = np.concatenate([_rotate(np.tile(self._cosines[:3], (n, 1)), axis, angle),
                              _rotate(np.tile(self._cosines[3:], (n, 1)), axis, angle)], axis=1)
        return ExposureTable.build(iso, cos, self._collimation4(), 1.0, self._hpe, 0.0, world_cosines)


class Beam:
    """The exposures of a source that sample one spectrum, heel table and bow-tie
    filter: one per source, two for dual-source CT (source.hpp:1384-1410), each run
    as a job of its own."""

    def __init__(self, exposures: ExposureTable, spectrum, heel, bowtie):
        self.exposures = exposures
        self.spectrum = spectrum
        self.heel = heel
        self.bowtie = bowtie


def _take(table: ExposureTable, rows) -> ExposureTable:
    return ExposureTable(table.position[rows].copy(), table.cosines[rows].copy(), table.beam_direction[rows].copy(),
                         table.collimation[rows].copy(), table.weight[rows].copy(), table.n_histories[rows].copy(),
                         table.mono_energy[rows].copy())


class _CTBase(Source):
    """CTBaseSource and CTSource (source.hpp:794-1076): the geometry, tube, heel,
    bow-tie and CTDI settings every CT source shares, and the construction of
    exposures around the gantry that their getExposure implementations repeat."""

    def __init__(self):
        super().__init__()
        self._sdd = 1190.0
        self._collimation = 38.4
        self._fov = 500.0
        self._start = 0.0
        self._scan = 100.0
        self._tilt = 0.0
        self._step = DEG_TO_RAD  # CTSource::m_exposureAngleStep
        self._tube = Tube()
        self._tube.setAlFiltration(7.0)
        self._heel = True
        self._bowtie = None
        self.setDirectionCosines([-1, 0, 0, 0, 0, 1])

    def tube(self):
        return self._tube

    def maxPhotonEnergyProduced(self):
        return self._tube.voltage()

    def setSourceDetectorDistance(self, sdd):
        self._sdd = abs(float(sdd))

    def sourceDetectorDistance(self):
        return self._sdd

    def setCollimation(self, c):
        self._collimation = abs(float(c))

    def collimation(self):
        return self._collimation

    def setFieldOfView(self, fov):
        self._fov = abs(float(fov))

    def fieldOfView(self):
        return self._fov

    def setGantryTiltAngle(self, a):
        self._tilt = min(max(float(a), -PI), PI)

    def setGantryTiltAngleDeg(self, a):
        self.setGantryTiltAngle(a * DEG_TO_RAD)

    def gantryTiltAngle(self):
        return self._tilt

    def gantryTiltAngleDeg(self):
        return self._tilt / DEG_TO_RAD

    def setStartAngle(self, a):
        self._start = float(a)

    def setStartAngleDeg(self, a):
        self._start = DEG_TO_RAD * a

    def startAngle(self):
        return self._start

    def startAngleDeg(self):
        return self._start / DEG_TO_RAD

    def setScanLenght(self, length):
        self._scan = abs(float(length))

    def setScanLength(self, length):
        self.setScanLenght(length)

    def scanLenght(self):
        return self._scan

    def setExposureAngleStep(self, a):
        self._step = min(max(abs(float(a)), DEG_TO_RAD / 10), PI / 2)

    def setExposureAngleStepDeg(self, a):
        self.setExposureAngleStep(a * DEG_TO_RAD)

    def exposureAngleStep(self):
        return self._step

    def exposureAngleStepDeg(self):
        return self._step / DEG_TO_RAD

    def setModelHeelEffect(self, on):
        self._heel = bool(on)

    def modelHeelEffect(self):
        return self._heel

    def setBowTieFilter(self, angles, weights):
        self._bowtie = (np.asarray(angles, np.float64), np.asarray(weights, np.float64))

    def bowtie(self):
        return self._bowtie

    def setCtdiVol(self, ctdivol: float):
        if ctdivol > 0.0:
            self._ctdivol = float(ctdivol)

    def ctdiVol(self) -> float:
        return getattr(self, "_ctdivol", 1.0)

    def setCtdiPhantomDiameter(self, mm: int):
        self._ctdi_diameter = max(int(mm), 160)

    def ctdiPhantomDiameter(self) -> int:
        return getattr(self, "_ctdi_diameter", 320)

    def exposuresPerRotatition(self) -> int:
        return int(2 * PI / self._step)

    def spectrum(self):
        e = self._tube.getEnergy()
        return Spectrum(e, self._tube.getSpecter(e))

    def _heel_span(self):
        return math.atan(self._collimation * 0.5 / self._sdd) * 2.0

    def heel(self):
        if not self._heel:
            return None
        return HeelFilter(self._tube, self._heel_span()).table()

    def exposures(self, world_cosines=(1, 0, 0, 0, 1, 0)):
        return self._memo_exposures(world_cosines, lambda: self._build_exposures(world_cosines))

    def _gantry(self, angle, z, sdd, fov, weight, world_cosines):
        """Exposures at gantry angles ``angle`` (the rotation about the tilted axis) with
        table offsets ``z``: the tube at half the source-detector distance from the
        isocentre, the fan from ``fov`` and the collimation at distance ``sdd``."""
        angle = np.asarray(angle, np.float64)
        n = len(angle)
        pos0 = np.array([0.0, -self._sdd / 2, 0.0])
        cos = np.tile(self._cosines, (n, 1))
        tilt_axis = np.array([1.0, 0, 0])
        tilt_corr = _rotate(pos0, tilt_axis, self._tilt)
        rot_axis = _rotate(cos[:, 3:], tilt_axis, self._tilt)
        other = _rotate(cos[:, :3], tilt_axis, self._tilt)
        pos = _rotate(np.tile(pos0, (n, 1)), rot_axis, angle)
        pos[:, 2] += z + tilt_corr[2]
        other = _rotate(other, rot_axis, angle)
        pos += self._position
        cosines = np.concatenate([other, rot_axis], axis=1)
        coll_x = np.arctan(np.asarray(fov, np.float64) / sdd) * 2.0
        coll_y = np.arctan(self._collimation / np.asarray(sdd, np.float64)) * 2.0
        coll = np.stack(np.broadcast_arrays(-coll_x / 2, coll_x / 2, -coll_y / 2, coll_y / 2), axis=-1)
        return ExposureTable.build(pos, cosines, coll, weight, self._hpe, 0.0, world_cosines)

    def _ct_calibration(self, copy, mean_weight: float, model: int, transport) -> float:
        """CTBaseSource::ctCalibration (source.hpp:925-988) on an axial copy of the
        source, the CTDI run as GPU jobs (one per beam)."""
        from . import calibration as cal
        ctx = transport.context() if transport is not None else GpuContext()
        copy.setDirectionCosines([-1, 0, 0, 0, 0, 1])
        copy.setPosition([0, 0, 0])
        copy.setScanLenght(copy.collimation())
        hpe = cal.calibration_histories_per_exposure(copy.exposuresPerRotatition(), copy.historiesPerExposure())
        world = cal.CTDIPhantom(copy.ctdiPhantomDiameter())
        copy.setHistoriesPerExposure(hpe)
        dose = cal.run_ctdi_beams(ctx, world, copy.beams(world.directionCosines()), int(model))
        return cal.ctdi_factor(world, dose, copy.collimation(), copy.ctdiVol(), mean_weight)

    def _base_state(self):
        # the CTBaseSource members a copy takes over (source.hpp:1005-1019)
        return {k: getattr(self, k) for k in ("_position", "_cosines", "_hpe", "_sdd", "_collimation", "_fov",
                                              "_start", "_scan", "_tilt", "_tube", "_heel", "_bowtie")
                if hasattr(self, k)} | {k: v for k, v in vars(self).items() if k in ("_ctdivol", "_ctdi_diameter")}


class CTSpiralSource(_CTBase):
    """CTSpiralSource (source.hpp:1286-1367)."""

    def __init__(self):
        super().__init__()
        self._pitch = 1.0

    def setPitch(self, p):
        self._pitch = max(0.01, float(p))

    def pitch(self):
        return self._pitch

    def setScanLenght(self, length):
        self._scan = max(abs(float(length)), self._collimation * self._pitch * 0.5)

    def totalExposures(self):
        return int(self._scan * 2 * PI / (self._collimation * self._pitch * self._step))

    def _build_exposures(self, world_cosines):
        idx = np.arange(self.totalExposures(), dtype=np.float64)
        angle = self._start + self._step * idx
        z = (idx * self._step) * self._collimation * self._pitch / (2 * PI)
        return self._gantry(angle, z, self._sdd, self._fov, 1.0, world_cosines)

    def _axial_copy(self):
        """CTAxialSource(const CTSpiralSource&) (source.hpp:1603-1608)."""
        a = CTAxialSource()
        for k, v in self._base_state().items():
            setattr(a, k, v)
        a._step = self._step
        a._axial_step = self._collimation
        a.setScanLenght(self._scan)
        return a

    def calibration_exposures(self, histories_per_exposure: int, world_cosines=(1, 0, 0, 0, 1, 0)) -> ExposureTable:
        """Exposures of the axial copy that ctCalibration runs (source.hpp:937-942,
        1203-1255): one rotation about the phantom axis at the origin, the
        source's angles, tilt, collimation and field of view."""
        a = self._axial_copy()
        a.setDirectionCosines([-1, 0, 0, 0, 0, 1])
        a.setPosition([0, 0, 0])
        a.setScanLenght(a.collimation())
        a.setHistoriesPerExposure(histories_per_exposure)
        return a.exposures(world_cosines)

    def getCalibrationValue(self, model=LOWENERGYCORRECTION.NONE, transport=None) -> float:
        """CTSpiralSource::getCalibrationValue (source.hpp:1358-1363): the CTDI
        calibration of the axial copy, run as a GPU job, times the pitch."""
        copy = self._axial_copy()
        mean_weight = float(np.mean(copy.exposures().weight))
        return self._ct_calibration(copy, mean_weight, model, transport) * self._pitch


class CTAxialSource(_CTBase):
    """CTAxialSource (source.hpp:1192-1285): rotations at table steps of ``step``
    (the collimation the source was constructed with, unless set)."""

    def __init__(self):
        super().__init__()
        self._axial_step = self._collimation
        self._scan = self._axial_step

    def setStep(self, step):
        n_steps = self._scan / self._axial_step
        a = abs(float(step))
        self._axial_step = a if a > 0.01 else 0.01
        self.setScanLenght(self._axial_step * n_steps)

    def step(self):
        return self._axial_step

    def setScanLenght(self, length):
        self._scan = max(self._axial_step * math.ceil(abs(float(length)) / self._axial_step), self._axial_step)

    def _rotations(self) -> int:
        return int(round(self._scan / self._axial_step))

    def totalExposures(self):
        return int(2 * PI / self._step) * self._rotations()

    def _build_exposures(self, world_cosines):
        apr = int(2 * PI / self._step)
        i = np.arange(self.totalExposures(), dtype=np.int64)
        rot = i // apr
        angle = self._start + self._step * (i - rot * apr).astype(np.float64)
        z = self._axial_step * rot.astype(np.float64)
        return self._gantry(angle, z, self._sdd, self._fov, 1.0, world_cosines)

    def getCalibrationValue(self, model=LOWENERGYCORRECTION.NONE, transport=None) -> float:
        """CTAxialSource::getCalibrationValue (source.hpp:1277-1281)."""
        copy = CTAxialSource()
        copy.__dict__.update({k: v for k, v in vars(self).items() if k != "_exposure_memo"})
        mean_weight = float(np.mean(copy.exposures().weight))
        return self._ct_calibration(copy, mean_weight, model, transport)


class _CTDual:
    """CTDualSource (source.hpp:1078-1190): a second tube B with its own spectrum,
    heel table, bow-tie filter, distance, field of view and start angle; the
    exposures alternate A, B, and each tube's weight is its share of mAs times
    its unnormalised spectrum, normalised to a mean of one."""

    def _init_dual(self):
        self._sdd_b = self._sdd
        self._fov_b = self._fov
        self._start_b = self._start + PI * 0.5
        self._tube_b = Tube()
        self._tube_b.setAlFiltration(self._tube.AlFiltration())
        self._mas_a = 100.0
        self._mas_b = 100.0
        self._bowtie_b = None

    def tubeB(self):
        return self._tube_b

    def tubeAmas(self):
        return self._mas_a

    def tubeBmas(self):
        return self._mas_b

    def setTubeAmas(self, mas):
        self._mas_a = max(0.0, float(mas))

    def setTubeBmas(self, mas):
        self._mas_b = max(0.0, float(mas))

    def maxPhotonEnergyProduced(self):
        return max(self._tube.voltage(), self._tube_b.voltage())

    def exposuresPerRotatition(self) -> int:
        return 2 * int(2 * PI / self._step)

    def setBowTieFilterB(self, angles, weights):
        self._bowtie_b = (np.asarray(angles, np.float64), np.asarray(weights, np.float64))

    def bowtieB(self):
        return self._bowtie_b

    def setSourceDetectorDistanceB(self, sdd):
        self._sdd_b = abs(float(sdd))

    def sourceDetectorDistanceB(self):
        return self._sdd_b

    def setFieldOfViewB(self, fov):
        self._fov_b = abs(float(fov))

    def fieldOfViewB(self):
        return self._fov_b

    def setStartAngleB(self, a):
        self._start_b = float(a)

    def setStartAngleDegB(self, a):
        self._start_b = DEG_TO_RAD * a

    def startAngleB(self):
        return self._start_b

    def startAngleDegB(self):
        return self._start_b / DEG_TO_RAD

    def tubeWeights(self):
        """(weight A, weight B) of CTDualSource::updateSpecterDistribution."""
        sa = float(np.sum(self._tube.getSpecter(self._tube.getEnergy(), normalize=False)))
        sb = float(np.sum(self._tube_b.getSpecter(self._tube_b.getEnergy(), normalize=False)))
        wa, wb = self._mas_a * sa, self._mas_b * sb
        return wa * 2.0 / (wa + wb), wb * 2.0 / (wa + wb)

    def spectrumB(self):
        e = self._tube_b.getEnergy()
        return Spectrum(e, self._tube_b.getSpecter(e))

    def heel(self):
        # the dual source builds both heel tables whatever modelHeelEffect says
        return HeelFilter(self._tube, self._heel_span()).table()

    def heelB(self):
        return HeelFilter(self._tube_b, self._heel_span()).table()

    def _tube_params(self, i):
        """Per total exposure index: (exposure index, sdd, start angle, fov, weight)."""
        tube_b = (i % 2) == 1
        wa, wb = self.tubeWeights()
        return (i // 2, np.where(tube_b, self._sdd_b, self._sdd), np.where(tube_b, self._start_b, self._start),
                np.where(tube_b, self._fov_b, self._fov), np.where(tube_b, wb, wa))

    def beams(self, world_cosines=(1, 0, 0, 0, 1, 0)):
        ex = self.exposures(world_cosines)
        return [Beam(_take(ex, slice(0, None, 2)), self.spectrum(), self.heel(), self.bowtie()),
                Beam(_take(ex, slice(1, None, 2)), self.spectrumB(), self.heelB(), self.bowtieB())]

    def _dual_state(self):
        return {k: getattr(self, k) for k in ("_sdd_b", "_fov_b", "_start_b", "_tube_b", "_mas_a", "_mas_b",
                                              "_bowtie_b")}


class CTSpiralDualSource(_CTDual, CTSpiralSource):
    """CTSpiralDualSource (source.hpp:1488-1600)."""

    def __init__(self):
        CTSpiralSource.__init__(self)
        self._init_dual()

    def totalExposures(self):
        return 2 * int(self._scan * 2 * PI / (self._collimation * self._pitch * self._step))

    def _build_exposures(self, world_cosines):
        i = np.arange(self.totalExposures(), dtype=np.int64)
        e, sdd, start, fov, weight = self._tube_params(i)
        ef = e.astype(np.float64)
        angle = start + self._step * ef
        z = (ef * self._step) * self._collimation * self._pitch / (2 * PI)
        return self._gantry(angle, z, sdd, fov, weight, world_cosines)

    def _axial_copy(self):
        """CTAxialDualSource(const CTSpiralDualSource&) (source.hpp:1610-1616)."""
        a = CTAxialDualSource()
        for k, v in {**self._base_state(), **self._dual_state()}.items():
            setattr(a, k, v)
        a._step = self._step
        a._axial_step = self._collimation
        a.setScanLenght(self._scan)
        return a


class CTAxialDualSource(_CTDual, CTAxialSource):
    """CTAxialDualSource (source.hpp:1369-1486)."""

    def __init__(self):
        CTAxialSource.__init__(self)
        self._init_dual()

    def totalExposures(self):
        return int(2 * PI / self._step) * self._rotations() * 2

    def _build_exposures(self, world_cosines):
        apr = int(2 * PI / self._step)
        i = np.arange(self.totalExposures(), dtype=np.int64)
        e, sdd, start, fov, weight = self._tube_params(i)
        rot = e // apr
        angle = start + self._step * (e - rot * apr).astype(np.float64)
        z = self._axial_step * rot.astype(np.float64)
        return self._gantry(angle, z, sdd, fov, weight, world_cosines)

    def getCalibrationValue(self, model=LOWENERGYCORRECTION.NONE, transport=None) -> float:
        copy = CTAxialDualSource()
        copy.__dict__.update({k: v for k, v in vars(self).items() if k != "_exposure_memo"})
        mean_weight = float(np.mean(copy.exposures().weight))
        return self._ct_calibration(copy, mean_weight, model, transport)


class CTTopogramSource(_CTBase):
    """CTTopogramSource (source.hpp:1618-1702): a fixed gantry angle and one exposure
    per millimetre of scan length."""

    def totalExposures(self):
        return max(int(math.ceil(self._scan)), 1)

    def _build_exposures(self, world_cosines):
        n = self.totalExposures()
        step = self._scan / (n - 1) if n > 1 else math.inf
        i = np.arange(n, dtype=np.float64)
        with np.errstate(invalid="ignore"):
            z = step * i
        return self._gantry(np.full(n, self._start), z, self._sdd, self._fov, 1.0, world_cosines)

    def getCalibrationValue(self, model=LOWENERGYCORRECTION.NONE, transport=None) -> float:
        """CTTopogramSource::getCalibrationValue (source.hpp:1679-1701): an axial copy
        stepping one collimation, CTDIvol scaled by the scan length over the
        collimation, at an angle step that matches the number of exposures."""
        copy = CTAxialSource()
        for k, v in self._base_state().items():
            setattr(copy, k, v)
        copy.setCtdiVol(self.ctdiVol() * self._scan / self._collimation)
        copy.setScanLenght(0)
        copy.setStep(self._collimation)
        n = self.totalExposures()
        copy.setExposureAngleStep(min(2 * PI / n, (2 * PI) / 72))
        mean_weight = float(np.mean(copy.exposures().weight))
        factor = self._ct_calibration(copy, mean_weight, model, transport)
        return factor * n / copy.totalExposures()


# ---------------------------------------------------------------------------
# Result (transport.hpp:42-65) and Transport (transport.hpp:114-840)
# ---------------------------------------------------------------------------
@dataclass
class Result:
    dose: np.ndarray
    nEvents: np.ndarray
    variance: np.ndarray
    numberOfHistories: int = 0
    simulationTime: float = 0.0
    dose_units: str = ""
    stats: dict = field(default_factory=dict)

    def relativeError(self) -> np.ndarray:
        with np.errstate(divide="ignore", invalid="ignore"):
            return np.where(self.dose > 0, np.sqrt(np.maximum(self.variance, 0)) / self.dose, 0.0)


_live_contexts: "weakref.WeakSet[GpuContext]" = weakref.WeakSet()


@atexit.register
def _close_contexts():
    """Releases every device object before interpreter teardown, children first,
    so that no world, LUT or job outlives the context it belongs to."""
    for ctx in list(_live_contexts):
        ctx.close()


class GpuContext:
    """Owns a dxmc_gpu_ctx; one per device per process is enough.  Closing it
    closes the batches, jobs, LUTs and worlds created on it first."""

    _CLOSE_ORDER = ("Batch", "Job", "DeviceLut", "DeviceWorld")

    def __init__(self, device: int = 0, block_size: int = 0, blocks_per_sm: int = 0, tally_mode: int = A.TALLY_F64,
                 memory_budget: int = 0, regen_threshold: int = 0, interact_threshold: int = 0,
                 queue_log2_chunk: int = 0, tracking: int = A.TRACKING_DEFAULT):
        """``tracking``: A.TRACKING_LOCAL (default) draws Woodcock flights with the
        local-majorant grid of each (world, LUT) pair, A.TRACKING_GLOBAL with the
        reference's single global majorant; both sample the same process."""
        self.lib = A.load()
        opts = A.GpuOptions(device, block_size, blocks_per_sm, tally_mode, memory_budget, regen_threshold,
                            interact_threshold, queue_log2_chunk, tracking)
        self.options = dict(device=device, block_size=block_size, blocks_per_sm=blocks_per_sm, tally_mode=tally_mode,
                            memory_budget=memory_budget, regen_threshold=regen_threshold,
                            interact_threshold=interact_threshold, queue_log2_chunk=queue_log2_chunk,
                            tracking=tracking)
        self.handle = C.c_void_p()
        self._children = weakref.WeakSet()
        A.check(self.lib.dxmc_gpu_ctx_create(C.byref(opts), C.byref(self.handle)), None, "dxmc_gpu_ctx_create")
        _live_contexts.add(self)

    def _register(self, obj):
        self._children.add(obj)

    def memory(self) -> tuple:
        """(budget, in_use) device bytes of the context's admission check."""
        b, u = C.c_uint64(), C.c_uint64()
        A.check(self.lib.dxmc_gpu_ctx_memory(self.handle, C.byref(b), C.byref(u)), self.handle, "dxmc_gpu_ctx_memory")
        return b.value, u.value

    def close(self):
        if self.handle:
            children = list(self._children)
            for kind in self._CLOSE_ORDER:
                for obj in children:
                    if type(obj).__name__ == kind:
                        obj.close()
            self.lib.dxmc_gpu_ctx_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class DeviceWorld:
    def __init__(self, ctx: GpuContext, world: World, layout: int = 0):
        if not world.isValid():
            raise ValueError("invalid world")
        self.ctx = ctx
        self.world = world
        d = A.WorldDesc()
        d.dims[:] = list(world.dimensions())
        d.spacing[:] = list(world.spacing())
        d.origin[:] = list(world.origin())
        d.direction_cosines[:] = list(world.directionCosines())
        dens = world.densityArray()
        mat = world.materialIndexArray()
        meas = world.measurementMapArray()
        d.density = dens.ctypes.data_as(A.FP)
        d.material = mat.ctypes.data_as(A.U8P)
        # the all-zero map that validation creates stays on the host (no forced scoring)
        d.measurement = meas.ctypes.data_as(A.U8P) if meas is not None and world._measurement_given else None
        d.n_materials = len(world.materialMap())
        d.layout = int(layout)
        self.handle = C.c_void_p()
        A.check(ctx.lib.dxmc_gpu_world_upload(ctx.handle, C.byref(d), C.byref(self.handle)), ctx.handle, "dxmc_gpu_world_upload")
        ctx._register(self)

    def radiological_path(self, dlut: "DeviceLut", rays) -> np.ndarray:
        """Siddon traversal (dxmc_gpu_radiological_path): ``rays`` (n, 7) origin (mm, grid
        frame), direction, energy (keV); returns sum mu/rho * density * length (cm)."""
        r = np.ascontiguousarray(rays, np.float32).reshape(-1, 7)
        out = np.zeros(len(r))
        A.check(self.ctx.lib.dxmc_gpu_radiological_path(self.ctx.handle, self.handle, dlut.handle,
                                                        r.ctypes.data_as(A.FP), len(r), out.ctypes.data_as(A.DP)),
                self.ctx.handle, "dxmc_gpu_radiological_path")
        return out

    def prepare(self, dlut: "DeviceLut"):
        """Builds the local-majorant grid for ``dlut`` ahead of the first job
        (dxmc_gpu_world_prepare); jobs with local tracking otherwise build it on first use."""
        A.check(self.ctx.lib.dxmc_gpu_world_prepare(self.ctx.handle, self.handle, dlut.handle), self.ctx.handle,
                "dxmc_gpu_world_prepare")

    def majorant(self, dlut: "DeviceLut"):
        """The local-majorant grid built for ``dlut``: (shift (3,), band edges in keV
        (bands - 1,), box (6,) lo / hi in mm of the cells above their band's emptiest
        level, cells (nz, ny, nx, bands, 2) holding 1 / scale and R in mm, R < 0
        outside the box)."""
        n = (C.c_uint32 * 3)()
        sh = (C.c_int32 * 3)()
        nb = C.c_int32()
        edges = np.zeros(8, np.float32)
        box = np.zeros(6, np.float32)
        A.check(self.ctx.lib.dxmc_gpu_world_majorant(self.ctx.handle, self.handle, dlut.handle, n, sh, C.byref(nb),
                                                     edges.ctypes.data_as(A.FP), box.ctypes.data_as(A.FP), None),
                self.ctx.handle, "dxmc_gpu_world_majorant")
        cells = np.zeros((n[2], n[1], n[0], nb.value, 2), np.float32)
        A.check(self.ctx.lib.dxmc_gpu_world_majorant(self.ctx.handle, self.handle, dlut.handle, n, sh, C.byref(nb),
                                                     None, None, cells.ctypes.data_as(A.FP)), self.ctx.handle,
                "dxmc_gpu_world_majorant")
        return (np.array(sh[:], np.int64), edges[:nb.value - 1].astype(np.float64), box.astype(np.float64), cells)

    def max_density(self) -> np.ndarray:
        n = len(self.world.materialMap())
        out = np.zeros(n)
        A.check(self.ctx.lib.dxmc_gpu_world_max_density(self.handle, out.ctypes.data_as(A.DP), n), self.ctx.handle,
                "dxmc_gpu_world_max_density")
        return out

    def close(self):
        if self.handle and self.ctx.handle:
            self.ctx.lib.dxmc_gpu_world_free(self.handle)
        self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class LutBlob:
    """Host LUT (AttenuationLut<T>::generate) built by libdxmc_gpu."""

    def __init__(self, materials: Sequence[Material], max_density: Sequence[float], max_energy: float):
        self.lib = A.load()
        provs = (A.MaterialProvider * len(materials))(*[m.provider for m in materials])
        md = np.ascontiguousarray(max_density, np.float64)
        self.handle = C.c_void_p()
        A.check(self.lib.dxmc_lut_build_max_density(provs, len(materials), md.ctypes.data_as(A.DP), float(max_energy),
                                                    C.byref(self.handle)), None, "dxmc_lut_build_max_density")
        self.n_materials = len(materials)

    _cache = {}
    _cache_order: list = []
    CACHE_SIZE = 16

    @classmethod
    def cached(cls, materials: Sequence[Material], max_density: Sequence[float], max_energy: float) -> "LutBlob":
        """LUT for a material set, per-material maximum density and maximum energy, built
        once and reused: the table depends on nothing else (attenuationlut.hpp:64-96)."""
        key = (tuple((m.name(), m.standardDensity()) for m in materials),
               tuple(float(d) for d in max_density), float(max_energy))
        blob = cls._cache.get(key)
        if blob is None:
            blob = cls(materials, max_density, max_energy)
            blob._materials_ref = list(materials)
            cls._cache[key] = blob
            cls._cache_order.append(key)
            if len(cls._cache_order) > cls.CACHE_SIZE:
                old = cls._cache_order.pop(0)
                cls._cache.pop(old).close()
        return blob

    @staticmethod
    def from_world(world: World, max_energy: float) -> "LutBlob":
        mats = world.materialMap()
        md = np.zeros(len(mats))
        dens = world.densityArray()
        mat = world.materialIndexArray()
        np.maximum.at(md, mat, dens.astype(np.float64))
        return LutBlob(mats, md, max_energy)

    def attenuation(self, material: int, energy: float) -> np.ndarray:
        out = np.zeros(3)
        A.check(self.lib.dxmc_lut_attenuation(self.handle, material, energy, out.ctypes.data_as(A.DP)))
        return out

    def max_attenuation_inverse(self, energy: float) -> float:
        return self.lib.dxmc_lut_max_attenuation_inverse(self.handle, energy)

    def scatter_factor(self, material: int, q: float) -> float:
        return self.lib.dxmc_lut_scatter_factor(self.handle, material, q)

    def info(self) -> dict:
        i = A.LutInfo()
        A.check(self.lib.dxmc_lut_get_info(self.handle, C.byref(i)))
        R, nm = i.n_energy, i.n_materials
        shells = np.zeros((nm, 12, 13))
        for k in range(nm * 12):
            s = i.shells[k]
            shells.reshape(-1, 13)[k] = [s.binding_energy, s.number_electrons, s.hartree_fock_j0,
                                         s.photo_ionization_probability, s.fluorescence_yield,
                                         *s.line_probabilities, *s.line_energies, s.Z, s.shell]
        return dict(
            n_energy=R, linear_index=i.linear_index, linear_step=i.linear_step, linear_energy=i.linear_energy,
            min_energy=i.min_energy, max_energy=i.max_energy,
            x=np.ctypeslib.as_array(i.log_energy, (R,)).copy(),
            coef=np.ctypeslib.as_array(i.coefficients, (nm * R * 6,)).copy(),
            maxcoef=np.ctypeslib.as_array(i.max_coefficients, (R * 2,)).copy(),
            rita=np.ctypeslib.as_array(i.rita, (nm * 4 * 56,)).reshape(nm, 4, 56).copy(),
            spline=np.ctypeslib.as_array(i.spline, (nm * 79,)).reshape(nm, 79).copy(),
            shells=shells.copy())

    def close(self):
        if self.handle:
            self.lib.dxmc_lut_blob_free(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class DeviceLut:
    def __init__(self, ctx: GpuContext, blob: LutBlob):
        self.ctx = ctx
        self.handle = C.c_void_p()
        A.check(ctx.lib.dxmc_gpu_lut_upload(ctx.handle, blob.handle, C.byref(self.handle)), ctx.handle, "dxmc_gpu_lut_upload")
        ctx._register(self)

    def probe(self, material: int, energies) -> tuple:
        e = np.ascontiguousarray(energies, np.float64)
        att = np.zeros((len(e), 3))
        mi = np.zeros(len(e))
        A.check(self.ctx.lib.dxmc_gpu_probe_lut(self.ctx.handle, self.handle, material, e.ctypes.data_as(A.DP), len(e),
                                                att.ctypes.data_as(A.DP), mi.ctypes.data_as(A.DP)), self.ctx.handle, "probe_lut")
        return att, mi

    def probe_interactions(self, material: int, model: int, kind: int, energy: float, n: int, seed: int = 1):
        c = np.zeros(n, np.float32)
        e = np.zeros(n, np.float32)
        d = np.zeros(n, np.float32)
        A.check(self.ctx.lib.dxmc_gpu_probe_interactions(self.ctx.handle, self.handle, material, model, kind, float(energy), n,
                                                         seed, c.ctypes.data_as(A.FP), e.ctypes.data_as(A.FP),
                                                         d.ctypes.data_as(A.FP)), self.ctx.handle, "probe_interactions")
        return c, e, d

    def close(self):
        if self.handle and self.ctx.handle:
            self.ctx.lib.dxmc_gpu_lut_free(self.handle)
        self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Job:
    """One submitted transport job (dxmc_gpu_job_*)."""

    def __init__(self, ctx: GpuContext, dworld: DeviceWorld, dlut: DeviceLut, exposures: ExposureTable,
                 spectrum: Optional[Spectrum] = None, heel: Optional[HeelTable] = None, bowtie=None,
                 seed: int = 1, model: int = LOWENERGYCORRECTION.LIVERMORE, tally_mode: int = -1,
                 launch: Optional[dict] = None, tracking: int = A.TRACKING_DEFAULT,
                 direction: int = A.DIRECTION_REFERENCE, precision: int = A.PRECISION_FP32):
        """``launch`` may set the keys of LAUNCH_KEYS for this job (an autotuner's
        choice); unset keys use the context's.  ``tracking``: A.TRACKING_* (the
        context's when DEFAULT).  ``direction``: A.DIRECTION_REFERENCE (the
        reference's peturb) or A.DIRECTION_NORMALIZED (unit scattering axis).
        ``precision``: A.PRECISION_FP32 (FP32 transport, FP64 tallies) or
        A.PRECISION_FP64 (FP64 everywhere, as Transport<double>)."""
        self.ctx = ctx
        self.dworld = dworld
        self._owned = True
        if tracking != A.TRACKING_DEFAULT:
            launch = dict(launch or {}, tracking=tracking)
        if direction != A.DIRECTION_REFERENCE:
            launch = dict(launch or {}, direction=direction)
        if precision != A.PRECISION_FP32:
            launch = dict(launch or {}, precision=precision)
        jd = self._describe(exposures, spectrum, heel, bowtie, seed, model, tally_mode, launch)
        self.handle = C.c_void_p()
        A.check(ctx.lib.dxmc_gpu_job_submit(ctx.handle, dworld.handle, dlut.handle, C.byref(jd), C.byref(self.handle)),
                ctx.handle, "dxmc_gpu_job_submit")
        ctx._register(self)

    @classmethod
    def _member(cls, ctx: GpuContext, dworld: DeviceWorld, handle: C.c_void_p) -> "Job":
        """Job handle owned by a Batch."""
        j = cls.__new__(cls)
        j.ctx, j.dworld, j.handle, j._owned = ctx, dworld, handle, False
        return j

    LAUNCH_KEYS = ("regen_threshold", "interact_threshold", "blocks_per_sm", "queue_log2_chunk", "woodcock_burst",
                   "block_size", "tracking", "direction", "precision")

    def _describe(self, exposures: ExposureTable, spectrum, heel, bowtie, seed, model, tally_mode,
                  launch: Optional[dict] = None) -> A.JobDesc:
        self._keep = []
        jd = A.JobDesc()
        ex = exposures.to_c()
        self._keep.append(ex)
        jd.exposures = ex.ctypes.data_as(C.POINTER(A.Exposure))
        jd.n_exposures = len(exposures)
        if spectrum is not None:
            se = np.ascontiguousarray(spectrum.energies, np.float64)
            sw = np.ascontiguousarray(spectrum.weights, np.float64)
            sd = A.SpectrumDesc(len(se), se.ctypes.data_as(A.DP), sw.ctypes.data_as(A.DP))
            self._keep += [se, sw, sd]
            jd.spectrum = C.pointer(sd)
        if heel is not None:
            hw = np.ascontiguousarray(heel.weights, np.float64)
            hd = A.HeelDesc(heel.energy_start, heel.energy_step, heel.energy_size, heel.angle_size,
                            heel.angle_start, heel.angle_step, hw.ctypes.data_as(A.DP))
            self._keep += [hw, hd]
            jd.heel = C.pointer(hd)
        if bowtie is not None:
            ba = np.ascontiguousarray(bowtie[0], np.float64)
            bw = np.ascontiguousarray(bowtie[1], np.float64)
            bd = A.BowtieDesc(len(ba), ba.ctypes.data_as(A.DP), bw.ctypes.data_as(A.DP))
            self._keep += [ba, bw, bd]
            jd.bowtie = C.pointer(bd)
        jd.seed = int(seed)
        jd.model = int(model)
        jd.tally_mode = int(tally_mode)
        for k, v in (launch or {}).items():
            if k not in self.LAUNCH_KEYS:
                raise ValueError(f"unknown launch parameter {k}")
            setattr(jd, k, int(v))
        self._keep.append(jd)
        return jd

    def wait(self, timeout_ms: int = -1) -> int:
        return self.ctx.lib.dxmc_gpu_job_wait(self.handle, timeout_ms)

    def cancel(self):
        A.check(self.ctx.lib.dxmc_gpu_job_cancel(self.handle), self.ctx.handle, "dxmc_gpu_job_cancel")

    def result(self, output_mode: int = A.OUTPUT_EV_PER_HISTORY, calibration: float = 1.0, want_events: bool = True,
               check: bool = True, out=None):
        """Post-processes on the device and copies to host arrays; ``out`` may supply
        (dose, variance, nEvents) buffers (e.g. pinned) to write into."""
        n = self.dworld.world.size()
        if out is not None:
            dose, var, nev = out
        else:
            dose = np.zeros(n)
            var = np.zeros(n)
            nev = np.zeros(n, np.uint32) if want_events else None
        st = A.JobStats()
        rc = self.ctx.lib.dxmc_gpu_job_result(self.handle, output_mode, calibration, dose.ctypes.data_as(A.DP),
                                              var.ctypes.data_as(A.DP),
                                              nev.ctypes.data_as(A.U32P) if nev is not None else None, C.byref(st))
        stats = dict(histories=st.histories, steps=st.steps, deposits=st.deposits,
                     rejection_overflows=st.rejection_overflows, kernel_ms=st.kernel_ms, job_ms=st.job_ms, status=rc)
        if check and rc not in (A.DXMC_OK,):
            A.check(rc, self.ctx.handle, "dxmc_gpu_job_result")
        return dose, var, nev, stats

    def result_async(self, output_mode: int = A.OUTPUT_EV_PER_HISTORY, calibration: float = 1.0, out=None,
                     dtype=np.float64, want_events: bool = True):
        """Queues the post-processing and the copies of the results behind the job
        and returns at once (dxmc_gpu_job_result_async); ``result_wait`` finishes it.
        ``out`` may supply (dose, variance, nEvents) buffers of ``dtype`` (float64:
        Result<double>, float32: Result<float>), page-locked for overlapped copies;
        they must stay alive until ``result_wait`` returns."""
        n = self.dworld.world.size()
        dtype = np.dtype(dtype)
        if out is not None:
            dose, var, nev = out
        else:
            dose, var = np.zeros(n, dtype), np.zeros(n, dtype)
            nev = np.zeros(n, np.uint32) if want_events else None
        for a in (dose, var):
            if a is not None and (a.dtype != dtype or a.size != n or not a.flags.c_contiguous):
                raise ValueError(f"result buffers must be contiguous {dtype} arrays of {n} elements")
        rtype = A.RESULT_F32 if dtype == np.float32 else A.RESULT_F64
        A.check(self.ctx.lib.dxmc_gpu_job_result_async(self.handle, output_mode, calibration, rtype,
                                                       dose.ctypes.data_as(A.VP) if dose is not None else None,
                                                       var.ctypes.data_as(A.VP) if var is not None else None,
                                                       nev.ctypes.data_as(A.U32P) if nev is not None else None),
                self.ctx.handle, "dxmc_gpu_job_result_async")
        self._async_out = (dose, var, nev)
        return self._async_out

    def result_wait(self, check: bool = True) -> tuple:
        """Waits for the asynchronous result; returns (dose, variance, nEvents, stats)."""
        st = A.JobStats()
        rc = self.ctx.lib.dxmc_gpu_job_result_wait(self.handle, C.byref(st))
        stats = dict(histories=st.histories, steps=st.steps, deposits=st.deposits,
                     rejection_overflows=st.rejection_overflows, kernel_ms=st.kernel_ms, job_ms=st.job_ms, status=rc)
        if check and rc != A.DXMC_OK:
            A.check(rc, self.ctx.handle, "dxmc_gpu_job_result_wait")
        out, self._async_out = self._async_out, None
        return (*out, stats)

    def progress(self) -> tuple:
        """(histories started, total) of a running job."""
        a, b = C.c_uint64(), C.c_uint64()
        A.check(self.ctx.lib.dxmc_gpu_job_progress(self.handle, C.byref(a), C.byref(b)), self.ctx.handle,
                "dxmc_gpu_job_progress")
        return a.value, b.value

    def preview(self, out: Optional[np.ndarray] = None) -> np.ndarray:
        """Energy imparted scored so far (keV per voxel) while the job runs."""
        n = self.dworld.world.size()
        out = np.zeros(n) if out is None else out
        A.check(self.ctx.lib.dxmc_gpu_job_preview(self.handle, out.ctypes.data_as(A.DP)), self.ctx.handle,
                "dxmc_gpu_job_preview")
        return out

    def release(self):
        """Frees the device buffers of a finished job (its results are gone)."""
        if self.handle and self.ctx.handle:
            A.check(self.ctx.lib.dxmc_gpu_job_release(self.handle), self.ctx.handle, "dxmc_gpu_job_release")

    def close(self):
        if self.handle and self._owned and self.ctx.handle:
            self.ctx.lib.dxmc_gpu_job_free(self.handle)
        self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class BatchEntry:
    """One job of a Batch: the arguments of Job without the context."""

    def __init__(self, dworld: DeviceWorld, dlut: DeviceLut, exposures: ExposureTable, spectrum: Optional[Spectrum] = None,
                 heel: Optional[HeelTable] = None, bowtie=None, seed: int = 1, model: int = LOWENERGYCORRECTION.LIVERMORE,
                 tally_mode: int = -1, launch: Optional[dict] = None):
        self.dworld, self.dlut = dworld, dlut
        self.args = (exposures, spectrum, heel, bowtie, seed, model, tally_mode, launch)


class Batch:
    """Many jobs in one persistent launch (dxmc_gpu_batch_*); ``jobs[i]`` gives entry i's results."""

    CONCURRENT = A.BATCH_CONCURRENT
    PERSISTENT = A.BATCH_PERSISTENT

    def __init__(self, ctx: GpuContext, entries: Sequence[BatchEntry], mode: int = A.BATCH_AUTO, chains: int = 0,
                 regen_threshold: int = 0, interact_threshold: int = 0, item_histories: int = 0):
        self.ctx = ctx
        self._entries = list(entries)  # worlds and LUTs stay referenced while the batch runs
        self._descs = []
        arr = (A.BatchEntry * len(entries))()
        for i, e in enumerate(entries):
            holder = Job._member(ctx, e.dworld, C.c_void_p())
            jd = holder._describe(*e.args)
            self._descs.append(holder)
            arr[i].world = e.dworld.handle
            arr[i].lut = e.dlut.handle
            arr[i].job = C.pointer(jd)
        self.handle = C.c_void_p()
        opts = A.BatchOptions(int(mode), int(chains), int(regen_threshold), int(interact_threshold), int(item_histories), 0)
        A.check(ctx.lib.dxmc_gpu_batch_submit(ctx.handle, arr, len(entries), C.byref(opts), C.byref(self.handle)),
                ctx.handle, "dxmc_gpu_batch_submit")
        ctx._register(self)
        self.jobs = []
        for i, e in enumerate(entries):
            h = C.c_void_p()
            A.check(ctx.lib.dxmc_gpu_batch_job(self.handle, i, C.byref(h)), ctx.handle, "dxmc_gpu_batch_job")
            self.jobs.append(Job._member(ctx, e.dworld, h))

    def wait(self, timeout_ms: int = -1) -> int:
        return self.ctx.lib.dxmc_gpu_batch_wait(self.handle, timeout_ms)

    def kernel_ms(self) -> float:
        return self.ctx.lib.dxmc_gpu_batch_kernel_ms(self.handle)

    def close(self):
        if self.handle:
            for j in self.jobs:
                j.handle = C.c_void_p()
            if self.ctx.handle:
                self.ctx.lib.dxmc_gpu_batch_free(self.handle)
        self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


BEAM_SEED_STRIDE = 0x9E3779B97F4A7C15


def beam_seed(seed: int, k: int) -> int:
    """Seed of beam k of a source: beam 0 keeps the caller's seed, the others get
    streams of their own (the per-history streams mix the seed before the history)."""
    return (int(seed) + k * BEAM_SEED_STRIDE) & 0xFFFFFFFFFFFFFFFF


def normalize_scoring(energy: np.ndarray, energy2: np.ndarray, histories: int):
    """Transport::normalizeScoring (transport.hpp:780-794) of raw tallies: eV per
    history and the variance of that mean."""
    d = energy * (1e3 / histories)
    v = (energy2 * (1e6 / histories) - d * d) * (1.0 / (histories - 1))
    return d, v


def energy_imparted_to_dose(world: World, energy: np.ndarray, energy2: np.ndarray, calibration: float = 1.0):
    """Transport::energyImpartedToDose (transport.hpp:796-816) of raw tallies:
    keV/kg times the calibration value, the variance field scaled by its square."""
    sp = world.spacing()
    voxel_volume = sp[0] * sp[1] * sp[2] / 1000.0  # cm3
    density = np.asarray(world.densityArray(), np.float64)
    mass = density * voxel_volume * 0.001  # kg
    with np.errstate(divide="ignore", invalid="ignore"):
        factor = np.where(density > 0.0, calibration / mass, 0.0)
    return np.where(density > 0.0, energy * factor, 0.0), np.where(density > 0.0, energy2 * factor * factor, 0.0)


class Transport:
    """GPU drop-in for dxmc::Transport<T> (transport.hpp:114-840)."""

    EV_PER_HISTORY = 0
    DOSE = 1

    def __init__(self, context: Optional[GpuContext] = None):
        self._model = LOWENERGYCORRECTION.LIVERMORE  # transport.hpp:839
        self._mode = Transport.DOSE                  # transport.hpp:838
        self._ctx = context or GpuContext()
        self._seed = 0x5EED
        self._tally_mode = -1

    def setLowEnergyCorrectionModel(self, m: int):
        self._model = int(m)

    def lowEnergyCorrectionModel(self) -> int:
        return self._model

    def setOutputMode(self, m: int):
        self._mode = int(m)

    def outputMode(self) -> int:
        return self._mode

    def setNumberOfWorkers(self, n: int):
        pass  # the GPU launch replaces the worker threads (transport.hpp:128)

    def setSeed(self, seed: int):
        self._seed = int(seed)

    def setTallyMode(self, mode: int):
        self._tally_mode = int(mode)

    def context(self) -> GpuContext:
        return self._ctx

    def __call__(self, world: World, source: Source, progressbar=None, useSourceDoseCalibration: bool = True) -> Result:
        n = world.size()
        empty = Result(np.zeros(n), np.zeros(n, np.uint32), np.zeros(n))
        if not world.isValid() or source is None:
            return empty
        source.updateFromWorld(world)
        source.validate()
        if not source.isValid():
            return empty
        beams = source.beams(world.directionCosines())
        histories = int(sum(int(np.sum(b.exposures.n_histories)) for b in beams))
        dworld = DeviceWorld(self._ctx, world)
        blob = LutBlob.cached(world.materialMap(), dworld.max_density(), source.maxPhotonEnergyProduced())
        dlut = DeviceLut(self._ctx, blob)
        t0 = time.perf_counter()
        # one job per beam (dual-source CT: one per tube), each on streams of its own
        jobs = [Job(self._ctx, dworld, dlut, b.exposures, b.spectrum, b.heel, b.bowtie, beam_seed(self._seed, k),
                    self._model, self._tally_mode) for k, b in enumerate(beams)]
        for job in jobs:
            job.wait()
        sim_time = time.perf_counter() - t0
        cal = 1.0
        if self._mode == Transport.DOSE:
            cal = source.getCalibrationValue(self._model, transport=self) if useSourceDoseCalibration else 1.0
            units = "mGy" if useSourceDoseCalibration else "keV/kg"
        else:
            units = "eV/history"
        if len(jobs) == 1:
            if self._mode == Transport.DOSE:
                dose, var, nev, stats = jobs[0].result(A.OUTPUT_DOSE, cal)
            else:
                dose, var, nev, stats = jobs[0].result(A.OUTPUT_EV_PER_HISTORY)
        else:
            # the beams' raw tallies add; then the reference's normalisation over all histories
            e = e2 = nev = None
            stats = {}
            for job in jobs:
                d, v, c, st = job.result(A.OUTPUT_RAW)
                e = d if e is None else e + d
                e2 = v if e2 is None else e2 + v
                nev = c if nev is None else nev + c
                for key, val in st.items():
                    stats[key] = stats.get(key, 0) + val if key in ("histories", "steps", "deposits",
                                                                      "rejection_overflows") else max(stats.get(key, 0), val)
            if self._mode == Transport.DOSE:
                dose, var = energy_imparted_to_dose(world, e, e2, cal)
            else:
                dose, var = normalize_scoring(e, e2, histories)
        for job in jobs:
            job.close()
        dlut.close()
        dworld.close()
        return Result(dose, nev, var, histories, sim_time, units, stats)
