"""X-ray tube spectrum and heel table (host side).

Spectrum generation stays on the host, as in DXMClib (tube.hpp:35-299,
beamfilters.hpp:435-569).  The spectrum is DXMClib's model, computed by the
library's host code (dxmc_tube_spectrum, csrc/host/tube_spectrum.cpp):
thick-target semi-relativistic Bethe-Heitler bremsstrahlung integrated over the
tabulated electron fluence in tungsten of Poludniowski and Evans (2007), with
self-absorption in the anode along the take-off direction, the tungsten K lines,
and added filtration exp(-mu/rho * rho * t) per filter material.

The interface mirrors Tube<T> (voltage, anode angle, energy resolution,
filtration setters, getEnergy, getSpecter) and HeelFilter<T> (energy grid
from 10 keV in 2 keV steps, 5 angle bins across the heel span).
"""
from __future__ import annotations

import collections
import math
import threading
from typing import List, Tuple

import numpy as np

DEG = math.pi / 180.0

_SPECTRUM_CACHE: "collections.OrderedDict" = collections.OrderedDict()
_SPECTRUM_CACHE_ENTRIES = 4096
_SPECTRUM_LOCK = threading.Lock()


class Tube:
    def __init__(self, voltage: float = 120.0, anode_angle_deg: float = 12.0, energy_resolution: float = 1.0):
        self._voltage = voltage
        self._anode = anode_angle_deg * DEG
        self._res = energy_resolution
        self._filters: List[Tuple[object, float]] = []

    @staticmethod
    def maxVoltage():
        return 150.0

    @staticmethod
    def minVoltage():
        return 50.0

    def voltage(self):
        return self._voltage

    def setVoltage(self, v: float):
        self._voltage = min(max(float(v), self.minVoltage()), self.maxVoltage())

    def anodeAngle(self):
        return self._anode

    def setAnodeAngleDeg(self, a: float):
        self.setAnodeAngle(a * DEG)

    def setAnodeAngle(self, a: float):
        self._anode = min(abs(a), math.pi / 2)

    def setEnergyResolution(self, r: float):
        self._res = float(r)

    def energyResolution(self):
        return self._res

    def _set_filter(self, symbol: str, mm: float):
        from .api import Material
        for i, (m, t) in enumerate(self._filters):
            if m.name() == symbol:
                self._filters[i] = (m, abs(mm))
                return
        self._filters.append((Material(symbol), abs(mm)))

    def setAlFiltration(self, mm: float):
        self._set_filter("Al", mm)

    def setCuFiltration(self, mm: float):
        self._set_filter("Cu", mm)

    def setSnFiltration(self, mm: float):
        self._set_filter("Sn", mm)

    def addFiltrationMaterial(self, material, mm: float):
        self._filters.append((material, abs(mm)))

    def filtration(self, symbol: str) -> float:
        for m, t in self._filters:
            if m.name() == symbol:
                return t
        return 0.0

    def AlFiltration(self) -> float:
        return self.filtration("Al")

    def CuFiltration(self) -> float:
        return self.filtration("Cu")

    def SnFiltration(self) -> float:
        return self.filtration("Sn")

    def getEnergy(self) -> np.ndarray:
        """tube.hpp:165-176: res, 2 res, ... <= voltage."""
        out = []
        hv = self._res
        while hv <= self._voltage:
            out.append(hv)
            hv = hv + self._res
        return np.asarray(out, np.float64)

    def _state(self):
        return (self._voltage, self._anode, self._res, tuple((m.name(), m.standardDensity(), t) for m, t in self._filters))

    def getSpecter(self, energies=None, anode_angle=None, normalize: bool = True) -> np.ndarray:
        e = self.getEnergy() if energies is None else np.asarray(energies, np.float64)
        a = self._anode if anode_angle is None else anode_angle
        # spectra are deterministic in the tube settings: memoised across every Tube
        # (sources built per request repeat a few settings)
        key = (self._state(), e.tobytes(), float(a), bool(normalize))
        with _SPECTRUM_LOCK:
            hit = _SPECTRUM_CACHE.get(key)
            if hit is not None:
                _SPECTRUM_CACHE.move_to_end(key)
                return hit.copy()
        spec = self._compute_specter(e, a, normalize)
        with _SPECTRUM_LOCK:
            _SPECTRUM_CACHE[key] = spec.copy()
            while len(_SPECTRUM_CACHE) > _SPECTRUM_CACHE_ENTRIES:
                _SPECTRUM_CACHE.popitem(last=False)
        return spec

    def _compute_specter(self, e: np.ndarray, a: float, normalize: bool) -> np.ndarray:
        """Tube<T>::getSpecter(energies, anodeAngle, normalize) (tube.hpp:195-213): the
        bremsstrahlung at take-off angle ``a``, the K lines at the tube's anode angle."""
        from . import _capi as A
        lib = A.load()
        e = np.ascontiguousarray(e, np.float64)
        out = np.zeros(len(e))
        filt = (A.MaterialProvider * max(len(self._filters), 1))()
        for i, (m, _) in enumerate(self._filters):
            filt[i] = m.provider
        mm = np.array([t for _, t in self._filters] or [0.0], np.float64)
        A.check(lib.dxmc_tube_spectrum(float(self._voltage), float(a), float(self._anode), e.ctypes.data_as(A.DP), len(e),
                                       filt, mm.ctypes.data_as(A.DP), len(self._filters), 1 if normalize else 0,
                                       out.ctypes.data_as(A.DP)), None, "dxmc_tube_spectrum")
        return out


class HeelFilter:
    """Heel-effect weight table in the layout of HeelFilter<T> (beamfilters.hpp:455-505)."""

    def __init__(self, tube: Tube, heel_angle_span: float = 0.0):
        self.energy_step = 2.0
        self.energy_start = 10.0
        self.angle_size = 5
        self.energy_size = max(int((tube.voltage() - self.energy_start) / self.energy_step), 2)
        energies = self.energy_start + self.energy_step * np.arange(self.energy_size)
        span = abs(heel_angle_span)
        if tube.anodeAngle() < span / 2:
            self.angle_start = -tube.anodeAngle()
        else:
            self.angle_start = -span / 2
        self.angle_step = (span / 2 - self.angle_start) / self.angle_size
        w = np.zeros((self.energy_size, self.angle_size))
        for i in range(self.angle_size):
            angle = self.angle_start + i * self.angle_step + tube.anodeAngle()
            w[:, i] = tube.getSpecter(energies, angle, normalize=False)
        mean = w.mean(axis=1, keepdims=True)
        with np.errstate(invalid="ignore", divide="ignore"):
            w = np.where(mean > 0, w / np.where(mean > 0, mean, 1), 1.0)
        self.weights = w.ravel()

    def table(self):
        from .api import HeelTable
        return HeelTable(self.energy_start, self.energy_step, self.energy_size, self.angle_start, self.angle_step,
                         self.angle_size, self.weights.copy())
