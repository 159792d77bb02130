"""X-ray tube spectrum and heel table (host side).

Spectrum generation stays on the host, as in DXMClib (tube.hpp:35-299,
beamfilters.hpp:435-569).  The project's own tube model is a thick-target
Kramers spectrum with depth-resolved anode self-absorption:

* electrons slow down in tungsten along the Thomson-Whiddington law
  T(x)^2 = T0^2 - C x, with C = T0^2 / R(T0) and R the Kanaya-Okayama range;
* at each depth the Kramers thin-target yield is 1/hv per unit electron
  energy loss for hv < T;
* photons emitted at mass depth x leave the anode through x / sin(angle) of
  tungsten (attenuation from the project physics model);
* tungsten K-lines (energies from the project shell model) are added with a
  yield proportional to ((T0 - E_K) / E_K)^1.63 (Green-Cosslett);
* added filtration is exp(-mu/rho * rho * t) per filter material.

The interface mirrors Tube<T> (voltage, anode angle, energy resolution,
filtration setters, getEnergy, getSpecter) and HeelFilter<T> (energy grid
from 10 keV in 2 keV steps, 5 angle bins across the heel span).
"""
from __future__ import annotations

import math
from typing import List, Tuple

import numpy as np

DEG = math.pi / 180.0


class Tube:
    def __init__(self, voltage: float = 120.0, anode_angle_deg: float = 12.0, energy_resolution: float = 1.0):
        self._voltage = voltage
        self._anode = anode_angle_deg * DEG
        self._res = energy_resolution
        self._filters: List[Tuple[object, float]] = []
        self._w_cache = {}

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

    def getEnergy(self) -> np.ndarray:
        """tube.hpp:165-176: res, 2 res, ... <= voltage."""
        out = []
        hv = self._res
        while hv <= self._voltage:
            out.append(hv)
            hv = hv + self._res
        return np.asarray(out, np.float64)

    def _tungsten(self):
        if "W" not in self._w_cache:
            from .api import Material
            self._w_cache["W"] = Material("W")
        return self._w_cache["W"]

    def _kramers_self_absorbed(self, energies: np.ndarray, anode_angle: float) -> np.ndarray:
        T0 = self._voltage
        W = self._tungsten()
        rho = 19.3
        # Kanaya-Okayama range (um -> cm) and Whiddington constant
        R_cm = 0.0276 * 183.84 * T0 ** 1.67 / (74 ** 0.889 * rho) * 1e-4
        Cw = T0 ** 2 / (rho * R_cm)  # keV^2 per g/cm2
        sin_a = max(math.sin(anode_angle), 1e-6)
        nT = 200
        out = np.zeros(len(energies))
        for i, hv in enumerate(energies):
            if hv <= 0 or hv >= T0:
                continue
            mu = W.getTotalAttenuation(float(hv))
            T = np.linspace(hv, T0, nT)
            x = (T0 ** 2 - T ** 2) / Cw  # g/cm2 depth where the electron has energy T
            f = np.exp(-mu * x / sin_a) / hv
            out[i] = np.trapezoid(f, T) if hasattr(np, "trapezoid") else np.trapz(f, T)
        return out

    def _characteristic(self, energies: np.ndarray, anode_angle: float, spec: np.ndarray) -> np.ndarray:
        """Tungsten K lines added to the nearest energy bin within 2 keV."""
        T0 = self._voltage
        import ctypes as C
        from . import _capi as A
        W = self._tungsten()
        shells = (A.ShellConfig * 12)()
        W.provider.shells(W.provider.user, shells)
        k = shells[0]
        EK = k.binding_energy
        if T0 <= EK:
            return spec
        sin_a = max(math.sin(anode_angle), 1e-6)
        yield_k = ((T0 - EK) / EK) ** 1.63
        # normalise against the bremsstrahlung just above the edge energy scale
        brem_ref = np.interp(EK * 0.8, energies, spec) if len(energies) > 1 else 0.0
        total = 0.15 * yield_k * brem_ref * len(energies) / 12.0
        out = spec.copy()
        for line in range(3):
            e = k.line_energies[line]
            p = k.line_probabilities[line]
            if e <= 0 or p <= 0:
                continue
            idx = np.searchsorted(energies, e)
            if idx < len(energies) and abs(energies[idx] - e) <= 2.0:
                mu = W.getTotalAttenuation(float(e))
                out[idx] += total * p * math.exp(-mu * 19.3 * 3e-4 / sin_a)
        return out

    def _state(self):
        return (self._voltage, self._anode, self._res, tuple((m.name(), m.standardDensity(), t) for m, t in self._filters))

    def getSpecter(self, energies=None, anode_angle=None, normalize: bool = True) -> np.ndarray:
        e = self.getEnergy() if energies is None else np.asarray(energies, np.float64)
        a = self._anode if anode_angle is None else anode_angle
        # spectra are deterministic in the tube settings: memoise them
        key = (self._state(), e.tobytes(), float(a), bool(normalize))
        cache = self._w_cache.setdefault("spectra", {})
        hit = cache.get(key)
        if hit is not None:
            return hit.copy()
        spec = self._compute_specter(e, a, normalize)
        cache[key] = spec.copy()
        return spec

    def _compute_specter(self, e: np.ndarray, a: float, normalize: bool) -> np.ndarray:
        spec = self._kramers_self_absorbed(e, a)
        spec = self._characteristic(e, a, spec)
        for m, mm in self._filters:
            cm = mm * 0.1
            mu = np.array([m.getTotalAttenuation(float(x)) for x in e])
            spec = spec * np.exp(-mu * m.standardDensity() * cm)
        if normalize and spec.sum() > 0:
            spec = spec / spec.sum()
        return spec


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
