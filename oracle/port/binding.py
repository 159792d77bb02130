"""ctypes binding to oracle/port/liboracle_port.so (CPU restatement of the
reference transport).  ORACLE TEST INFRASTRUCTURE: imported only by tests/,
__graft_entry__.smoke and bench.py's CPU-baseline / reference legs."""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle_port.so"
SRC = HERE / "dxmc_port.cpp"
CORE = HERE / "port_core.inc"

DP = C.POINTER(C.c_double)


class PortLut(C.Structure):
    _fields_ = [("n_materials", C.c_int), ("n_energy", C.c_int), ("linear_index", C.c_int), ("pad", C.c_int),
                ("linear_step", C.c_double), ("linear_energy", C.c_double), ("log_energy", DP),
                ("coefficients", DP), ("max_coefficients", DP), ("rita", DP), ("spline", DP), ("shells", DP)]


class PortWorld(C.Structure):
    _fields_ = [("dims", C.c_uint64 * 3), ("spacing", C.c_double * 3), ("origin", C.c_double * 3),
                ("density", DP), ("material", C.POINTER(C.c_uint8)), ("measurement", C.POINTER(C.c_uint8))]


class PortSource(C.Structure):
    _fields_ = [("exposures", DP), ("n_exposures", C.c_uint64), ("spec_n", C.c_int), ("spec_energies", DP),
                ("spec_weights", DP), ("heel_ne", C.c_int), ("heel_na", C.c_int), ("heel_e0", C.c_double),
                ("heel_es", C.c_double), ("heel_a0", C.c_double), ("heel_as", C.c_double), ("heel_weights", DP),
                ("bowtie_n", C.c_int), ("bowtie_angles", DP), ("bowtie_weights", DP)]


def build(force: bool = False) -> Path:
    if force or not LIB.exists() or LIB.stat().st_mtime < max(SRC.stat().st_mtime, CORE.stat().st_mtime):
        r = subprocess.run(["g++", "-std=c++20", "-O3", "-fPIC", "-shared", "-pthread", "-o", str(LIB), str(SRC)],
                           capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("oracle port build failed:\n" + r.stderr)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(str(LIB))
        _lib.oracle_port_set_direction.argtypes = [C.c_int]
        _lib.oracle_port_set_direction.restype = None
        _lib.oracle_port_transport_ex.restype = C.c_double
        _lib.oracle_port_transport_ex.argtypes = [C.POINTER(PortLut), C.POINTER(PortWorld), C.POINTER(PortSource),
                                                  C.c_int, C.c_int, C.c_uint64, C.c_int, DP, DP, C.POINTER(C.c_uint32),
                                                  C.POINTER(C.c_uint64)]
    return _lib


def _d(a):
    return a.ctypes.data_as(DP)


def lut_from_fixture(g: dict, prefix: str = "lut_") -> dict:
    """LUT tables in the form transport() takes, from a golden fixture that stores
    the reference's own AttenuationLut<double> tables (tests/golden/make_golden.py):
    the port then runs without the product library."""
    meta = g[prefix + "meta"]
    return dict(x=g[prefix + "x"], coef=g[prefix + "coef"], maxcoef=g[prefix + "maxcoef"], rita=g[prefix + "rita"],
                spline=g[prefix + "spline"], shells=g[prefix + "shells"], n_energy=int(meta[0]),
                linear_index=int(meta[1]), linear_step=float(meta[2]), linear_energy=float(meta[3]),
                min_energy=float(meta[4]), max_energy=float(meta[5]))


def transport(lut_info: dict, dims, spacing, density, material, exposures19, model: int = 1, n_threads: int = 0,
              seed: int = 1, spectrum=None, heel=None, bowtie=None, measurement=None, origin=(0, 0, 0),
              normalized_direction: bool = False, precision: str = "double"):
    """Runs the CPU restatement; returns (energy, energy^2, nEvents, seconds, steps) raw tallies.
    normalized_direction selects the normalised physics mode (unit scattering axis);
    precision "double" or "float" (Transport<double> / Transport<float>)."""
    keep = []
    L = PortLut()
    x = np.ascontiguousarray(lut_info["x"], np.float64)
    coef = np.ascontiguousarray(lut_info["coef"], np.float64)
    mcoef = np.ascontiguousarray(lut_info["maxcoef"], np.float64)
    rita = np.ascontiguousarray(lut_info["rita"], np.float64)
    spl = np.ascontiguousarray(lut_info["spline"], np.float64)
    sh = np.ascontiguousarray(lut_info["shells"], np.float64)
    keep += [x, coef, mcoef, rita, spl, sh]
    L.n_materials = rita.shape[0]
    L.n_energy = len(x)
    L.linear_index = int(lut_info["linear_index"])
    L.linear_step = float(lut_info["linear_step"])
    L.linear_energy = float(lut_info["linear_energy"])
    L.log_energy, L.coefficients, L.max_coefficients, L.rita, L.spline, L.shells = map(_d, (x, coef, mcoef, rita, spl, sh))
    W = PortWorld()
    W.dims[:] = list(dims)
    W.spacing[:] = list(spacing)
    W.origin[:] = list(origin)
    dens = np.ascontiguousarray(density, np.float64).ravel()
    mat = np.ascontiguousarray(material, np.uint8).ravel()
    keep += [dens, mat]
    W.density = _d(dens)
    W.material = mat.ctypes.data_as(C.POINTER(C.c_uint8))
    if measurement is not None:
        meas = np.ascontiguousarray(measurement, np.uint8).ravel()
        keep.append(meas)
        W.measurement = meas.ctypes.data_as(C.POINTER(C.c_uint8))
    S = PortSource()
    ex = np.ascontiguousarray(exposures19, np.float64)
    keep.append(ex)
    S.exposures = _d(ex)
    S.n_exposures = len(ex)
    if spectrum is not None:
        se = np.ascontiguousarray(spectrum[0], np.float64)
        sw = np.ascontiguousarray(spectrum[1], np.float64)
        keep += [se, sw]
        S.spec_n, S.spec_energies, S.spec_weights = len(se), _d(se), _d(sw)
    if heel is not None:
        hw = np.ascontiguousarray(heel["weights"], np.float64)
        keep.append(hw)
        S.heel_ne, S.heel_na = int(heel["energy_size"]), int(heel["angle_size"])
        S.heel_e0, S.heel_es = float(heel["energy_start"]), float(heel["energy_step"])
        S.heel_a0, S.heel_as = float(heel["angle_start"]), float(heel["angle_step"])
        S.heel_weights = _d(hw)
    if bowtie is not None:
        ba = np.ascontiguousarray(bowtie[0], np.float64)
        bw = np.ascontiguousarray(bowtie[1], np.float64)
        keep += [ba, bw]
        S.bowtie_n, S.bowtie_angles, S.bowtie_weights = len(ba), _d(ba), _d(bw)
    n = int(np.prod(dims))
    e = np.zeros(n)
    e2 = np.zeros(n)
    nev = np.zeros(n, np.uint32)
    steps = C.c_uint64(0)
    lib().oracle_port_set_direction(1 if normalized_direction else 0)
    prec = {"double": 0, "float": 1}[precision]
    secs = lib().oracle_port_transport_ex(C.byref(L), C.byref(W), C.byref(S), int(model), int(n_threads), int(seed),
                                          prec, _d(e), _d(e2), nev.ctypes.data_as(C.POINTER(C.c_uint32)),
                                          C.byref(steps))
    return e, e2, nev, secs, steps.value


def ev_per_history(e, e2, histories):
    """normalizeScoring (transport.hpp:780-794)."""
    d = e * 1e3 / histories
    v = (e2 * 1e6 / histories - d * d) / (histories - 1)
    return d, v
