"""ctypes binding to oracle/_ref/libdxmc_ref.so (the reference DXMClib headers
compiled unmodified with the project Material backend).

Oracle test infrastructure: used only by the golden-fixture generator and by
tests that run where the reference library was built.  Structures mirror
oracle/ref_api.cpp.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parents[2]
LIB_PATH = REPO / "oracle" / "_ref" / "libdxmc_ref.so"

PENCIL, ISOTROPIC, DX, CTSPIRAL, CTAXIAL, CBCT, ISOTROPIC_CT = range(7)


class RefWorldDesc(C.Structure):
    _fields_ = [
        ("dims", C.c_uint64 * 3),
        ("spacing", C.c_double * 3),
        ("origin", C.c_double * 3),
        ("direction_cosines", C.c_double * 6),
        ("density", C.POINTER(C.c_double)),
        ("material", C.POINTER(C.c_uint8)),
        ("measurement", C.POINTER(C.c_uint8)),
        ("n_materials", C.c_int),
        ("material_names", C.POINTER(C.c_char_p)),
        ("material_densities", C.POINTER(C.c_double)),
    ]


class RefSourceDesc(C.Structure):
    _fields_ = [
        ("type", C.c_int),
        ("heel", C.c_int),
        ("position", C.c_double * 3),
        ("direction_cosines", C.c_double * 6),
        ("histories_per_exposure", C.c_uint64),
        ("total_exposures", C.c_uint64),
        ("energy", C.c_double),
        ("collimation", C.c_double * 4),
        ("spec_energies", C.POINTER(C.c_double)),
        ("spec_weights", C.POINTER(C.c_double)),
        ("spec_n", C.c_int),
        ("kvp", C.c_double),
        ("anode_angle_deg", C.c_double),
        ("al_mm", C.c_double),
        ("cu_mm", C.c_double),
        ("field_size", C.c_double * 2),
        ("sdd", C.c_double),
        ("source_angles_deg", C.c_double * 2),
        ("tube_rotation_deg", C.c_double),
        ("span_deg", C.c_double),
        ("step_deg", C.c_double),
        ("ct_collimation", C.c_double),
        ("pitch", C.c_double),
        ("scan_length", C.c_double),
        ("angle_step_deg", C.c_double),
        ("start_angle_deg", C.c_double),
        ("fov", C.c_double),
        ("tilt_deg", C.c_double),
        ("bowtie_angles", C.POINTER(C.c_double)),
        ("bowtie_weights", C.POINTER(C.c_double)),
        ("bowtie_n", C.c_int),
        ("axial_step", C.c_double),
        ("set_b", C.c_int),
        ("kvp_b", C.c_double),
        ("al_mm_b", C.c_double),
        ("cu_mm_b", C.c_double),
        ("mas_a", C.c_double),
        ("mas_b", C.c_double),
        ("sdd_b", C.c_double),
        ("fov_b", C.c_double),
        ("start_angle_b_deg", C.c_double),
    ]


def available() -> bool:
    return LIB_PATH.exists()


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(str(LIB_PATH))
    return _lib


def _dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class WorldArgs:
    """Keeps the numpy buffers alive while the descriptor is in use."""

    def __init__(self, dims, spacing, density, material, material_names, material_densities=None,
                 measurement=None, origin=(0, 0, 0), cosines=(1, 0, 0, 0, 1, 0)):
        self.density = np.ascontiguousarray(density, dtype=np.float64).ravel()
        self.material = np.ascontiguousarray(material, dtype=np.uint8).ravel()
        self.measurement = None if measurement is None else np.ascontiguousarray(measurement, dtype=np.uint8).ravel()
        self.names = (C.c_char_p * len(material_names))(*[n.encode() for n in material_names])
        md = material_densities if material_densities is not None else [-1.0] * len(material_names)
        self.mdens = np.asarray(md, dtype=np.float64)
        d = RefWorldDesc()
        d.dims[:] = list(dims)
        d.spacing[:] = list(spacing)
        d.origin[:] = list(origin)
        d.direction_cosines[:] = list(cosines)
        d.density = _dptr(self.density)
        d.material = self.material.ctypes.data_as(C.POINTER(C.c_uint8))
        d.measurement = None if self.measurement is None else self.measurement.ctypes.data_as(C.POINTER(C.c_uint8))
        d.n_materials = len(material_names)
        d.material_names = self.names
        d.material_densities = _dptr(self.mdens)
        self.desc = d
        self.size = int(np.prod(dims))


class SourceArgs:
    def __init__(self, type, **kw):
        s = RefSourceDesc()
        s.type = type
        s.heel = int(kw.get("heel", 1))
        s.position[:] = list(kw.get("position", (0, 0, 0)))
        s.direction_cosines[:] = list(kw.get("cosines", (1, 0, 0, 0, 1, 0)))
        s.histories_per_exposure = int(kw.get("histories_per_exposure", 1000))
        s.total_exposures = int(kw.get("total_exposures", 1))
        s.energy = float(kw.get("energy", 60.0))
        s.collimation[:] = list(kw.get("collimation", (0, 0, 0, 0)))
        self.spec_e = np.asarray(kw.get("spec_energies", [60.0]), dtype=np.float64)
        self.spec_w = np.asarray(kw.get("spec_weights", [1.0]), dtype=np.float64)
        s.spec_energies = _dptr(self.spec_e)
        s.spec_weights = _dptr(self.spec_w)
        s.spec_n = len(self.spec_e)
        s.kvp = float(kw.get("kvp", 120.0))
        s.anode_angle_deg = float(kw.get("anode_angle_deg", 12.0))
        s.al_mm = float(kw.get("al_mm", 2.0))
        s.cu_mm = float(kw.get("cu_mm", 0.0))
        s.field_size[:] = list(kw.get("field_size", (100.0, 100.0)))
        s.sdd = float(kw.get("sdd", 1000.0))
        s.source_angles_deg[:] = list(kw.get("source_angles_deg", (0.0, 0.0)))
        s.tube_rotation_deg = float(kw.get("tube_rotation_deg", 0.0))
        s.span_deg = float(kw.get("span_deg", 180.0))
        s.step_deg = float(kw.get("step_deg", 1.0))
        s.ct_collimation = float(kw.get("ct_collimation", 38.4))
        s.pitch = float(kw.get("pitch", 1.0))
        s.scan_length = float(kw.get("scan_length", 100.0))
        s.angle_step_deg = float(kw.get("angle_step_deg", 1.0))
        s.start_angle_deg = float(kw.get("start_angle_deg", 0.0))
        s.fov = float(kw.get("fov", 500.0))
        s.tilt_deg = float(kw.get("tilt_deg", 0.0))
        bowtie = kw.get("bowtie")
        if bowtie is not None:
            self.bt_a = np.ascontiguousarray(bowtie[0], np.float64)
            self.bt_w = np.ascontiguousarray(bowtie[1], np.float64)
            s.bowtie_angles = _dptr(self.bt_a)
            s.bowtie_weights = _dptr(self.bt_w)
            s.bowtie_n = len(self.bt_a)
        else:
            s.bowtie_n = 0
        s.axial_step = float(kw.get("axial_step", 0.0))
        s.set_b = int("kvp_b" in kw)
        s.kvp_b = float(kw.get("kvp_b", 120.0))
        s.al_mm_b = float(kw.get("al_mm_b", 7.0))
        s.cu_mm_b = float(kw.get("cu_mm_b", 0.0))
        s.mas_a = float(kw.get("mas_a", 100.0))
        s.mas_b = float(kw.get("mas_b", 100.0))
        s.sdd_b = float(kw.get("sdd_b", 1190.0))
        s.fov_b = float(kw.get("fov_b", 500.0))
        s.start_angle_b_deg = float(kw.get("start_angle_b_deg", 90.0))
        self.desc = s


def bowtie(angles, weights, queries):
    """BowTieFilter<double>(angles, weights): its normalised (angle, weight) table and
    sampleIntensityWeight at the query angles (beamfilters.hpp:102-190)."""
    a = np.ascontiguousarray(angles, np.float64)
    w = np.ascontiguousarray(weights, np.float64)
    q = np.ascontiguousarray(queries, np.float64)
    ta, tw, out = np.zeros(len(a)), np.zeros(len(a)), np.zeros(len(q))
    rc = lib().ref_bowtie(_dptr(a), _dptr(w), C.c_int(len(a)), _dptr(q), C.c_int(len(q)), _dptr(ta), _dptr(tw),
                          _dptr(out))
    if rc != 0:
        raise RuntimeError(f"ref_bowtie failed: {rc}")
    return ta, tw, out


def transport(world: WorldArgs, source: SourceArgs, model: int = 1, n_threads: int = 0):
    n = world.size
    dose = np.zeros(n, np.float64)
    var = np.zeros(n, np.float64)
    nev = np.zeros(n, np.uint32)
    meta = np.zeros(4, np.float64)
    rc = lib().ref_transport(C.byref(world.desc), C.byref(source.desc), C.c_int(model), C.c_int(n_threads),
                             _dptr(dose), _dptr(var), nev.ctypes.data_as(C.POINTER(C.c_uint32)), _dptr(meta))
    if rc != 0:
        raise RuntimeError(f"ref_transport failed: {rc}")
    return dose, var, nev, int(meta[0]), float(meta[1])


def lut_dump(world: WorldArgs, max_energy: float, energies, q):
    energies = np.ascontiguousarray(energies, np.float64)
    q = np.ascontiguousarray(q, np.float64)
    nm = world.desc.n_materials
    ne, nq = len(energies), len(q)
    att = np.zeros(nm * ne * 3)
    maxinv = np.zeros(ne)
    sf = np.zeros(nm * nq)
    shells = np.zeros(nm * 12 * 13)
    rita = np.zeros(nm * 4 * 56)
    spline = np.zeros(nm * 79)
    meta = np.zeros(16)
    cap = 1 << 20
    xs = np.zeros(cap)
    coef = np.zeros(cap)
    mcoef = np.zeros(cap)
    rc = lib().ref_lut_dump(C.byref(world.desc), C.c_double(max_energy), _dptr(energies), C.c_int(ne),
                            _dptr(att), _dptr(maxinv), _dptr(q), C.c_int(nq), _dptr(sf), _dptr(shells),
                            _dptr(rita), _dptr(spline), _dptr(meta), _dptr(xs), _dptr(coef), _dptr(mcoef),
                            C.c_int(cap))
    if rc != 0:
        raise RuntimeError(f"ref_lut_dump failed: {rc}")
    nx, nc, nmc = int(meta[6]), int(meta[7]), int(meta[8])
    return dict(
        att=att.reshape(nm, ne, 3), maxinv=maxinv, sf=sf.reshape(nm, nq), shells=shells.reshape(nm, 12, 13),
        rita=rita.reshape(nm, 4, 56), spline=spline.reshape(nm, 79), meta=meta[:6].copy(),
        x=xs[:nx].copy(), coef=coef[:nc].copy(), maxcoef=mcoef[:nmc].copy())


def source_tables(source: SourceArgs, world: WorldArgs, cap_exposures: int = 200000):
    ex = np.zeros(cap_exposures * 19)
    nexp = C.c_uint64(0)
    cap = 4096
    se, sw, sp = np.zeros(cap), np.zeros(cap), np.zeros(cap)
    sa = np.zeros(cap, np.uint64)
    sn = C.c_int(0)
    hm = np.zeros(8)
    hw = np.zeros(65536)
    maxe = C.c_double(0)
    rc = lib().ref_source_tables(C.byref(source.desc), C.byref(world.desc), _dptr(ex), C.c_uint64(cap_exposures),
                                 C.byref(nexp), _dptr(se), _dptr(sw), _dptr(sp),
                                 sa.ctypes.data_as(C.POINTER(C.c_uint64)), C.byref(sn), C.c_int(cap),
                                 _dptr(hm), _dptr(hw), C.c_int(len(hw)), C.byref(maxe))
    if rc != 0:
        raise RuntimeError(f"ref_source_tables failed: {rc}")
    n = nexp.value
    k = sn.value
    out = dict(exposures=ex[: n * 19].reshape(n, 19).copy(), max_energy=maxe.value,
               spec_energies=se[:k].copy(), spec_weights=sw[:k].copy(), spec_probs=sp[:k].copy(),
               spec_alias=sa[:k].copy(), heel_meta=hm.copy())
    if hm[0] > 0:
        ne, na = int(hm[3]), int(hm[6])
        out["heel_weights"] = hw[: ne * na].copy()
    return out


def exposure_tables(source: SourceArgs, world: WorldArgs, index: int):
    """The spectrum alias table and heel table exposure ``index`` samples with, and
    tube B's energies and normalised weights for dual sources."""
    cap = 4096
    sp = np.zeros(cap)
    sa = np.zeros(cap, np.uint64)
    sn = C.c_int(0)
    hm = np.zeros(8)
    hw = np.zeros(65536)
    be, bw = np.zeros(cap), np.zeros(cap)
    bn = C.c_int(0)
    rc = lib().ref_exposure_tables(C.byref(source.desc), C.byref(world.desc), C.c_uint64(index), _dptr(sp),
                                   sa.ctypes.data_as(C.POINTER(C.c_uint64)), C.byref(sn), C.c_int(cap), _dptr(hm),
                                   _dptr(hw), C.c_int(len(hw)), _dptr(be), _dptr(bw), C.byref(bn))
    if rc != 0:
        raise RuntimeError(f"ref_exposure_tables failed: {rc}")
    k, nb = sn.value, bn.value
    out = dict(spec_probs=sp[:k].copy(), spec_alias=sa[:k].copy(), heel_meta=hm.copy(),
               tube_b_energies=be[:nb].copy(), tube_b_weights=bw[:nb].copy())
    if hm[0] > 0:
        out["heel_weights"] = hw[: int(hm[3]) * int(hm[6])].copy()
    return out


def alias_table(weights):
    w = np.ascontiguousarray(weights, np.float64)
    p = np.zeros(len(w))
    a = np.zeros(len(w), np.uint64)
    lib().ref_alias_table(_dptr(w), C.c_int(len(w)), _dptr(p), a.ctypes.data_as(C.POINTER(C.c_uint64)))
    return p, a


def interactions(world: WorldArgs, max_energy: float, model: int, kind: int, energy: float, n: int,
                 nbins: int = 100, seed: int = 1):
    hc = np.zeros(nbins)
    he = np.zeros(nbins)
    sums = np.zeros(3)
    rc = lib().ref_interactions(C.byref(world.desc), C.c_double(max_energy), C.c_int(model), C.c_int(kind),
                                C.c_double(energy), C.c_uint64(n), C.c_int(nbins), C.c_uint64(seed),
                                _dptr(hc), _dptr(he), _dptr(sums))
    if rc != 0:
        raise RuntimeError(f"ref_interactions failed: {rc}")
    return hc, he, sums


CT_CALIBRATION = 7  # the axial copy a CT spiral source calibrates with
CTSPIRAL_DUAL, CTAXIAL_DUAL, CTTOPOGRAM = 8, 9, 10


def ctdi_phantom(diameter: int):
    """CTDIPhantom<double> arrays and hole index lists (Center, West, East, South, North)."""
    dims = (C.c_uint64 * 3)()
    counts = (C.c_uint64 * 5)()
    rc = lib().ref_ctdi_phantom(C.c_int(diameter), dims, None, None, None, counts, None, C.c_uint64(0))
    if rc != 0:
        raise RuntimeError(f"ref_ctdi_phantom failed: {rc}")
    n = dims[0] * dims[1] * dims[2]
    dens = np.zeros(n)
    mat = np.zeros(n, np.uint8)
    meas = np.zeros(n, np.uint8)
    total = int(sum(counts))
    holes = np.zeros(total, np.uint64)
    rc = lib().ref_ctdi_phantom(C.c_int(diameter), dims, _dptr(dens), mat.ctypes.data_as(C.POINTER(C.c_uint8)),
                                meas.ctypes.data_as(C.POINTER(C.c_uint8)), counts,
                                holes.ctypes.data_as(C.POINTER(C.c_uint64)), C.c_uint64(total))
    if rc != 0:
        raise RuntimeError(f"ref_ctdi_phantom failed: {rc}")
    return (tuple(int(d) for d in dims), dens, mat, meas, [int(c) for c in counts], holes)


def ct_calibration(source: "SourceArgs", model: int, ctdivol: float, diameter: int):
    """CTSpiralSource<double>::getCalibrationValue with the reference's own transport."""
    factor = C.c_double(0)
    meta = np.zeros(3)
    rc = lib().ref_ct_calibration(C.byref(source.desc), C.c_int(model), C.c_int(0), C.c_double(ctdivol),
                                  C.c_int(diameter), C.byref(factor), _dptr(meta))
    if rc != 0:
        raise RuntimeError(f"ref_ct_calibration failed: {rc}")
    return factor.value, meta


def transport_ex(world: WorldArgs, source: SourceArgs, model: int = 1, n_threads: int = 0, output_mode: int = 0,
                 use_calibration: bool = False, precision: int = 0):
    """Transport<T>::operator() in T = double (precision 0) or float (1), in
    EV_PER_HISTORY (output_mode 0) or DOSE (1) mode.  Returns (dose, variance,
    nEvents, histories, simulation seconds, units) with units 0 eV/history,
    1 keV/kg, 2 mGy."""
    n = world.size
    dose = np.zeros(n, np.float64)
    var = np.zeros(n, np.float64)
    nev = np.zeros(n, np.uint32)
    meta = np.zeros(4, np.float64)
    rc = lib().ref_transport_ex(C.byref(world.desc), C.byref(source.desc), C.c_int(model), C.c_int(n_threads),
                                C.c_int(output_mode), C.c_int(1 if use_calibration else 0), C.c_int(precision),
                                _dptr(dose), _dptr(var), nev.ctypes.data_as(C.POINTER(C.c_uint32)), _dptr(meta))
    if rc != 0:
        raise RuntimeError(f"ref_transport_ex failed: {rc}")
    return dose, var, nev, int(meta[0]), float(meta[1]), int(meta[3])


def calibration_value(world: WorldArgs, source: SourceArgs, model: int = 1) -> float:
    """Source::getCalibrationValue after updateFromWorld / validate (the factor DOSE
    mode multiplies keV/kg by to give mGy)."""
    v = C.c_double(0)
    rc = lib().ref_calibration_value(C.byref(world.desc), C.byref(source.desc), C.c_int(model), C.byref(v))
    if rc != 0:
        raise RuntimeError(f"ref_calibration_value failed: {rc}")
    return v.value
