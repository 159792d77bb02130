"""ctypes declarations for the C ABI in include/dxmc_gpu.h.

The shared library is built in-tree by ``dxmclib_gb300.build`` into
``dxmclib_gb300/lib/libdxmc_gpu.so``.  Loading it never falls back to another
implementation: a missing or unloadable library raises ``RuntimeError``.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
LIB_DIR = PKG_DIR / "lib"
LIB_NAME = "libdxmc_gpu.so"

DXMC_OK = 0
DXMC_ERR_INVALID = -1
DXMC_ERR_OOM = -2
DXMC_ERR_DEVICE = -3
DXMC_ERR_REJECTION_CAP = -4
DXMC_ERR_TIMEOUT = -5
DXMC_ERR_CANCELLED = -6
DXMC_ERR_NO_DEVICE = -7
DXMC_ERR_STATE = -8

STATUS_NAMES = {
    0: "DXMC_OK", -1: "DXMC_ERR_INVALID", -2: "DXMC_ERR_OOM", -3: "DXMC_ERR_DEVICE",
    -4: "DXMC_ERR_REJECTION_CAP", -5: "DXMC_ERR_TIMEOUT", -6: "DXMC_ERR_CANCELLED",
    -7: "DXMC_ERR_NO_DEVICE", -8: "DXMC_ERR_STATE",
}

MODEL_NONE, MODEL_LIVERMORE, MODEL_IA = 0, 1, 2
OUTPUT_RAW, OUTPUT_EV_PER_HISTORY, OUTPUT_DOSE = 0, 1, 2
TALLY_F64, TALLY_F32, TALLY_WARP_F64 = 0, 1, 2
TRACKING_DEFAULT, TRACKING_GLOBAL, TRACKING_LOCAL = 0, 1, 2
DIRECTION_REFERENCE, DIRECTION_NORMALIZED = 0, 1
PRECISION_FP32, PRECISION_FP64 = 0, 1
RESULT_F64, RESULT_F32 = 0, 1

D = C.c_double
DP = C.POINTER(C.c_double)
FP = C.POINTER(C.c_float)
U8P = C.POINTER(C.c_uint8)
U32P = C.POINTER(C.c_uint32)
U64P = C.POINTER(C.c_uint64)
VP = C.c_void_p


class ShellConfig(C.Structure):
    _fields_ = [
        ("binding_energy", D), ("number_electrons", D), ("hartree_fock_j0", D),
        ("photo_ionization_probability", D), ("fluorescence_yield", D),
        ("line_probabilities", D * 3), ("line_energies", D * 3),
        ("Z", C.c_int32), ("shell", C.c_int32),
    ]


PHOTO_CB = C.CFUNCTYPE(D, VP, D)
EDGES_CB = C.CFUNCTYPE(C.c_int, VP, D, DP, C.c_int)
SHELLS_CB = C.CFUNCTYPE(None, VP, C.POINTER(ShellConfig))


class MaterialProvider(C.Structure):
    _fields_ = [
        ("user", VP), ("standard_density", D),
        ("photoelectric", PHOTO_CB), ("compton", PHOTO_CB), ("rayleigh", PHOTO_CB),
        ("form_factor_squared", PHOTO_CB), ("scatter_factor", PHOTO_CB),
        ("binding_energies", EDGES_CB), ("shells", SHELLS_CB),
    ]


class LutInfo(C.Structure):
    _fields_ = [
        ("n_materials", C.c_int32), ("n_energy", C.c_int32), ("linear_index", C.c_int32), ("pad", C.c_int32),
        ("linear_step", D), ("linear_energy", D), ("min_energy", D), ("max_energy", D),
        ("log_energy", DP), ("coefficients", DP), ("max_coefficients", DP), ("rita", DP), ("spline", DP),
        ("shells", C.POINTER(ShellConfig)),
    ]


class Exposure(C.Structure):
    _fields_ = [
        ("position", D * 3), ("direction_cosines", D * 6), ("beam_direction", D * 3),
        ("collimation", D * 4), ("weight", D), ("n_histories", C.c_uint64), ("mono_energy", D),
    ]


class SpectrumDesc(C.Structure):
    _fields_ = [("n", C.c_int32), ("energies", DP), ("weights", DP)]


class HeelDesc(C.Structure):
    _fields_ = [
        ("energy_start", D), ("energy_step", D), ("energy_size", C.c_int32), ("angle_size", C.c_int32),
        ("angle_start", D), ("angle_step", D), ("weights", DP),
    ]


class BowtieDesc(C.Structure):
    _fields_ = [("n", C.c_int32), ("angles", DP), ("weights", DP)]


class GpuOptions(C.Structure):
    _fields_ = [
        ("device", C.c_int32), ("block_size", C.c_int32), ("blocks_per_sm", C.c_int32),
        ("tally_mode", C.c_int32), ("memory_budget", C.c_uint64),
        ("regen_threshold", C.c_int32), ("interact_threshold", C.c_int32),
        ("queue_log2_chunk", C.c_int32), ("tracking", C.c_int32),
    ]


class WorldDesc(C.Structure):
    _fields_ = [
        ("dims", C.c_uint64 * 3), ("spacing", D * 3), ("origin", D * 3), ("direction_cosines", D * 6),
        ("density", FP), ("material", U8P), ("measurement", U8P), ("n_materials", C.c_int32), ("layout", C.c_int32),
    ]


class JobDesc(C.Structure):
    _fields_ = [
        ("exposures", C.POINTER(Exposure)), ("n_exposures", C.c_uint64),
        ("spectrum", C.POINTER(SpectrumDesc)), ("heel", C.POINTER(HeelDesc)), ("bowtie", C.POINTER(BowtieDesc)),
        ("seed", C.c_uint64), ("model", C.c_int32), ("tally_mode", C.c_int32),
        ("regen_threshold", C.c_int32), ("interact_threshold", C.c_int32), ("blocks_per_sm", C.c_int32),
        ("queue_log2_chunk", C.c_int32), ("woodcock_burst", C.c_int32), ("block_size", C.c_int32),
        ("tracking", C.c_int32), ("direction", C.c_int32), ("precision", C.c_int32),
    ]


class JobStats(C.Structure):
    _fields_ = [
        ("histories", C.c_uint64), ("steps", C.c_uint64), ("deposits", C.c_uint64),
        ("rejection_overflows", C.c_uint64), ("kernel_ms", D), ("job_ms", D),
    ]


class BatchEntry(C.Structure):
    _fields_ = [("world", VP), ("lut", VP), ("job", C.POINTER(JobDesc))]


BATCH_AUTO, BATCH_CONCURRENT, BATCH_PERSISTENT = 0, 1, 2


class BatchOptions(C.Structure):
    _fields_ = [("mode", C.c_int32), ("chains", C.c_int32), ("regen_threshold", C.c_int32),
                ("interact_threshold", C.c_int32), ("item_histories", C.c_int32), ("pad", C.c_int32)]


# name -> (restype, argtypes)
SIGNATURES = {
    "dxmc_gpu_abi_version": (C.c_int, []),
    "dxmc_udiv_invariant": (C.c_int, [C.POINTER(C.c_uint32), C.c_uint64, C.c_uint32, C.POINTER(C.c_uint32)]),
    "dxmc_physics_material": (C.c_int, [C.c_char_p, D, C.POINTER(MaterialProvider)]),
    "dxmc_physics_material_free": (None, [C.POINTER(MaterialProvider)]),
    "dxmc_physics_mass_energy_absorption": (C.c_int, [C.POINTER(MaterialProvider), D, DP]),
    "dxmc_tube_spectrum": (C.c_int, [D, D, D, DP, C.c_int, C.POINTER(MaterialProvider), DP, C.c_int, C.c_int, DP]),
    "dxmc_physics_element_material": (C.c_int, [C.c_int, C.POINTER(MaterialProvider)]),
    "dxmc_lut_build": (C.c_int, [C.POINTER(MaterialProvider), C.c_int, FP, U8P, C.c_uint64, D, C.POINTER(VP)]),
    "dxmc_lut_build_max_density": (C.c_int, [C.POINTER(MaterialProvider), C.c_int, DP, D, C.POINTER(VP)]),
    "dxmc_lut_blob_free": (None, [VP]),
    "dxmc_lut_attenuation": (C.c_int, [VP, C.c_int, D, DP]),
    "dxmc_lut_max_attenuation_inverse": (D, [VP, D]),
    "dxmc_lut_scatter_factor": (D, [VP, C.c_int, D]),
    "dxmc_lut_get_info": (C.c_int, [VP, C.POINTER(LutInfo)]),
    "dxmc_alias_table": (C.c_int, [DP, C.c_int, DP, U64P]),
    "dxmc_bowtie_table": (C.c_int, [DP, DP, C.c_int, DP, DP]),
    "dxmc_stream_seed": (C.c_int, [C.c_uint64, C.c_uint64, U32P]),
    "dxmc_gpu_ctx_create": (C.c_int, [C.POINTER(GpuOptions), C.POINTER(VP)]),
    "dxmc_gpu_ctx_destroy": (None, [VP]),
    "dxmc_gpu_last_error": (C.c_char_p, [VP]),
    "dxmc_gpu_device_count": (C.c_int, []),
    "dxmc_gpu_world_upload": (C.c_int, [VP, C.POINTER(WorldDesc), C.POINTER(VP)]),
    "dxmc_gpu_world_max_density": (C.c_int, [VP, DP, C.c_int]),
    "dxmc_gpu_world_free": (None, [VP]),
    "dxmc_gpu_world_prepare": (C.c_int, [VP, VP, VP]),
    "dxmc_gpu_world_majorant": (C.c_int, [VP, VP, VP, C.POINTER(C.c_uint32), C.POINTER(C.c_int32),
                                          C.POINTER(C.c_int32), FP, FP, FP]),
    "dxmc_gpu_lut_upload": (C.c_int, [VP, VP, C.POINTER(VP)]),
    "dxmc_gpu_lut_free": (None, [VP]),
    "dxmc_gpu_job_submit": (C.c_int, [VP, VP, VP, C.POINTER(JobDesc), C.POINTER(VP)]),
    "dxmc_gpu_job_wait": (C.c_int, [VP, C.c_int64]),
    "dxmc_gpu_job_cancel": (C.c_int, [VP]),
    "dxmc_gpu_job_result": (C.c_int, [VP, C.c_int, D, DP, DP, U32P, C.POINTER(JobStats)]),
    "dxmc_gpu_job_free": (None, [VP]),
    "dxmc_gpu_job_result_async": (C.c_int, [VP, C.c_int, D, C.c_int, VP, VP, U32P]),
    "dxmc_gpu_job_result_wait": (C.c_int, [VP, C.POINTER(JobStats)]),
    "dxmc_gpu_probe_lut": (C.c_int, [VP, VP, C.c_int, DP, C.c_int, DP, DP]),
    "dxmc_gpu_job_release": (C.c_int, [VP]),
    "dxmc_gpu_job_progress": (C.c_int, [VP, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    "dxmc_gpu_job_preview": (C.c_int, [VP, DP]),
    "dxmc_gpu_radiological_path": (C.c_int, [VP, VP, VP, FP, C.c_uint64, DP]),
    "dxmc_gpu_ctx_memory": (C.c_int, [VP, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    "dxmc_gpu_host_alloc": (C.c_int, [C.c_uint64, C.POINTER(VP)]),
    "dxmc_gpu_host_free": (None, [VP]),
    "dxmc_gpu_batch_submit": (C.c_int, [VP, C.POINTER(BatchEntry), C.c_int, C.POINTER(BatchOptions), C.POINTER(VP)]),
    "dxmc_gpu_batch_wait": (C.c_int, [VP, C.c_int64]),
    "dxmc_gpu_batch_job": (C.c_int, [VP, C.c_int, C.POINTER(VP)]),
    "dxmc_gpu_batch_kernel_ms": (D, [VP]),
    "dxmc_gpu_batch_free": (None, [VP]),
    "dxmc_gpu_transport_noalloc": (C.c_int, [VP, VP, VP, C.POINTER(JobDesc), VP, VP, C.POINTER(JobStats)]),
    "dxmc_gpu_probe_interactions": (C.c_int, [VP, VP, C.c_int, C.c_int, C.c_int, D, C.c_uint64, C.c_uint64, FP, FP, FP]),
    "dxmc_gpu_probe_uniform": (C.c_int, [VP, C.c_uint64, C.c_uint64, C.c_uint32, C.c_int, C.c_int32, U64P]),
}

_lib = None


def library_path() -> Path:
    override = os.environ.get("DXMC_GPU_LIBRARY")
    return Path(override) if override else LIB_DIR / LIB_NAME


def load():
    """Load libdxmc_gpu.so; raises RuntimeError if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not path.exists():
        raise RuntimeError(
            f"{path} is missing: build the CUDA extension first (python -c 'import dxmclib_gb300.build as b; b.build()')")
    lib = C.CDLL(str(path), mode=C.RTLD_GLOBAL)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(rc: int, ctx=None, what: str = "") -> None:
    if rc != DXMC_OK:
        msg = STATUS_NAMES.get(rc, str(rc))
        if ctx is not None and _lib is not None:
            err = _lib.dxmc_gpu_last_error(ctx)
            if err:
                msg += ": " + err.decode(errors="replace")
        raise DxmcError(rc, f"{what} failed: {msg}")


class DxmcError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(message)
        self.status = status
