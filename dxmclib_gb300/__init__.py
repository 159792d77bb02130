"""GB300-native (sm_103a) photon-transport engine for DXMClib's hot path.

The public Python surface mirrors DXMClib's World / Material / Source /
Transport API; the transport runs in hand-written CUDA kernels behind the C
ABI declared in include/dxmc_gpu.h.
"""
from ._capi import DxmcError, load as load_library  # noqa: F401
from .api import (  # noqa: F401
    LOWENERGYCORRECTION, Batch, BatchEntry, Beam, CBCTSource, CTAxialDualSource, CTAxialSource, CTSpiralDualSource, CTSpiralSource,
    CTTopogramSource, DAPSource, DeviceLut, DeviceWorld, DXSource, ExposureTable, GpuContext, HeelTable, IsotropicCTSource, IsotropicSource, Job, LutBlob,
    Material, PencilSource, Result, Source, Spectrum, Transport, World,
)
from .tube import HeelFilter, Tube  # noqa: F401
from . import workloads  # noqa: F401

__all__ = [
    "LOWENERGYCORRECTION", "Batch", "BatchEntry", "Beam", "CBCTSource", "DAPSource", "IsotropicCTSource", "CTAxialDualSource", "CTAxialSource", "CTSpiralDualSource",
    "CTSpiralSource", "CTTopogramSource", "DeviceLut", "DeviceWorld", "DXSource", "ExposureTable", "GpuContext",
    "HeelTable", "IsotropicSource", "Job", "LutBlob", "Material", "PencilSource", "Result", "Source", "Spectrum",
    "Transport", "World", "HeelFilter", "Tube", "DxmcError", "load_library",
]
