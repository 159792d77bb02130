"""In-tree build of libdxmc_gpu.so (sm_103a) and of the CPU oracle libraries.

Host C++ is compiled with g++, CUDA with nvcc for ``sm_103a`` only; the
translation units compile in parallel and link into
``dxmclib_gb300/lib/libdxmc_gpu.so``.  No cmake, no torch extension machinery.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
REPO = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "lib"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CXX = os.environ.get("CXX", "g++")
NVCC = os.environ.get("NVCC", shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc")

HOST_SOURCES = [
    CSRC / "physics" / "physics_model.cpp",
    CSRC / "host" / "lut_builder.cpp",
    CSRC / "host" / "capi_host.cpp",
    CSRC / "host" / "tube_spectrum.cpp",
]
CUDA_SOURCES = [
    CSRC / "kernels" / "transport_kernels.cu",
    CSRC / "device" / "capi_device.cu",
    CSRC / "device" / "noalloc.cu",
    CSRC / "kernels" / "siddon_kernels.cu",
    CSRC / "kernels" / "majorant_kernels.cu",
]
INCLUDES = [f"-I{REPO / 'include'}", f"-I{CSRC}"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(map(str, cmd))}\n{r.stdout}\n{r.stderr}")
    return r


def _stale(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def _headers():
    return list(CSRC.rglob("*.hpp")) + list(CSRC.rglob("*.cuh")) + list((REPO / "include").rglob("*.h"))


def build(verbose: bool = False, force: bool = False) -> Path:
    """Compile everything that is out of date; returns the path of libdxmc_gpu.so.

    DXMC_NVCC_DEFINES (e.g. "-DDXMC_MIN_BLOCKS_PER_SM=3") adds preprocessor
    definitions to the CUDA translation units; a change of it forces a rebuild."""
    BUILD.mkdir(exist_ok=True)
    LIB.mkdir(exist_ok=True)
    defines = os.environ.get("DXMC_NVCC_DEFINES", "").split()
    stamp = BUILD / "nvcc_defines.txt"
    if not stamp.exists() or stamp.read_text() != " ".join(defines):
        force = True
        stamp.write_text(" ".join(defines))
    headers = _headers()
    jobs = []
    objects = []
    for src in HOST_SOURCES:
        obj = BUILD / (src.stem + ".o")
        objects.append(obj)
        if force or _stale(obj, [src, *headers]):
            # no contraction of a * b + c into fused multiply-adds: the host tables (LUT,
            # tube spectra) must come out the same on x86-64 and aarch64 (where GCC fuses
            # by default), as the reference's own x86 build computes them
            jobs.append([CXX, "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-Wall", "-c", str(src), "-o", str(obj),
                         *INCLUDES])
    for src in CUDA_SOURCES:
        obj = BUILD / (src.stem + ".o")
        objects.append(obj)
        if force or _stale(obj, [src, *headers]):
            # the transport kernels use the fast single-precision intrinsics (Monte Carlo
            # sampling tolerates their ulp-level error; tallies stay FP64)
            fast = ["-use_fast_math"] if src.name == "transport_kernels.cu" else []
            jobs.append([NVCC, *ARCH, "-lineinfo", "-O3", "-std=c++17", *fast, "-Xcompiler", "-fPIC,-ffp-contract=off", *defines, "-c", str(src), "-o",
                         str(obj), *INCLUDES])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for r in ex.map(_run, jobs):
            if verbose and (r.stdout or r.stderr):
                print(r.stdout, r.stderr, file=sys.stderr)
    out = LIB / "libdxmc_gpu.so"
    if force or _stale(out, objects):
        _run([NVCC, *ARCH, "-shared", "-o", str(out), *map(str, objects), "-lcudart", "-lpthread"])
    return out


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
