"""CPU test of the C++ drop-in adapter (include/dxmc_gpu/transport.hpp).

Compiles the adapter together with DXMClib's unmodified headers (and the
project Material backend that stands in for xraylib) and runs its host-side
checks.  Needs the reference checkout, named by DXMC_REFERENCE; skipped without it.
"""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parents[1]
REF = Path(os.environ["DXMC_REFERENCE"]) if os.environ.get("DXMC_REFERENCE") else None


def test_cpp_adapter_host_checks(lib, tmp_path):
    if REF is None or not (REF / "include" / "dxmc").is_dir():
        pytest.skip("DXMClib headers not available (set DXMC_REFERENCE to a reference checkout)")
    exe = tmp_path / "adapter_check"
    cmd = ["g++", "-std=c++20", "-O1", "-pthread", f"-I{REF / 'include'}", f"-I{REPO / 'include'}", f"-I{REPO / 'oracle'}",
           str(REPO / "tests" / "adapter" / "adapter_check.cpp"), str(REPO / "oracle" / "material_backend.cpp"),
           str(REPO / "dxmclib_gb300" / "csrc" / "physics" / "physics_model.cpp"),
           f"-L{REPO / 'dxmclib_gb300' / 'lib'}", "-ldxmc_gpu", f"-Wl,-rpath,{REPO / 'dxmclib_gb300' / 'lib'}",
           "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "FAIL" not in r.stdout
