"""Shared pytest configuration: the ``gpu`` marker, the in-tree library build
and access to the golden fixtures produced by the reference."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parents[1]
GOLDEN = REPO / "tests" / "golden"
sys.path.insert(0, str(REPO))
sys.path.insert(0, str(REPO / "tests"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300); run with -m gpu")


@pytest.fixture(scope="session")
def lib():
    """Builds (if stale) and loads libdxmc_gpu.so."""
    from dxmclib_gb300 import build as b
    b.build()
    from dxmclib_gb300 import _capi
    return _capi.load()


@pytest.fixture(scope="session")
def golden():
    def load(name: str):
        path = GOLDEN / name
        if not path.exists():
            pytest.fail(f"golden fixture {name} is missing; regenerate with tests/golden/make_golden.py")
        with np.load(path, allow_pickle=False) as f:
            return {k: f[k] for k in f.files}
    return load


@pytest.fixture(scope="session")
def gpu_ctx(lib):
    from dxmclib_gb300 import GpuContext
    if lib.dxmc_gpu_device_count() < 1:
        pytest.fail("no CUDA device visible: GPU tests need a GB300")
    ctx = GpuContext()
    yield ctx
    ctx.close()
