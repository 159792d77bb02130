"""GPU test: uniformity of the device random streams.

Every device sampler draws from per-history xoshiro128+ streams whose state is
SplitMix64 of (seed, history).  DXMClib checks its own generator by
binning 1e8 uniforms into 100 bins and requiring each bin within 5 % of the
nominal count (tests/testrandom.cpp:21-58).  The same check runs here on the
device streams through dxmc_gpu_probe_uniform (the C ABI), with a chi-square
test on top: at 1e6 counts per bin the 5 % bound alone would pass a visibly
biased generator.  The streams are short (100 draws each, as a history uses
them) and many (1e6 histories), so the check also covers the seeding.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest
from scipy import stats as sps

pytestmark = pytest.mark.gpu

DRAWS = 100_000_000
BINS = 100


def _histogram(ctx, kind, n_bins=BINS, streams=1_000_000, seed=20261204):
    from dxmclib_gb300 import _capi as A
    hist = np.zeros(n_bins + 1, np.uint64)
    rc = ctx.lib.dxmc_gpu_probe_uniform(ctx.handle, seed, streams, DRAWS // streams, kind, n_bins,
                                        hist.ctypes.data_as(C.POINTER(C.c_uint64)))
    A.check(rc, ctx.handle, "dxmc_gpu_probe_uniform")
    return hist[:n_bins].astype(np.float64), int(hist[n_bins])


@pytest.mark.parametrize("kind,label", [(0, "uniform [0, 1)"), (1, "uniform (0, 1]"), (2, "integer below n")])
def test_device_stream_uniformity(gpu_ctx, kind, label):
    counts, outside = _histogram(gpu_ctx, kind)
    assert outside == 0, f"{label}: {outside} values outside the range"
    assert counts.sum() == DRAWS
    nominal = DRAWS / BINS
    diff_pct = counts * 100.0 / nominal - 100.0
    # the reference's criterion (testrandom.cpp:48): every bin within 5 %
    assert np.all(np.abs(diff_pct) < 5.0), diff_pct
    # chi-square against uniform: a p-value below 1e-6 fails
    chi2 = float(np.sum((counts - nominal) ** 2 / nominal))
    p = float(sps.chi2.sf(chi2, BINS - 1))
    print(f"{label}: chi2/dof {chi2 / (BINS - 1):.3f}, p {p:.3g}, max |diff| {np.abs(diff_pct).max():.3f} %")
    assert p > 1e-6, (chi2, p)


def test_device_streams_fine_bins_and_seeds(gpu_ctx):
    """4096 bins resolve the 23-bit float mantissa mapping near 0 and 1, and two
    seeds give different but equally uniform histograms (independent streams)."""
    a, _ = _histogram(gpu_ctx, 0, n_bins=4096, seed=1)
    b, _ = _histogram(gpu_ctx, 0, n_bins=4096, seed=2)
    assert not np.array_equal(a, b)
    for h in (a, b):
        nominal = h.sum() / len(h)
        chi2 = float(np.sum((h - nominal) ** 2 / nominal))
        assert sps.chi2.sf(chi2, len(h) - 1) > 1e-6, chi2 / (len(h) - 1)
