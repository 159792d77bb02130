"""Statistical parity checks between two Monte Carlo tallies.

DXMClib's RNG is seeded from std::random_device (dxmcrandom.hpp:42-48), so
agreement with the reference is statistical: per-voxel differences are judged
against the combined standard error sqrt(var_a + var_b) built from each side's
variance field (transport.hpp:780-794, EV_PER_HISTORY mode).
"""
from __future__ import annotations

import numpy as np

# Acceptance thresholds.
THREE_SIGMA_FRACTION = 0.99   # voxels above 1 % of max within 3 combined standard errors (expect 0.997)
TOTAL_ENERGY_RTOL = 0.005     # total energy imparted within 0.5 %
MEAN_BIAS_RTOL = 0.01         # dose-weighted mean per-voxel relative difference within 1 %


def compare_sparse(ref: dict, dose: np.ndarray, var: np.ndarray, min_frac: float = 0.01) -> dict:
    idx = ref["idx"].astype(np.int64)
    d1, v1 = ref["dose"], ref["var"]
    # select on the mean of both tallies so that neither side's noise biases the selection
    mean = 0.5 * (d1 + dose[idx])
    sel = mean > min_frac * mean.max()
    i = idx[sel]
    d1, v1 = d1[sel], v1[sel]
    d2, v2 = dose[i], var[i]
    sigma = np.sqrt(np.maximum(v1, 0) + np.maximum(v2, 0))
    z = (d2 - d1) / np.where(sigma > 0, sigma, np.inf)
    return dict(
        n_voxels=int(sel.sum()),
        frac_3sigma=float(np.mean(np.abs(z) <= 3.0)),
        chi2=float(np.mean(z * z)),
        total_ratio=float(dose.sum() / ref["total"][0]),
        # dose-weighted mean relative difference: sum(d2 - d1) / sum(d1); the unweighted
        # mean of ratios is biased by noise in the denominator when voxels are noisy
        mean_bias=float(np.sum(d2 - d1) / np.sum(d1)),
        mean_rel_unweighted=float(np.mean((d2 - d1) / d1)),
        mean_abs_rel=float(np.mean(np.abs(d2 - d1) / d1)),
        max_abs_z=float(np.max(np.abs(z))) if len(z) else 0.0,
    )


def assert_parity(stats: dict, label: str = "") -> None:
    msg = f"{label}: {stats}"
    assert stats["n_voxels"] > 10, msg
    assert stats["frac_3sigma"] >= THREE_SIGMA_FRACTION, msg
    assert abs(stats["total_ratio"] - 1.0) <= TOTAL_ENERGY_RTOL, msg
    assert abs(stats["mean_bias"]) <= MEAN_BIAS_RTOL, msg
