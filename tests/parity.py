"""Statistical parity checks between two Monte Carlo tallies.

DXMClib's RNG is seeded from std::random_device (dxmcrandom.hpp:42-48), so
agreement with the reference is statistical: per-voxel differences are judged
against the combined standard error sqrt(var_a + var_b) built from each side's
variance field (transport.hpp:780-794, EV_PER_HISTORY mode).
"""
from __future__ import annotations

import numpy as np

# Acceptance thresholds.
# Voxels above 1 % of max beyond 3 combined standard errors: a Gaussian tally has
# 0.27 % of them; the count may exceed that by 4 binomial standard deviations
# (false-alarm rate about 1e-4 per comparison), and no voxel may be beyond 6.
P_BEYOND_3SIGMA = 0.0027
MAX_ABS_Z = 6.0
# The variance field sums squared deposits per event, not per history
# (transport.hpp:601, 609, 621, 629), so it under-estimates the variance of the
# mean when one history deposits more than once in a voxel; the reference
# restated on the CPU shows chi2/dof = 1.03 against the reference itself on the
# forced-interaction case.  z is therefore rescaled by the observed
# overdispersion (chi2/dof, at least 1) before counting, and chi2/dof itself is
# bounded so that real per-voxel disagreements still fail.
MAX_CHI2 = 1.2
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
    with np.errstate(divide="ignore", invalid="ignore"):  # a voxel of one tally may be empty
        rel = (d2 - d1) / d1
    return dict(
        n_voxels=int(sel.sum()),
        frac_3sigma=float(np.mean(np.abs(z) <= 3.0)),
        chi2=float(np.mean(z * z)),
        beyond_3sigma=int(np.sum(np.abs(z) / np.sqrt(max(1.0, float(np.mean(z * z)))) > 3.0)),
        total_ratio=float(dose.sum() / ref["total"][0]),
        # dose-weighted mean relative difference: sum(d2 - d1) / sum(d1); the unweighted
        # mean of ratios is biased by noise in the denominator when voxels are noisy
        mean_bias=float(np.sum(d2 - d1) / np.sum(d1)),
        mean_rel_unweighted=float(np.mean(rel)),
        mean_abs_rel=float(np.mean(np.abs(rel))),
        max_abs_z=float(np.max(np.abs(z)) / np.sqrt(max(1.0, float(np.mean(z * z))))) if len(z) else 0.0,
    )


def assert_parity(stats: dict, label: str = "", correlated: bool = False, max_chi2: float = MAX_CHI2) -> None:
    """correlated=True for forced-interaction scoring, where every Woodcock step in a
    measured voxel scores a deposit: the per-event variance field is then far from
    Gaussian voxel to voxel (the reference restated on the CPU exceeds the plain
    Gaussian count against the reference itself), so twice the Gaussian rate of
    3-sigma exceedances is allowed.  max_chi2 replaces the chi2/dof bound where a
    same-method comparison measured the overdispersion of the pair."""
    msg = f"{label}: {stats}"
    report(stats, label)
    assert stats["n_voxels"] > 10, msg
    n = stats["n_voxels"]
    p_beyond = P_BEYOND_3SIGMA * (2.0 if correlated else 1.0)
    allowed = int(p_beyond * n + 4.0 * np.sqrt(p_beyond * (1 - p_beyond) * n)) + 1
    assert stats["beyond_3sigma"] <= allowed, msg + f" (allowed {allowed} beyond 3 sigma)"
    assert stats["max_abs_z"] <= MAX_ABS_Z, msg
    # chi2/dof of n standard normals has standard deviation sqrt(2 / n)
    assert stats["chi2"] <= max_chi2 + 4.0 * np.sqrt(2.0 / n), msg
    assert abs(stats["total_ratio"] - 1.0) <= TOTAL_ENERGY_RTOL, msg
    assert abs(stats["mean_bias"]) <= MEAN_BIAS_RTOL, msg


def block_sums(values: np.ndarray, dims, block) -> np.ndarray:
    """Sums of a voxel array (x fastest, dims = (nx, ny, nz)) over blocks of
    block = (bx, by, bz) voxels, in the block grid's x-fastest order."""
    nx, ny, nz = (int(d) for d in dims)
    bx, by, bz = (int(b) for b in block)
    a = np.asarray(values, np.float64).reshape(nz // bz, bz, ny // by, by, nx // bx, bx)
    return a.sum(axis=(1, 3, 5)).ravel()


def report(stats: dict, label: str) -> None:
    """One line per parity case with chi2/dof, printed into the test output."""
    print(f"[parity] {label}: chi2/n {stats['chi2']:.3f} over {stats['n_voxels']} voxels, "
          f"{stats['beyond_3sigma']} beyond 3 sigma, max |z| {stats['max_abs_z']:.2f}, "
          f"total ratio {stats['total_ratio']:.5f}, mean bias {stats['mean_bias']:+.5f}")
