"""CPU checks of the Siddon restatement in oracle/siddon.py against closed-form
chord lengths (its parity with DXMClib is unpinned: DXMClib has no Siddon
traversal)."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parents[1] / "oracle"))
import siddon  # noqa: E402


def test_chords_through_a_homogeneous_box():
    dims, sp, lo = (10, 8, 6), (2.0, 3.0, 4.0), (-10.0, -12.0, -12.0)
    n = int(np.prod(dims))
    dens = np.full(n, 2.0)
    mat = np.zeros(n, np.uint8)
    mu = lambda m, e: 0.5  # noqa: E731
    rays = np.array([
        [-50, 0.1, 0.2, 1, 0, 0, 60],       # along x: chord 20 mm
        [0.3, -50, 0.2, 0, 1, 0, 60],       # along y: chord 24 mm
        [0.3, 0.1, -50, 0, 0, 1, 60],       # along z: chord 24 mm
        [0.0, 0.0, 0.0, 1, 0, 0, 60],       # from the centre: 10 mm
        [-50, -50, -50, 1, 1, 1, 60],       # diagonal through the origin
        [-50, 100, 0, 1, 0, 0, 60],         # misses
        [5.0, 5.0, 5.0, -1, -1, -1, 60],    # from inside backwards through the corner region
    ], float)
    out = siddon.radiological_path(dims, sp, lo, dens, mat, mu, rays)
    k = 0.5 * 2.0 * 0.1
    # the diagonal enters at the largest slab entry and leaves at the smallest exit
    d = np.ones(3) / np.sqrt(3)
    hi = np.array(lo) + np.array(sp) * np.array(dims)
    t1 = (np.array(lo) - (-50)) / d
    t2 = (hi - (-50)) / d
    diag = min(t2) - max(t1)
    t1b = (np.array(lo) - 5.0) / -d
    back = min(t1b)  # from (5,5,5) backwards until the first face
    np.testing.assert_allclose(out, [20 * k, 24 * k, 24 * k, 10 * k, diag * k, 0.0, back * k], rtol=1e-12, atol=1e-12)


def test_segments_sum_over_materials():
    # two slabs of different material along x
    dims, sp, lo = (4, 1, 1), (5.0, 5.0, 5.0), (0.0, 0.0, 0.0)
    dens = np.array([1.0, 1.0, 3.0, 3.0])
    mat = np.array([0, 0, 1, 1], np.uint8)
    mu = lambda m, e: [0.2, 0.4][m]  # noqa: E731
    out = siddon.radiological_path(dims, sp, lo, dens, mat, mu, [[-1, 2.5, 2.5, 1, 0, 0, 50]])
    assert abs(out[0] - 0.1 * (0.2 * 1.0 * 10 + 0.4 * 3.0 * 10)) < 1e-12
