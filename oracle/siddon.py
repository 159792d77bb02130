"""CPU restatement of the radiological path through a voxel grid (Siddon,
Med. Phys. 12 (1985) 252: every crossing of a voxel boundary plane is a
parametric value along the ray; the sorted values cut the ray into segments
whose midpoints give the voxel).  ORACLE TEST INFRASTRUCTURE: imported only by
tests/ as the checker of dxmc_gpu_radiological_path.

Parity unpinned: DXMClib has no Siddon traversal (it tracks photons with
Woodcock steps only, docs/sphinx/physicsmodel.rst:27), so there is no
reference output to pin against; this restatement is checked against
closed-form chord lengths in tests/test_siddon_oracle.py instead.
"""
from __future__ import annotations

import numpy as np


def radiological_path(dims, spacing, lower, density, material, mu_rho, rays) -> np.ndarray:
    """``rays``: (n, 7) origin (mm), direction, energy (keV); ``mu_rho(material,
    energy)`` the mass attenuation (cm^2/g).  Returns sum mu/rho * density *
    length (cm) over the forward part of each ray inside the grid."""
    dims = np.asarray(dims, np.int64)
    sp = np.asarray(spacing, np.float64)
    lo = np.asarray(lower, np.float64)
    hi = lo + sp * dims
    dens = np.asarray(density, np.float64).ravel()
    mat = np.asarray(material).ravel()
    rays = np.asarray(rays, np.float64)
    out = np.zeros(len(rays))
    cache = {}
    for r, ray in enumerate(rays):
        o, d, e = ray[0:3], ray[3:6].copy(), ray[6]
        n = np.linalg.norm(d)
        if n == 0 or e <= 0:
            continue
        d /= n
        tmin, tmax = 0.0, np.inf
        miss = False
        for k in range(3):
            if d[k] != 0:
                t1, t2 = (lo[k] - o[k]) / d[k], (hi[k] - o[k]) / d[k]
                tmin, tmax = max(tmin, min(t1, t2)), min(tmax, max(t1, t2))
            elif not (lo[k] <= o[k] < hi[k]):
                miss = True
        if miss or not tmax > tmin:
            continue
        alphas = [np.array([tmin, tmax])]
        for k in range(3):
            if d[k] != 0:
                t = (lo[k] + sp[k] * np.arange(dims[k] + 1) - o[k]) / d[k]
                alphas.append(t[(t > tmin) & (t < tmax)])
        a = np.unique(np.concatenate(alphas))
        mid = 0.5 * (a[:-1] + a[1:])
        length = np.diff(a)
        pos = o[None, :] + d[None, :] * mid[:, None]
        idx = np.clip(np.floor((pos - lo) / sp).astype(np.int64), 0, dims - 1)
        lin = idx[:, 2] * dims[0] * dims[1] + idx[:, 1] * dims[0] + idx[:, 0]
        m = mat[lin]
        mu = np.empty(len(m))
        for u in np.unique(m):
            key = (int(u), float(e))
            if key not in cache:
                cache[key] = float(mu_rho(int(u), float(e)))
            mu[m == u] = cache[key]
        out[r] = 0.1 * float(np.sum(mu * dens[lin] * length))
    return out
