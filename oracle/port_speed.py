"""ORACLE TEST INFRASTRUCTURE — speed of the oracle port against the reference.

bench.py's CPU legs time the oracle port (oracle/port), because the reference
(oracle/_ref, DXMClib's headers compiled here) cannot be built where the GPU
tests run.  This script times both on the same machine, workload and thread
count so that the port's number can be converted into the reference's: the
headline CT helical workload (512 x 512 x 200 seeded phantom, 120 kVp helical
scan, every exposure of it) at a reduced number of histories per exposure,
Transport<float> and Transport<double> against the port in float and double,
interleaved over several rounds (this machine's speed drifts) with the median
kept.  The time compared is the transport alone: Result::simulationTime for
the reference (transport.hpp:166-174), the port's own timer likewise.

Usage: make -C oracle REF=<reference checkout> && python oracle/port_speed.py [--rounds 3] [--hpe 1111]
"""
from __future__ import annotations

import argparse
import json
import os
import sys
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(REPO))
sys.path.insert(0, str(REPO / "tests" / "golden"))
sys.path.insert(0, str(REPO / "oracle" / "port"))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--rounds", type=int, default=3)
    ap.add_argument("--hpe", type=int, default=1111, help="histories per exposure (4500 exposures)")
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    a = ap.parse_args()
    import binding as port
    import ref_binding as R
    from dxmclib_gb300.workloads import CT_MATERIALS, ct_phantom_arrays
    g = dict(np.load(REPO / "tests" / "golden" / "bench_ct_helical.npz"))
    dims, spacing = tuple(int(x) for x in g["dims"]), tuple(float(x) for x in g["spacing"])
    mat, dens = ct_phantom_arrays(*dims, spacing=spacing, seed=int(g["phantom_seed"]))
    dens = dens.astype(np.float64)
    names = [n for n, _ in CT_MATERIALS]
    w = R.WorldArgs(dims, spacing, dens, mat, names, material_densities=[d for _, d in CT_MATERIALS])
    length = dims[2] * spacing[2]
    s = R.SourceArgs(R.CTSPIRAL, position=(0, 0, -length / 2), kvp=120, al_mm=2.5, ct_collimation=40, pitch=1.0,
                     scan_length=length, angle_step_deg=1.0, start_angle_deg=0, fov=500, sdd=1190, heel=1,
                     histories_per_exposure=a.hpe)
    ex = g["exposures"].copy()
    ex[:, 17] = a.hpe
    n = int(ex[:, 17].sum())
    hm = g["heel_meta"]
    heel = dict(energy_start=hm[1], energy_step=hm[2], energy_size=hm[3], angle_start=hm[4], angle_step=hm[5],
                angle_size=hm[6], weights=g["heel_weights"])
    lut = port.lut_from_fixture(g)
    rates = {k: [] for k in ("reference_float", "reference_double", "port_float", "port_double")}
    for r in range(a.rounds):
        for prec, code in (("float", 1), ("double", 0)):
            _, _, _, N, secs, _ = R.transport_ex(w, s, model=1, n_threads=a.threads, precision=code)
            assert N == n, (N, n)
            rates[f"reference_{prec}"].append(N / secs)
            _, _, _, secs, _ = port.transport(lut, dims, spacing, dens, mat, ex, model=1, n_threads=a.threads,
                                              seed=11 + r, spectrum=(g["spec_energies"], g["spec_weights"]),
                                              heel=heel, precision=prec)
            rates[f"port_{prec}"].append(n / secs)
        print(json.dumps({k: v[-1] for k, v in rates.items()}), flush=True)
    med = {k: float(np.median(v)) for k, v in rates.items()}
    out = {"histories": n, "threads": a.threads, "rounds": a.rounds, "median_histories_per_s": med,
           "port_over_reference_float": med["port_float"] / med["reference_float"],
           "port_over_reference_double": med["port_double"] / med["reference_double"], "all": rates}
    print(json.dumps(out))


if __name__ == "__main__":
    main()
