"""Benchmark: photon histories per second on one GB300 for the CT helical workload.

Workload (the configuration the headline metric is quoted on): 120 kVp CT
helical scan (2.5 mm Al, 40 mm collimation, pitch 1, 1 degree steps, heel
effect) over a seeded 512 x 512 x 200 body phantom (0.8 x 0.8 x 2.5 mm voxels,
air / soft tissue / lung / bone), 1e8 histories per step, LIVERMORE model,
FP32 transport with FP64 tallies.

* value: histories/s with world, LUT and source tables resident in HBM; one
  step = one transport job (tally clear + transport kernel), timed with CUDA
  events on the job's stream.  The tallies (1 GB) exceed the 129 MB L2 but the
  compact voxel grid (52 MB) does not, so L2 is flushed (256 MB write) before
  every step, outside the timed events.
* e2e: the same metric through the public API with host buffers: world H2D
  from pinned memory, device max-density scan, host LUT build and upload, job,
  device post-processing and D2H of dose, variance and event counts.
* roofline: algorithmic bytes of the transport kernel per launch,
  5 B per Woodcock step (u8 material + f32 density) + 20 B per deposit
  (FP64 energy + FP64 energy^2 + u32 count), plus 8 B per step for the cell of
  the local-majorant grid when the job tracks with local majorants, from the
  kernel's own step and deposit counters, over the kernel's CUDA-event
  duration, against the measured HBM copy bandwidth.
* cpu_baseline / --impl reference: the oracle port (oracle/port, a C++
  restatement of the reference's Transport<T>, pinned to the reference's own
  tallies on this configuration) in float precision, as Transport<float>, on
  all host cores.  Each step is a fixed sample of the workload: every 10th
  exposure at the workload's histories per exposure (about 1e7 histories),
  with the reference's own exposure, spectrum, heel and LUT tables from the
  golden fixture; the reference arm loads no product library.

Multi-GPU (torchrun, N > 1): every rank runs an independent replica of the job
(histories are independent; no data-path collective), barrier + max over ranks.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parent
sys.path.insert(0, str(REPO))


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(x: float, dist=None, device: str = "cuda") -> float:
    """The largest value over the ranks (the slowest replica's time)."""
    if dist is None:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(ws: int, histories_per_step: int, steps: int, seconds_max: float) -> float:
    """Whole-job throughput of N independent replicas: all ranks' histories over the
    slowest rank's time (weak scaling)."""
    return ws * histories_per_step * steps / seconds_max


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons (every 50 ms, time-stamped by
    nvidia-smi).  Started before the warm-up so that the sampler is running when
    the timed region begins; mark() / done() bracket the timed region, and the
    summary uses the samples inside it (or the nearest one if the region is
    shorter than the interval)."""

    FIELDS = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.samples = []
        self._proc = None
        self.t0 = self.t1 = None

    def __enter__(self):
        try:
            self._proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                           "-lms", "50", "-i", str(self.device)], stdout=subprocess.PIPE,
                                          stderr=subprocess.DEVNULL, text=True)
            self._thread = threading.Thread(target=self._read, daemon=True)
            self._thread.start()
        except Exception:
            self._proc = None
        return self

    def _read(self):
        import datetime
        for line in self._proc.stdout:
            f = [x.strip() for x in line.split(",")]
            try:
                t = datetime.datetime.strptime(f[0], "%Y/%m/%d %H:%M:%S.%f").timestamp()
            except ValueError:
                t = None
            self.samples.append((t, f[1:]))

    def mark(self):
        self.t0 = time.time()

    def done(self):
        self.t1 = time.time()
        time.sleep(0.12)  # let the sample that follows the region arrive

    def __exit__(self, *a):
        if self._proc:
            self._proc.terminate()
            try:
                self._proc.wait(timeout=5)
            except Exception:
                self._proc.kill()

    def summary(self):
        if not self.samples:
            return None
        inside = [f for t, f in self.samples if t is not None and self.t0 is not None and self.t0 - 0.025 <= t <= self.t1 + 0.025]
        if not inside:  # region shorter than the interval: the sample nearest to it
            timed = [(abs(t - 0.5 * (self.t0 + self.t1)), f) for t, f in self.samples if t is not None and self.t0 is not None]
            inside = [min(timed, key=lambda x: x[0])[1]] if timed else [self.samples[-1][1]]
        sm = [float(s[1]) for s in inside if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in inside if s[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for s in inside:
            for i, n in enumerate(names):
                if len(s) > 5 + i and s[5 + i].lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(inside)}


def measured_peaks():
    p = REPO / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def committed_traffic():
    """DRAM bytes per launch of the transport kernel from the committed ncu summary (if any)."""
    p = REPO / "profiles" / "transport_kernel_ct_helical.json"
    if p.exists():
        try:
            return json.loads(p.read_text())
        except Exception:
            return None
    return None


def issue_roofline(profile, histories_per_s: float, clocks, sms: int = 152):
    """The instruction-issue roofline of the transport kernel, the one that binds
    it: warp instructions per history (committed ncu capture) x histories/s
    against one warp instruction per cycle per SM sub-partition (4 per SM) at the
    SM clock sampled during the timed region."""
    if not profile or "warp_instructions_per_history" not in profile:
        return None
    mhz = (clocks or {}).get("sm_mhz") or 2070.0
    peak = sms * 4 * mhz * 1e6
    achieved = profile["warp_instructions_per_history"] * histories_per_s
    return {"achieved": achieved, "peak": peak, "unit": "warp instructions/s", "frac": achieved / peak,
            "warp_instructions_per_history": profile["warp_instructions_per_history"],
            "active_lanes_per_instruction": profile.get("active_lanes_per_instruction"),
            "sm_mhz": mhz}


def build_workload(histories: int):
    from dxmclib_gb300 import workloads
    return workloads.ct_helical(histories=histories)


CT_FIXTURE = REPO / "tests" / "golden" / "bench_ct_helical.npz"
CPU_SAMPLE_STRIDE = 10  # the CPU legs run every 10th exposure of the workload


class CpuWorkload:
    """The CT helical workload as the CPU legs run it, without the product library:
    the seeded phantom (numpy), and the reference's own exposure, spectrum, heel and
    LUT tables for this configuration from the golden fixture the reference
    produced (tests/golden/make_golden.py).  The sample is every
    CPU_SAMPLE_STRIDE-th exposure at the workload's histories per exposure."""

    def __init__(self, histories: int):
        from dxmclib_gb300.workloads import ct_phantom_arrays
        g = dict(np.load(CT_FIXTURE))
        self.dims = tuple(int(x) for x in g["dims"])
        self.spacing = tuple(float(x) for x in g["spacing"])
        mat, dens = ct_phantom_arrays(*self.dims, spacing=self.spacing, seed=int(g["phantom_seed"]))
        self.material, self.density = mat, dens.astype(np.float64)
        ex = g["exposures"].copy()
        self.n_exposures = len(ex)
        self.hpe = -(-int(histories) // self.n_exposures)  # as workloads.ct_source: ceil(histories / exposures)
        ex[:, 17] = self.hpe
        self.sample = ex[::CPU_SAMPLE_STRIDE].copy()
        self.sample_histories = int(self.sample[:, 17].sum())
        self.spectrum = (g["spec_energies"], g["spec_weights"])
        hm = g["heel_meta"]
        self.heel = dict(energy_start=hm[1], energy_step=hm[2], energy_size=hm[3], angle_start=hm[4],
                         angle_step=hm[5], angle_size=hm[6], weights=g["heel_weights"])
        self.g = g
        self.describe = (f"{len(self.sample)} of {self.n_exposures} exposures (every {CPU_SAMPLE_STRIDE}th) x "
                         f"{self.hpe} histories = {self.sample_histories} histories per step; reference exposure, "
                         f"spectrum, heel and LUT tables from tests/golden/bench_ct_helical.npz")

    def run(self, n_threads: int, model: int, precision: str, seed: int = 99):
        """One sample step of the oracle port; returns its transport seconds."""
        sys.path.insert(0, str(REPO / "oracle" / "port"))
        import binding as port
        _, _, _, secs, _ = port.transport(port.lut_from_fixture(self.g), self.dims, self.spacing, self.density,
                                          self.material, self.sample, model=model, n_threads=n_threads, seed=seed,
                                          spectrum=self.spectrum, heel=self.heel, precision=precision)
        return secs


def bench_config(args, n_hist: int, n_exposures: int) -> dict:
    """The `config` object of both arms' JSON lines (identical by construction)."""
    return {"workload": f"ct_helical_512x512x{200}", "histories_per_step": n_hist, "exposures": n_exposures,
            "model": ["NONE", "LIVERMORE", "IA"][args.model], "tally": "fp64",
            "l2": "flushed between steps (256 MB write); 1 GB tallies per step, 52 MB palette grid",
            "parallelism": f"replicas{_dist()[0]}",
            "voxel_layout": "palette-u8" if args.layout == 0 else "8-byte",
            "regen_threshold": args.regen or "default", "interact_threshold": args.interact or "default",
            "woodcock_burst": args.burst or "default", "tracking": args.tracking}


def serving_measurement(ctx, n_jobs: int, rates, chains: int, seconds_per_rate: float = 30.0,
                        seed: int = 20261205) -> dict:
    """Mixed-stream serving (pencil / DX / CT jobs, Poisson arrivals at each rate)
    through DoseServer against the plain one-job-per-call path (Transport: upload
    the world, run one job, copy the result back) on the same jobs and seeds.
    Each rate serves the first min(n_jobs, rate x seconds_per_rate) jobs of the
    stream (at least 20); a saturating burst submits all n_jobs at once, so its
    served rate is the server's capacity rather than the offered load."""
    import queue as _queue
    import threading
    import dxmclib_gb300 as dx
    from dxmclib_gb300.serve import DoseServer
    from dxmclib_gb300.workloads import serving_stream

    def sample(dose):
        # what the client keeps of each result: every 4099th voxel, and the sum over
        # every 257th voxel (one cache line in sixteen), so that reading a result takes
        # well under a millisecond and the client hands the page-locked buffers back
        # as fast as the server fills them
        return dose[::4099].copy(), float(np.sum(dose[::257], dtype=np.float64))

    # results as Result<float> (a Transport<float> caller's): 12 bytes per voxel over the link
    server = DoseServer(ctx, chains=chains, result_dtype=np.float32)
    base = serving_stream(n_jobs=n_jobs, rate_per_s=max(rates), seed=seed)
    # warm-up: one small job per phantom makes every world and LUT resident
    warm = {}
    for j in base:
        warm.setdefault(j.world_key, j)
    for j in warm.values():
        hpe = j.source.historiesPerExposure()
        j.source.setHistoriesPerExposure(max(1, 100_000 // max(1, len(j.source.exposures(j.world.directionCosines())))))
        server.submit(j.world, j.source, seed=1, world_key=j.world_key).result().release()
        j.source.setHistoriesPerExposure(hpe)

    def run_stream(rate, jobs):
        # the same jobs at another arrival rate (the job draws do not depend on the rate);
        # rate None: every job arrives at once
        if rate is None:
            arrivals = np.zeros(len(jobs))
        else:
            arrivals = np.cumsum(np.random.default_rng(seed).exponential(1.0 / rate, len(jobs)))
        server.reset_metrics()
        served = [None] * len(jobs)
        done_q = _queue.Queue()

        def consumer():  # the client reads a sample of every result, then hands the buffers back
            while True:
                item = done_q.get()
                if item is None:
                    return
                i, fut = item
                r = fut.result()
                served[i] = sample(r.dose)
                r.release()

        reader = threading.Thread(target=consumer, daemon=True)
        reader.start()
        t0 = time.perf_counter()
        for i, j in enumerate(jobs):
            delay = arrivals[i] - (time.perf_counter() - t0)
            if delay > 0:
                time.sleep(delay)
            fut = server.submit(j.world, j.source, seed=j.seed, world_key=j.world_key)
            fut.add_done_callback(lambda f, i=i: done_q.put((i, f)))
        server.drain()
        m = server.metrics()
        done_q.put(None)
        reader.join()
        return m, served

    def line(rate, n, m):
        return {"rate_jobs_per_s": rate, "jobs": n, "served_histories_per_s": m["histories_per_s"],
                "p50_ms": m["p50_ms"], "p99_ms": m["p99_ms"], "mean_queue_ms": m["mean_queue_ms"],
                "batches": m["batches"], "mean_batch_jobs": m["mean_batch_jobs"]}

    sweep = []
    for rate in sorted(rates):
        n = min(len(base), max(20, int(math.ceil(rate * seconds_per_rate))))
        m, _ = run_stream(rate, base[:n])
        sweep.append(line(rate, n, m))
    m, served = run_stream(None, base)
    saturation = line("burst", len(base), m)
    server.close()

    # plain: one Transport call per job, back to back (no arrival gaps)
    tr = dx.Transport(ctx)
    tr.setOutputMode(dx.Transport.EV_PER_HISTORY)
    plain_s = 0.0
    worst = 0.0
    for i, j in enumerate(base):
        tr.setSeed(j.seed)
        t = time.perf_counter()
        res = tr(j.world, j.source)
        plain_s += time.perf_counter() - t
        ps, ptot = sample(res.dose)
        ss, stot = served[i]
        scale = max(float(np.abs(ps).max()), 1e-300)
        worst = max(worst, float(np.abs(ss - ps).max()) / scale, abs(stot - ptot) / max(abs(ptot), 1e-300))
    # plain with resident data: worlds and LUTs uploaded once, then one job per launch,
    # back to back, each result copied to the host before the next job starts
    from dxmclib_gb300 import _capi as A
    resident = {}
    for j in base:
        if j.world_key not in resident:
            dw = dx.DeviceWorld(ctx, j.world)
            resident[j.world_key] = (dw, dw.max_density())
    luts = {}
    t = time.perf_counter()
    for j in base:
        dw, md = resident[j.world_key]
        src = j.source
        key = (j.world_key, float(src.maxPhotonEnergyProduced()))
        if key not in luts:
            luts[key] = dx.DeviceLut(ctx, dx.LutBlob.cached(j.world.materialMap(), md, src.maxPhotonEnergyProduced()))
        job = dx.Job(ctx, dw, luts[key], src.exposures(j.world.directionCosines()), src.spectrum(), src.heel(),
                     src.bowtie(), seed=j.seed, model=1)
        job.result(A.OUTPUT_EV_PER_HISTORY)
        job.close()
    resident_s = time.perf_counter() - t
    for dl in luts.values():
        dl.close()
    for dw, _ in resident.values():
        dw.close()
    hist = int(sum(j.histories for j in base))
    kinds = {k: sum(1 for j in base if j.kind == k) for k in ("pencil", "dx", "ct")}
    plain = hist / plain_s
    return {"workload": "mixed stream: 40% pencil 64^3, 40% DX 128^3-256^3, 20% CT 512x512x(100-400); "
                        "histories log-uniform 1e6-1e8; seeded phantom pool",
            "jobs": len(base), "kinds": kinds, "histories": hist, "chains": chains,
            "seconds_per_rate": seconds_per_rate,
            "saturation": saturation,
            "served_histories_per_s": saturation["served_histories_per_s"], "plain_histories_per_s": plain,
            "served_over_plain": saturation["served_histories_per_s"] / plain,
            "plain_resident_histories_per_s": hist / resident_s,
            "served_over_plain_resident": saturation["served_histories_per_s"] / (hist / resident_s),
            "p50_ms": saturation["p50_ms"], "p99_ms": saturation["p99_ms"], "sweep": sweep,
            "max_rel_dose_diff_vs_plain": worst}


def layout8_measurement(ctx, src, model: int, steps: int = 3, seed: int = 20261206) -> dict:
    """The CT helical job on the same phantom with continuous per-voxel densities
    (each voxel's density times a seeded factor uniform in [0.95, 1.05]), as a
    CT-derived phantom has them: far more than 256 distinct voxels, so the world
    takes the 8-byte voxel layout (f32 density, u8 material, u8 measurement)."""
    import dxmclib_gb300 as dx
    from dxmclib_gb300 import _capi as A
    from dxmclib_gb300.workloads import ct_world
    w = ct_world(200)
    dens = (w.densityArray() * np.random.default_rng(seed).uniform(0.95, 1.05, w.size())).astype(np.float32)
    w.setDensityArray(dens)
    # (the densities alone rule out the palette; layout 1 states it)
    dw = dx.DeviceWorld(ctx, w, layout=1)
    dl = dx.DeviceLut(ctx, dx.LutBlob(w.materialMap(), dw.max_density(), src.maxPhotonEnergyProduced()))
    ex = src.exposures(w.directionCosines())
    n_hist = int(np.sum(ex.n_histories))
    ms, st = [], None
    for k in range(steps + 1):
        job = dx.Job(ctx, dw, dl, ex, src.spectrum(), src.heel(), None, seed=500 + k, model=model)
        job.wait()
        s = A.JobStats()
        A.check(ctx.lib.dxmc_gpu_job_result(job.handle, A.OUTPUT_RAW, 1.0, None, None, None, dx.api.C.byref(s)),
                ctx.handle, "job_result")
        job.close()
        if k:
            ms.append(s.kernel_ms)
            st = s
    out = {"workload": "ct_helical_512x512x200 with continuous densities (x U[0.95, 1.05] per voxel)",
           "voxel_layout": "8-byte", "distinct_densities": int(np.unique(dens).size),
           "histories_per_s": n_hist / (float(np.mean(ms)) / 1e3), "kernel_ms": float(np.mean(ms)),
           "steps_per_history": st.steps / n_hist, "deposits_per_history": st.deposits / n_hist}
    dl.close()
    dw.close()
    return out


def siddon_measurement(ctx, dworld, dlut, world, n_rays: int = 1 << 20, seed: int = 5) -> dict:
    """Siddon traversal throughput: rays from the 1 m source circle through random
    points of the resident CT grid (a projection-like pattern), 40-120 keV."""
    rng = np.random.default_rng(seed)
    ext = np.array(world.matrixExtent()).reshape(3, 2)
    lo, hi = ext[:, 0], ext[:, 1]
    ang = rng.uniform(0, 2 * np.pi, n_rays)
    src = np.stack([500 * np.cos(ang), 500 * np.sin(ang), rng.uniform(lo[2], hi[2], n_rays)], 1)
    tgt = rng.uniform(lo, hi, (n_rays, 3))
    rays = np.concatenate([src, tgt - src, rng.uniform(40, 120, (n_rays, 1))], 1).astype(np.float32)
    dworld.radiological_path(dlut, rays[:1024])
    t = time.perf_counter()
    out = dworld.radiological_path(dlut, rays)
    wall = time.perf_counter() - t
    return {"rays": n_rays, "rays_per_s_e2e": n_rays / wall, "mean_path": float(out.mean()),
            "note": "host rays in, host results out (28 B + 8 B per ray over the link)"}


def batch_measurement(ctx, n_jobs: int = 64, seed: int = 20261204) -> dict:
    """Batched projection radiography: the uneven DX jobs one job per launch
    (resident worlds and LUTs, default launch parameters) against one batch with
    per-class launch parameters and the chain count chosen by the autotuner."""
    import dxmclib_gb300 as dx
    from dxmclib_gb300 import _capi as A
    from dxmclib_gb300.autotune import Autotuner
    from dxmclib_gb300.workloads import dx_batch

    jobs = dx_batch(n_jobs=n_jobs, seed=seed)
    prepared = []
    for k, wl in enumerate(jobs):
        src = wl.source
        src.updateFromWorld(wl.world)
        src.validate()
        dw = dx.DeviceWorld(ctx, wl.world)
        dl = dx.DeviceLut(ctx, dx.LutBlob.cached(wl.world.materialMap(), dw.max_density(), src.maxPhotonEnergyProduced()))
        prepared.append((wl, dw, dl, src.exposures(wl.world.directionCosines()), src.spectrum(), src.heel(), 100 + k))
    hist = int(sum(np.sum(p[3].n_histories) for p in prepared))
    tuner = Autotuner(ctx, sample_histories=2_000_000, repeats=1, rounds=1)
    launches = []
    for wl, dw, dl, ex, spec, heel, sd in prepared:
        r = tuner.tune_job(wl.world, dw, dl, ex, spec, heel, None, 1, wl.source.maxPhotonEnergyProduced())
        launches.append(r["launch"])

    def plain():
        ms = 0.0
        t = time.perf_counter()
        for wl, dw, dl, ex, spec, heel, sd in prepared:
            job = dx.Job(ctx, dw, dl, ex, spec, heel, None, seed=sd, model=1)
            job.wait()
            st = A.JobStats()
            A.check(ctx.lib.dxmc_gpu_job_result(job.handle, A.OUTPUT_RAW, 1.0, None, None, None, dx.api.C.byref(st)),
                    ctx.handle, "job_result")
            ms += st.job_ms
            job.close()
        return ms, (time.perf_counter() - t) * 1e3

    def entries():
        return [dx.BatchEntry(dw, dl, ex, spec, heel, None, sd, 1, -1, launch)
                for (wl, dw, dl, ex, spec, heel, sd), launch in zip(prepared, launches)]

    chains = tuner.tune_chains(entries(), f"dx_batch_{n_jobs}")

    def batched(mode, c):
        t = time.perf_counter()
        b = dx.Batch(ctx, entries(), mode=mode, chains=c)
        b.wait()
        ms = b.kernel_ms()
        b.close()
        return ms, (time.perf_counter() - t) * 1e3

    plain()
    batched(A.BATCH_CONCURRENT, chains["chains"])
    p_ms, p_wall = plain()
    b_ms, b_wall = batched(A.BATCH_CONCURRENT, chains["chains"])
    batched(A.BATCH_PERSISTENT, 0)
    pers_ms, _ = batched(A.BATCH_PERSISTENT, 0)
    for wl, dw, dl, *_ in prepared:
        dl.close()
        dw.close()
    classes = {k: v for k, v in tuner.cache.items() if k.startswith("job|")}
    return {"workload": f"{n_jobs} DX jobs, grids 64^3-256^3, 70-90 kVp, 1e6-1e7 histories (seed {seed})",
            "histories": hist,
            "plain_histories_per_s": hist / (p_ms / 1e3), "plain_wall_histories_per_s": hist / (p_wall / 1e3),
            "batched_histories_per_s": hist / (b_ms / 1e3), "batched_wall_histories_per_s": hist / (b_wall / 1e3),
            "persistent_histories_per_s": hist / (pers_ms / 1e3),
            "chains": chains["chains"], "chain_ms": chains["ms"],
            "tuned_classes": {k: {"launch": v["launch"], "speedup": round(v["speedup"], 3)} for k, v in classes.items()}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--histories", type=float, default=1e8)
    ap.add_argument("--model", type=int, default=1)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-precision", choices=("float", "both"), default="float",
                    help="reference arm: time the port in float only, or in float and then double")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end leg (profiling runs)")
    ap.add_argument("--regen", type=int, default=0, help="warp refill threshold (0 = library default)")
    ap.add_argument("--interact", type=int, default=0, help="interaction-pass threshold (0 = library default)")
    ap.add_argument("--layout", type=int, default=0, help="0 = compact palette when possible, 1 = 8-byte voxels")
    ap.add_argument("--block-size", type=int, default=0)
    ap.add_argument("--blocks-per-sm", type=int, default=0)
    ap.add_argument("--queue-log2", type=int, default=0, help="photon queue chunk 2^n (0 = default: in-kernel generation)")
    ap.add_argument("--burst", type=int, default=0, help="Woodcock steps per loop iteration (0 = library default)")
    ap.add_argument("--tracking", choices=("local", "global"), default="local",
                    help="Woodcock majorant: local grid (default) or the reference's global majorant")
    ap.add_argument("--no-serve", action="store_true", help="skip the served-vs-plain mixed-stream leg")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched DX leg")
    ap.add_argument("--no-precision", action="store_true", help="skip the tally-precision study")
    ap.add_argument("--no-siddon", action="store_true", help="skip the Siddon traversal leg")
    ap.add_argument("--no-layout8", action="store_true", help="skip the 8-byte voxel layout leg")
    ap.add_argument("--precision-histories", type=float, default=1e9)
    ap.add_argument("--precision-slices", type=int, default=400)
    ap.add_argument("--batch-jobs", type=int, default=64)
    ap.add_argument("--serve-jobs", type=int, default=500)
    ap.add_argument("--serve-rates", default="1,10,25,100,200", help="Poisson arrival rates of the mixed stream (jobs/s)")
    ap.add_argument("--serve-seconds", type=float, default=30.0,
                    help="each rate serves at most rate x this many jobs of the stream")
    ap.add_argument("--serve-chains", type=int, default=4)
    args = ap.parse_args()
    ws, rank, local = _dist()
    metric = "histories/s"
    histories = int(args.histories)

    if args.impl == "reference":
        # the reference's CPU transport (the oracle port, a C++ restatement of DXMClib's
        # Transport<T>, in float as Transport<float>) on all host cores; no product code
        if rank != 0:
            return
        cw = CpuWorkload(histories)
        # the cores this process may run on (a container or cgroup may offer fewer
        # than the machine has), and the share of them the transport got: the
        # process's CPU seconds, less the single-threaded set-up around the port's
        # timed transport, over the transport's seconds x cores (about 1 when no
        # other work shared the cores)
        import resource
        threads = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)
        secs, secs64, share = [], [], []
        for step in range(args.warmup + args.steps):
            r0, w0 = resource.getrusage(resource.RUSAGE_SELF), time.perf_counter()
            t = cw.run(threads, args.model, "float", seed=100 + step)
            r1, w1 = resource.getrusage(resource.RUSAGE_SELF), time.perf_counter()
            if step >= args.warmup:
                secs.append(t)
                cpu_s = (r1.ru_utime - r0.ru_utime) + (r1.ru_stime - r0.ru_stime) - max((w1 - w0) - t, 0.0)
                share.append(round(cpu_s / max(t * threads, 1e-9), 3))
        if args.cpu_precision == "both":  # Transport<double> beside the fair float baseline
            for step in range(args.warmup + args.steps):
                t = cw.run(threads, args.model, "double", seed=200 + step)
                if step >= args.warmup:
                    secs64.append(t)
        v = cw.sample_histories * len(secs) / float(np.sum(secs))
        n_hist = cw.hpe * cw.n_exposures
        line = {"metric": metric, "value": v, "unit": "histories/s", "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": 1e3 * float(np.mean(secs)), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": bench_config(args, n_hist, cw.n_exposures),
                "impl": "reference", "histories_per_sample_step": cw.sample_histories,
                "cpu_baseline": {"value": v, "unit": "histories/s", "cores": threads, "kind": "port",
                                 "precision": "float", "sample": cw.describe,
                                 "double_value": (cw.sample_histories * len(secs64) / float(np.sum(secs64))
                                                  if secs64 else None),
                                 "sample_seconds": [round(t, 3) for t in secs],
                                 "double_sample_seconds": [round(t, 3) for t in secs64],
                                 "core_share": share},
                "e2e": {"value": v, "unit": "histories/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        # the CPU baseline runs first, in a fresh process of the reference arm's own code
        # (no CUDA context, no threads of this process competing for the host cores):
        # one warm-up and two timed fixed-sample steps in float, then the same in double
        r = subprocess.run([sys.executable, str(REPO / "bench.py"), "--impl", "reference", "--steps", "2", "--warmup",
                            "1", "--cpu-precision", "both", "--model", str(args.model),
                            "--histories", str(args.histories)], capture_output=True, text=True)
        lines = [x for x in r.stdout.splitlines() if x.startswith("{")]
        cpu = json.loads(lines[-1])["cpu_baseline"] if r.returncode == 0 and lines else {"error": r.stderr[-500:]}

    import torch
    import dxmclib_gb300 as dx
    from dxmclib_gb300 import _capi as A
    from dxmclib_gb300 import build as b
    b.build()
    device = local if ws > 1 else 0
    torch.cuda.set_device(device)
    dist = None
    if ws > 1:
        import torch.distributed as tdist
        tdist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
        dist = tdist

    wl = build_workload(histories)
    world, src = wl.world, wl.source
    tracking = A.TRACKING_LOCAL if args.tracking == "local" else A.TRACKING_GLOBAL
    ctx = dx.GpuContext(device=device, block_size=args.block_size, blocks_per_sm=args.blocks_per_sm,
                        regen_threshold=args.regen, interact_threshold=args.interact, queue_log2_chunk=args.queue_log2,
                        tracking=tracking)
    dworld = dx.DeviceWorld(ctx, world, layout=args.layout)
    md = dworld.max_density()
    blob = dx.LutBlob(world.materialMap(), md, src.maxPhotonEnergyProduced())
    dlut = dx.DeviceLut(ctx, blob)
    exposures = src.exposures(world.directionCosines())
    spec, heel = src.spectrum(), src.heel()
    n_hist = int(np.sum(exposures.n_histories))

    def barrier():
        torch.cuda.synchronize()
        if dist:
            dist.barrier()

    def run_job(seed):
        job = dx.Job(ctx, dworld, dlut, exposures, spec, heel, None, seed=seed, model=args.model,
                     launch={"woodcock_burst": args.burst} if args.burst else None)
        job.wait()
        st = dx.api.A.JobStats()
        A.check(ctx.lib.dxmc_gpu_job_result(job.handle, A.OUTPUT_RAW, 1.0, None, None, None, dx.api.C.byref(st)),
                ctx.handle, "job_result")
        job.close()
        return st

    # the compact voxel grid (1 byte per voxel) fits in L2, so L2 is flushed between
    # steps by writing a buffer larger than it (outside the jobs' timed events)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def flush_l2():
        flush.fill_(1)
        torch.cuda.synchronize()

    with ClockSampler(device) as clocks:
        for w in range(args.warmup):
            flush_l2()
            run_job(1000 + w)
        barrier()
        clocks.mark()
        stats = []
        for step in range(args.steps):
            flush_l2()
            stats.append(run_job(2000 + step))
        barrier()
        clocks.done()
    job_ms = np.array([s.job_ms for s in stats])
    kern_ms = np.array([s.kernel_ms for s in stats])
    total_ms = max_over_ranks(float(job_ms.sum()), dist)
    value = replica_throughput(ws, n_hist, args.steps, total_ms / 1e3)
    steps_per_hist = float(np.mean([s.steps for s in stats])) / n_hist
    deps_per_hist = float(np.mean([s.deposits for s in stats])) / n_hist
    # algorithmic bytes per launch: 5 B per Woodcock step inside the grid (u8 material +
    # f32 density) and 20 B per deposit (FP64 energy, FP64 energy^2, u32 count); the
    # local-majorant grid adds an 8-byte cell per step, reported beside it
    mean_steps = float(np.mean([s.steps for s in stats]))
    mean_deps = float(np.mean([s.deposits for s in stats]))
    alg_bytes = 5.0 * mean_steps + 20.0 * mean_deps
    alg_bytes_cells = alg_bytes + (8.0 * mean_steps if tracking == A.TRACKING_LOCAL else 0.0)
    kernel_s = float(kern_ms.mean()) / 1e3
    achieved = alg_bytes / kernel_s / 1e9
    peak, peak_kind = measured_peaks()
    traffic = committed_traffic()

    # ---- e2e through the public API with pinned host buffers -------------------------
    n_vox = world.size()
    pin_d = torch.empty(n_vox, dtype=torch.float32, pin_memory=True)
    pin_m = torch.empty(n_vox, dtype=torch.uint8, pin_memory=True)
    pin_d.numpy()[:] = world.densityArray()
    pin_m.numpy()[:] = world.materialIndexArray()
    e2e_world = dx.World()
    e2e_world.setDimensions(world.dimensions())
    e2e_world.setSpacing(world.spacing())
    e2e_world.setDensityArray(pin_d.numpy())
    e2e_world.setMaterialIndexArray(pin_m.numpy())
    for m in world.materialMap():
        e2e_world.addMaterialToMap(m)
    assert e2e_world.isValid()
    # results as a Transport<float> caller receives them (Result<float>: float dose and
    # variance, u32 counts = 12 B per voxel), into two page-locked buffer sets so that
    # job k's result copies run on the copy engine while job k + 1 is transported
    def pinned_result():
        return (torch.empty(n_vox, dtype=torch.float32, pin_memory=True).numpy(),
                torch.empty(n_vox, dtype=torch.float32, pin_memory=True).numpy(),
                torch.empty(n_vox, dtype=torch.int32, pin_memory=True).numpy().view(np.uint32))
    out_bufs = [pinned_result(), pinned_result()]
    e2e_steps = max(1, min(args.steps, 5))

    def e2e_submit(seed, buf):
        # the source's host tables first: they are built while the previous job runs,
        # the world upload then waits for its kernel to leave the SMs
        ex = src.exposures(e2e_world.directionCosines())
        spectrum, heel = src.spectrum(), src.heel()
        dw = dx.DeviceWorld(ctx, e2e_world, layout=args.layout)
        bl = dx.LutBlob.cached(e2e_world.materialMap(), dw.max_density(), src.maxPhotonEnergyProduced())
        dl = dx.DeviceLut(ctx, bl)
        job = dx.Job(ctx, dw, dl, ex, spectrum, heel, None, seed=seed, model=args.model)
        job.result_async(A.OUTPUT_EV_PER_HISTORY, out=buf, dtype=np.float32)
        return job, dl, dw

    def e2e_finish(handle):
        job, dl, dw = handle
        job.result_wait()
        job.close()
        dl.close()
        dw.close()

    if args.no_e2e:
        e2e_steps = 0
        e2e_s = float("nan")
    else:
        e2e_finish(e2e_submit(1, out_bufs[0]))
        barrier()
        t0 = time.perf_counter()
        pending = None
        for step in range(e2e_steps):
            h = e2e_submit(3000 + step, out_bufs[step % 2])
            if pending is not None:
                e2e_finish(pending)
            pending = h
        e2e_finish(pending)
        barrier()
        e2e_s = time.perf_counter() - t0
    e2e_s = max_over_ranks(e2e_s, dist)
    e2e_value = replica_throughput(ws, n_hist, e2e_steps, e2e_s) if e2e_steps else None
    h2d = n_vox * 5 + len(exposures) * 80
    d2h = n_vox * (4 + 4 + 4)

    layout8 = None
    if rank == 0 and not args.no_layout8:
        layout8 = layout8_measurement(ctx, src, args.model)

    siddon = None
    if rank == 0 and not args.no_siddon:
        siddon = siddon_measurement(ctx, dworld, dlut, world)

    precision = None
    if rank == 0 and not args.no_precision:
        from dxmclib_gb300 import precision as prec
        from dxmclib_gb300.workloads import ct_helical
        pw = ct_helical(nz=args.precision_slices, histories=int(args.precision_histories))
        precision = {"workload": pw.name, **prec.study(ctx, pw.world, pw.source, repeats=1)}

    batching = None
    if rank == 0 and not args.no_batch:
        batching = batch_measurement(ctx, args.batch_jobs)

    serving = None
    if rank == 0 and not args.no_serve:
        serving = serving_measurement(ctx, args.serve_jobs, [float(r) for r in args.serve_rates.split(",")],
                                      args.serve_chains, args.serve_seconds)


    if rank == 0:
        line = {
            "metric": metric, "value": value, "unit": "histories/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": bench_config(args, n_hist, len(exposures)),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "peak_kind": peak_kind,
                         # DRAM bytes per launch from the committed ncu capture of a 1e7-history
                         # launch, scaled by histories (traffic grows in proportion)
                         "traffic": None if not traffic else traffic["dram_bytes_per_history"] * n_hist,
                         "algorithmic_bytes_per_launch": alg_bytes, "kernel_ms": float(kern_ms.mean()),
                         "steps_per_history": steps_per_hist, "deposits_per_history": deps_per_hist,
                         "bytes_formula": "5 B x steps + 20 B x deposits",
                         "with_majorant_cells": {"bytes_per_launch": alg_bytes_cells,
                                                 "achieved": alg_bytes_cells / kernel_s / 1e9,
                                                 "frac": alg_bytes_cells / kernel_s / 1e9 / peak},
                         "issue": issue_roofline(traffic, n_hist / kernel_s, clocks.summary())},
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": "histories/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "steps": e2e_steps},
            # per step: the transport kernel, or one generation pass and one transport launch per queue chunk
            "gpu_launches": args.steps * (1 if args.queue_log2 <= 0 else 2 * max(1, -(-n_hist // (1 << args.queue_log2)))),
            "clocks": clocks.summary(),
            "batching": batching,
            "precision": precision,
            "siddon": siddon,
            "layout_8byte": layout8,
            "serving": serving,
        }
        print(json.dumps(line), flush=True)
    dlut.close()
    dworld.close()
    ctx.close()
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
