"""Benchmark: batched DC3D0 Green's-function build (GF entries/s) on the
16x8-patch, 5x5-Gauss-point, 400-station workload, plus the nested-SMC
throughput when the inner sampler is available.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Prints one JSON line (rank 0).  The reference arm times the CPU restatement of
the reference path (oracle/) on all host cores.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "GF entries/sec (batched DC3D0 Green's build); nested-SMC outer particles/sec reported alongside"
UNIT = "GF entries/s"
# Algorithmic FP64 operations per unique (theta, patch, Gauss point, station)
# evaluation of the displacement-only DC3D0 for both slip directions
# (fault-frame offsets 7, UB0 displacement terms 75 incl. 1 sqrt + 2 div,
# quadrature weight and 6 accumulations 15), counted from greens.cu's
# dc3d0 displacement terms.
FLOPS_PER_EVAL = 97


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--n-theta", type=int, default=8192)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-nested", action="store_true")
    p.add_argument("--no-c2", action="store_true", help="skip the c2 (D = 256) nested measurements")
    p.add_argument("--no-c3", action="store_true", help="skip the c3 (per-geometry meshes) nested sample")
    p.add_argument("--no-c4", action="store_true", help="skip the c4 (D = 1024) nested sample")
    p.add_argument("--c4-full", action="store_true", help="c4: full nested evaluations (about 7.5 minutes)")
    p.add_argument("--fp64-stages", type=int, default=3, help="c0 outer stages timed in FP64")
    p.add_argument("--equal-error-study", type=str, default=None, metavar="OUT_JSON",
                   help="instead of the benchmark: full c0 outer-SMC runs over several seeds in MIXED and FP64 "
                        "(posterior mean / std of every geometry parameter and the evidence), written to OUT_JSON")
    p.add_argument("--study-seeds", type=str, default="8,3", help="MIXED,FP64 seeds of the equal-error study")
    p.add_argument("--study-seed0", type=str, default="1000,1000",
                   help="equal-error study: MIXED,FP64 seed offsets (seeds are offset + 1, offset + 2, ...)")
    p.add_argument("--equal-error-points", type=str, default=None, metavar="THETAS",
                   help="c0: -log Z in MIXED and FP64 over 512 streams at the given geometries "
                        "('x,y,top,length,width,strike,dip,log_alpha2;...')")
    p.add_argument("--study-no-evidence", action="store_true",
                   help="equal-error study: only the outer-SMC runs (no 512-stream evidence comparison)")
    return p.parse_args()


_T0 = time.perf_counter()
PEAKS = {}   # MEASURED_PEAKS.json, loaded by the GPU arm


def log(msg: str) -> None:
    """Progress on stderr (the JSON line alone goes to stdout)."""
    print(f"[bench {time.perf_counter() - _T0:7.1f} s] {msg}", file=sys.stderr, flush=True)


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def max_over_ranks(x, world, device):
    """The job's time of a per-rank time: the maximum over the ranks (one
    all_reduce MAX on the job's process group); x itself on one rank."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as tdist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
    return float(t.item())


def workload(n_theta):
    from smc_inversion_fort_gb300.configs import make_stations, preset, random_thetas
    w = preset("c1")
    obs = make_stations(w, np.random.default_rng(2024))
    obs["dvec"] = np.zeros(len(obs["obs_sigma"]))
    th = random_thetas(w, n_theta, seed=7)
    return w, obs, th


def c1_config(n_theta, nobs, D):
    return {"workload": "c1: 8192 geometries x 16x8 patches x 5x5 Gauss points x 400 stations (3-comp), "
                        "patch-constant basis, FP64",
            "n_theta": n_theta, "nobs": nobs, "D": D, "entries_per_step": n_theta * nobs * D,
            "l2": "output 20.1 GB per step, larger than L2; no flush needed"}


def cpu_greens_rate(w, obs, th, target_s=15.0, max_theta=512):
    """Oracle (timing build) Green's build on all host threads over a bounded
    sample of the geometries; returns the rate and the sample's wall time."""
    from oracle import pyoracle
    pyoracle.build()
    o = pyoracle.Oracle(w.settings, obs)
    nthreads = os.cpu_count() or 1
    t0 = time.perf_counter()
    o.greens_batch(th[:nthreads], nthreads=nthreads)
    t1 = time.perf_counter() - t0
    n = int(min(max_theta, max(nthreads, nthreads * round(target_s / max(t1, 1e-3)))))
    n = min(n, len(th))
    t0 = time.perf_counter()
    o.greens_batch(th[:n], nthreads=nthreads)
    dt = time.perf_counter() - t0
    D, nobs = o.dims["D"], o.nobs
    return {"value": n * nobs * D / dt, "unit": UNIT, "cores": nthreads, "kind": "port",
            "sample": f"{n} of {len(th)} geometries, full 1200x256 matrices, {dt:.1f} s wall (oracle timing "
                      f"build, -O3)", "wall_s": dt}


def reference_arm(args):
    """The CPU restatement of the reference path (oracle/, -O3 timing build)
    on every host thread: a step is a bounded sample of the c1 workload (the
    same geometries as the GPU arm's step), its value the sample's entries
    over its wall time."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from oracle import pyoracle
    pyoracle.use_timing_build()
    w, obs, th = workload(args.n_theta)
    vals, walls = [], []
    cb = None
    for k in range(args.warmup + args.steps):
        r = cpu_greens_rate(w, obs, th, target_s=8.0 if k >= args.warmup else 2.0, max_theta=256)
        if k >= args.warmup:
            vals.append(r["value"])
            walls.append(r["wall_s"])
            cb = r
    v = statistics.median(vals)
    D = w.settings.dims()["D"]
    nobs = 3 * 400
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": statistics.mean(walls) * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded stations, prior-box "
            "geometries)", "impl": "reference",
            "config": c1_config(args.n_theta, nobs, D),
            "step": "a bounded sample of the workload's geometries per step (ms_per_step is its measured wall time)",
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cb["cores"], "kind": "port", "sample": cb["sample"]},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


class ClockSampler:
    def __init__(self, index):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={index}", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        self.p.wait()
        self.f.flush()
        self.f.seek(0)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f.read().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.f.name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak_fp64_tflops(torch, dev):
    """FP64 throughput of cuBLAS DGEMM on this GPU (the FP64 ceiling)."""
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device=dev)
    b = torch.randn(n, n, dtype=torch.float64, device=dev)
    for _ in range(2):
        a @ b
    torch.cuda.synchronize()
    best = 1e9
    for _ in range(3):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        a @ b
        e.record()
        e.synchronize()
        best = min(best, s.elapsed_time(e))
    return 2.0 * n ** 3 / (best * 1e-3) / 1e12


def load_traffic():
    p = os.path.join(ROOT, "profiles", "greens_c1_traffic.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)
    return None


def nested_workload(pkg, name="c0", seed=2024):
    """Seeded observations of a named workload, data from its known fault
    (the GPU Green's build of the true geometry plus Gaussian noise)."""
    from smc_inversion_fort_gb300.configs import fixed_mesh, make_stations, preset, prior_range, true_slip, true_theta
    w = preset(name)
    rng = np.random.default_rng(seed)
    obs = make_stations(w, rng)
    obs["dvec"] = np.zeros(len(obs["obs_sigma"]))
    wf = fixed_mesh(w, true_theta(w))   # the true geometry's own mesh (per-geometry meshes)
    g = pkg.SmcGpu(wf.settings)
    g.set_data(obs)
    G = g.calc_greens_func(true_theta(w)[None])[0]
    g.close()
    obs["dvec"] = G.T @ true_slip(wf) + rng.standard_normal(G.shape[1]) * obs["obs_sigma"]
    return w, obs, prior_range(w), true_theta(w), true_slip(wf)


def inner_roofline(st, ntau, D, peak, peak_name):
    """Algorithmic flops of the inner SMC kernel over a run: every HMC
    trajectory (tuning and sampling) takes ntau + 1 Gram-matrix products
    M x (2 D^2 each) and one A x for its end-point energy (2 D^2), the Gram
    form of slip_calc_grad / slip_calc_likelihood (smc_slip.f90:56-182)."""
    flops = st["inner_trajectories"] * (ntau + 2) * 2.0 * D * D
    ach = flops / (st["inner_kernel_ms"] * 1e-3) / 1e12 if st["inner_kernel_ms"] > 0 else 0.0
    return {"bound": "tensor" if "bf16" in peak_name else "fp64", "achieved": ach, "peak": peak,
            "unit": "TFLOP/s", "frac": ach / peak if peak else None, "peak_source": peak_name,
            "flops_per_trajectory": (ntau + 2) * 2 * D * D, "trajectories": st["inner_trajectories"],
            "inner_kernel_s": st["inner_kernel_ms"] * 1e-3, "inner_share_of_nested_batches":
                st["inner_kernel_ms"] / st["nested_ms"] if st["nested_ms"] else None,
            "mean_inner_stages": st["inner_stages"] / max(st["nested_evals"], 1)}


def timed_outer_run(pkg, w, obs, rg, prec, seed, max_stages=0):
    """fault_smc_exec with every stage timed (host wall clock around each
    stage's device batches) and the run statistics on."""
    import dataclasses
    s = dataclasses.replace(w.settings, max_outer_stages=max_stages)
    g = pkg.SmcGpu(s, prec)
    g.set_data(obs)
    g.stats_reset(True)
    parts, lik, ev, ns = g.fault_smc_exec(rg, w.n_outer, seed)
    st = g.stats()
    sec, evs = g.outer_stage_times()
    g.close()
    return {"parts": parts, "evidence": ev, "nstage": ns, "stats": st, "stage_s": sec[1:], "stage_evals": evs[1:],
            "init_s": float(sec[0])}


def nested_bench(pkg, torch, peaks, fp64_peak, cpu=True, fp64_stages=3):
    """Nested SMC on c0 (one rectangle, 8x4 patches x 2 components = 64 slip
    parameters, 60 GNSS stations, 500 outer x 500 inner particles, ntau 50):
    outer particles/s averaged over every stage of a full MIXED run; FP64 on
    its first stages (a full FP64 run is about 13 minutes); MIXED vs FP64 on
    the same stages; the inner kernel's roofline; the equal-error checks."""
    w, obs, rg, th_true, s_true = nested_workload(pkg, "c0")
    N, D, ntau = w.n_outer, w.settings.dims()["D"], w.settings.ntau
    out = {"workload": "c0: 8x4 patches (D=64), 60 GNSS stations (180 obs), 500 inner x 500 outer particles, "
                       "ntau 50, CV 2 / 0.2", "n_outer": N}
    runs = {}
    for name, prec, k in (("mixed", pkg.PREC_MIXED, 0), ("fp64", pkg.PREC_FP64, fp64_stages)):
        log(f"c0 outer SMC {name}")
        r = timed_outer_run(pkg, w, obs, rg, prec, 17, k)
        runs[name] = r
        ss = r["stage_s"]
        peak = peaks.get("bf16_tflops_sustained", 1700.0) if name == "mixed" else fp64_peak
        pname = "bf16_tflops_sustained (MEASURED_PEAKS.json)" if name == "mixed" else "cuBLAS DGEMM in this run"
        out[name] = {"outer_stages_timed": len(ss), "outer_stages_total": r["nstage"] if k == 0 else None,
                     "outer_particles_per_s": N * len(ss) / ss.sum(),
                     "s_per_outer_stage_mean": float(ss.mean()),
                     "per_stage_outer_particles_per_s": [round(N / x, 1) for x in ss],
                     "nested_evals_per_s": float(r["stage_evals"].sum() / ss.sum()),
                     "init_eval_s": r["init_s"], "evidence": r["evidence"] if k == 0 else None,
                     "roofline_inner": inner_roofline(r["stats"], ntau, D, peak, pname)}
    k = len(runs["fp64"]["stage_s"])
    same = runs["mixed"]["stage_s"][:k].sum()
    out["mixed_speedup_vs_fp64"] = {"same_stages": float(runs["fp64"]["stage_s"].sum() / same), "stages": k,
                                    "mixed_all_stages_vs_fp64_first_stages":
                                        out["mixed"]["outer_particles_per_s"] / out["fp64"]["outer_particles_per_s"]}
    log("c0 equal-error checks")
    out["mixed_vs_fp64"] = equal_error_c0(pkg, w, obs, rg, th_true)
    out["mixed_vs_fp64"]["outer_posterior"] = ("full outer-SMC runs over several seeds in both precisions take "
                                               "about 13 minutes per FP64 run: bench.py --equal-error-study, "
                                               "summarised in profiles/equal_error_c0.md")
    if cpu:
        log("c0 CPU baseline")
        out["cpu_baseline"] = cpu_nested_rate(w, obs, rg)
        out["mixed_speedup_vs_cpu"] = out["mixed"]["outer_particles_per_s"] / out["cpu_baseline"]["value"]
    return out


def equal_error_c0(pkg, w, obs, rg, th_true, reps=64, n_prior=16):
    """MIXED against FP64 at equal work: -log Z at the true geometry and at
    n_prior prior-box geometries (reps independent streams each), and the
    inner slip posterior (mean and std of every slip component of the final
    population) at the true geometry over 16 streams."""
    rng = np.random.default_rng(77)
    ths = np.vstack([th_true[None], rg[:, 0] + rng.uniform(0, 1, (n_prior, len(rg))) * (rg[:, 1] - rg[:, 0])])
    thr = np.repeat(ths, reps, axis=0)
    st = np.arange(len(thr), dtype=np.uint64)
    res = {}
    for name, prec in (("mixed", pkg.PREC_MIXED), ("fp64", pkg.PREC_FP64)):
        g = pkg.SmcGpu(w.settings, prec)
        g.set_data(obs)
        v, s = g.fault_calc_likelihood(thr, 99, st + (0 if name == "fp64" else 10**6))
        res[name] = (v.reshape(len(ths), reps), s)
        g.close()
    a, b = res["mixed"][0], res["fp64"][0]
    d = a.mean(1) - b.mean(1)
    se = np.sqrt((a.var(1, ddof=1) + b.var(1, ddof=1)) / reps)
    ev = {"geometries": len(ths), "reps_per_geometry": reps, "delta_neglog_evidence": [round(float(x), 4) for x in d],
          "standard_error": [round(float(x), 4) for x in se], "fp64_mean": [round(float(x), 3) for x in b.mean(1)],
          "max_abs_delta": float(np.abs(d).max()), "max_abs_delta_over_se": float((np.abs(d) / se).max()),
          "within_0p1_nat": int((np.abs(d) <= 0.1).sum()),
          "within_0p1_nat_or_2se": int((np.abs(d) <= np.maximum(0.1, 2 * se)).sum()),
          "status_max": int(max(res["mixed"][1].max(), res["fp64"][1].max())),
          "note": "entry 0 is the true geometry, the others prior-box draws"}
    # inner slip posterior at the true geometry
    post = {}
    for name, prec in (("mixed", pkg.PREC_MIXED), ("fp64", pkg.PREC_FP64)):
        g = pkg.SmcGpu(w.settings, prec)
        g.set_data(obs)
        ms, ss = [], []
        for k in range(16):
            p = g.fault_likelihood_posterior(th_true, 123, k + (0 if name == "fp64" else 10**6))
            ms.append(p["particles"].mean(0))
            ss.append(p["particles"].std(0))
        post[name] = (np.array(ms), np.array(ss))
        g.close()
    (mm, sm), (mf, sf) = post["mixed"], post["fp64"]
    peak = float(np.abs(mf.mean(0)).max())
    dmean = np.abs(mm.mean(0) - mf.mean(0))
    dstd = np.abs(sm.mean(0) - sf.mean(0))
    se_m = np.sqrt((mm.var(0, ddof=1) + mf.var(0, ddof=1)) / 16)
    slip = {"streams": 16, "components": int(mm.shape[1]),
            "max_abs_mean_diff_rel_peak": float(dmean.max() / peak),
            "max_abs_std_diff_rel_peak": float(dstd.max() / peak),
            "max_mean_diff_over_se": float((dmean / np.maximum(se_m, 1e-12)).max()),
            "fp64_peak_mean_slip_m": peak}
    return {"evidence": ev, "slip_posterior_at_truth": slip}


def nested_c2_bench(pkg, torch, cpu=True, fp64_sample=152, sample_stages=2):
    """c2 (16x8 patches x 2 components, D = 256; 400 GNSS stations and 2000
    InSAR points in two paths with a 5 km exponential covariance, 3200
    observations; 2048 inner particles, ntau 50): one outer stage of the
    4096-particle outer SMC in MIXED (timed apart from the initial
    evaluation); FP64 against MIXED on one wave of prior geometries, both
    stopped after the same first inner stages (a full FP64 evaluation at this
    size takes about 2.5 minutes of one SM); the oracle's per-stage cost on
    the host cores."""
    import dataclasses
    w, obs, rg, th_true, s_true = nested_workload(pkg, "c2")
    log("c2 outer stage (MIXED)")
    r = timed_outer_run(pkg, w, obs, rg, pkg.PREC_MIXED, 19, 1)
    ss = r["stage_s"]
    st = r["stats"]
    out = {"workload": "c2: 16x8 patches (D=256), 400 GNSS + 2000 InSAR points (3200 obs, 5 km exponential "
                       "covariance), 4096 outer x 2048 inner particles, ntau 50",
           "mixed": {"outer_particles_per_s": w.n_outer / float(ss[0]), "s_outer_stage": float(ss[0]),
                     "stage_evals": int(r["stage_evals"][0]),
                     "nested_evals_per_s": float(r["stage_evals"][0] / ss[0]), "init_eval_s": r["init_s"],
                     "mean_inner_stages": st["inner_stages"] / max(st["nested_evals"], 1),
                     "roofline_inner": inner_roofline(st, w.settings.ntau, w.settings.dims()["D"],
                                                      PEAKS.get("bf16_tflops_sustained", 1700.0),
                                                      "bf16_tflops_sustained (MEASURED_PEAKS.json)")}}
    # FP64 against MIXED on one wave of prior geometries
    from smc_inversion_fort_gb300.configs import random_thetas
    th = random_thetas(w, fp64_sample, seed=12)
    rates = {}
    for name, prec in (("mixed", pkg.PREC_MIXED), ("fp64", pkg.PREC_FP64)):
        log(f"c2 sample {name}")
        g = pkg.SmcGpu(dataclasses.replace(w.settings, max_stages=sample_stages), prec)
        g.set_data(obs)
        g.fault_calc_likelihood(th[:2], 5, np.arange(2, dtype=np.uint64))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        nl, stt = g.fault_calc_likelihood(th, 6, np.arange(len(th), dtype=np.uint64) + 100)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        rates[name] = {"geometry_stages_per_s": len(th) * sample_stages / dt, "s_per_batch": dt}
        g.close()
    out["sample"] = {"geometries": len(th), "inner_stages": sample_stages,
                     "note": "one wave of prior geometries (one per SM), both precisions, each evaluation stopped "
                             "after the same first inner stages (initial Gibbs population included)",
                     **{k: v for k, v in rates.items()},
                     "mixed_speedup_vs_fp64": rates["fp64"]["s_per_batch"] / rates["mixed"]["s_per_batch"]}
    if cpu:
        log("c2 CPU baseline")
        out["cpu_baseline"] = cpu_stage_rate(w, obs, th, out["mixed"]["mean_inner_stages"])
        out["mixed_speedup_vs_cpu"] = out["mixed"]["outer_particles_per_s"] / out["cpu_baseline"]["value"]
    return out


def cpu_stage_rate(w, obs, th, mean_stages, stages=2):
    """The oracle (timing build) on all host threads, one geometry per
    thread, stopped after `stages` inner stages; a nested evaluation's cost
    is that per-stage cost times the mean inner stage count of the GPU run
    (outer particles/s = evaluations/s / 2)."""
    import dataclasses
    from oracle import pyoracle
    pyoracle.build()
    s = dataclasses.replace(w.settings, max_stages=stages)
    o = pyoracle.Oracle(s, obs)
    nthreads = os.cpu_count() or 1
    t0 = time.perf_counter()
    o.fault_likelihood_batch(th[:nthreads], 6, np.arange(nthreads, dtype=np.uint64) + 100, nthreads=nthreads)
    dt = time.perf_counter() - t0
    per_eval = dt / stages * mean_stages
    return {"value": nthreads / per_eval / 2.0, "unit": "outer particles/s", "cores": nthreads, "kind": "port",
            "sample": f"{nthreads} prior geometries, one per thread, first {stages} inner stages in {dt:.1f} s, "
                      f"scaled to the GPU run's mean of {mean_stages:.1f} inner stages per evaluation"}


def nested_c4_bench(pkg, torch, sample=152, stages=2):
    """c4 slip size (32x16 patches x 2 components, D = 1024; 400 GNSS and
    10000 InSAR points in eight paths, 11200 observations; 4096 inner
    particles, ntau 50), MIXED on the global-matrix engine, one wave of prior
    geometries (one per SM).  A full evaluation takes about 7.5 minutes at
    this size, so by default every evaluation stops after `stages` inner
    stages (stages = 0: full evaluations) and the rate is reported per
    geometry-stage."""
    import dataclasses
    from smc_inversion_fort_gb300.configs import random_thetas
    log("c4 data")
    w, obs, rg, th_true, s_true = nested_workload(pkg, "c4")
    log("c4 sample")
    if stages:
        w = dataclasses.replace(w, settings=dataclasses.replace(w.settings, max_stages=stages))
    g = pkg.SmcGpu(w.settings, pkg.PREC_MIXED)
    g.set_data(obs)
    th = random_thetas(w, sample, seed=13)
    g.stats_reset(True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    nl, stt = g.fault_calc_likelihood(th, 7, np.arange(len(th), dtype=np.uint64))
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    st = g.stats()
    g.close()
    D = w.settings.dims()["D"]
    # the global-matrix engine streams M (D^2 FP32) once per leapfrog step of
    # a group's 16 chain slots and A once per trajectory end of those slots:
    # 4 D^2 (ntau + 2) bytes per round of 16 trajectories (slots assumed full,
    # so the figure is a lower bound on the bytes read)
    traj = st["inner_trajectories"]
    gbs = traj / 16.0 * (w.settings.ntau + 2) * 4.0 * D * D / (st["inner_kernel_ms"] * 1e-3) / 1e9
    if stt.max() and not stages:
        log(f"c4: status bits {int(stt.max())}")
    res = {"workload": "c4: 32x16 patches (D=1024), 400 GNSS + 10000 InSAR points (11200 obs, 5 km exponential "
                       "covariance, 8 paths), 4096 inner particles, ntau 50, MIXED",
           "sample": f"{len(th)} prior geometries in one batch (one per SM)" +
                     (f", every evaluation stopped after {stages} inner stages" if stages else ""),
           "s_per_batch": dt, "geometry_stages_per_s": st["inner_stages"] / dt,
           "mean_inner_stages": st["inner_stages"] / max(st["nested_evals"], 1),
            "roofline_inner": {"bound": "hbm", "achieved": gbs, "peak": PEAKS.get("hbm_gbs"), "unit": "GB/s",
                               "frac": gbs / PEAKS["hbm_gbs"] if PEAKS.get("hbm_gbs") else None,
                               "note": "stage matrix (FP32, D^2) streamed per leapfrog step, A per trajectory end; "
                                       "algorithmic bytes 4 D^2 (ntau + 2) per round of 16 trajectories (one per chain slot)",
                               "inner_kernel_s": st["inner_kernel_ms"] * 1e-3}}
    if not stages:
        res.update({"nested_evals_per_s": len(th) / dt, "outer_particles_per_s": len(th) / dt / 2,
                    "status_max": int(stt.max()), "neglog_median": float(np.median(nl))})
    return res


def nested_c3_bench(pkg, torch, sample=304, cmp_sample=152, stages=2, cmp_stages=1):
    """c3: per-geometry meshes (2.5 km patches on a 10-60 km x 5-30 km
    rectangle: 4x2 ... 24x12 patches, D = 16 ... 576) with the c2
    observations and 2048 inner particles, engines from the autotuner's
    table (SMCGPU_ENGINE_AUTO).  A full evaluation of the largest meshes takes
    minutes (FP64: tens of minutes), so every evaluation stops after the same
    first inner stages: MIXED geometry-stages/s on `sample` prior geometries
    (each call splits the batch by mesh and runs the parts concurrently), and
    MIXED against FP64 on the first `cmp_sample` of them, both stopped after
    `cmp_stages` stages (the initial Gibbs population included)."""
    import dataclasses
    from smc_inversion_fort_gb300.configs import mesh_of, random_thetas
    w, obs, rg, th_true, s_true = nested_workload(pkg, "c3")
    th = random_thetas(w, sample, seed=14)
    D = np.array([2 * np.prod(mesh_of(w.settings, t)) for t in th])
    out = {"workload": "c3: 2.5 km patches on 10-60 x 5-30 km rectangles (4x2 ... 24x12 patches, D 16-576), "
                       "400 GNSS + 2000 InSAR points (3200 obs), 2048 inner particles, ntau 50, engines from "
                       "the autotuner's table",
           "meshes_in_sample": int(len({mesh_of(w.settings, t) for t in th})),
           "D_min_median_max": [int(D.min()), float(np.median(D)), int(D.max())]}

    def run(prec, n, k, seed):
        g = pkg.SmcGpu(dataclasses.replace(w.settings, max_stages=k), prec)
        g.set_data(obs)
        g.fault_calc_likelihood(th[:n], 5, np.arange(n, dtype=np.uint64))   # meshes' contexts and buffers
        g.stats_reset(True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        nl, st = g.fault_calc_likelihood(th[:n], seed, np.arange(n, dtype=np.uint64) + 1000)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        stt = g.stats()
        g.close()
        return {"geometries": n, "inner_stages": k, "s_per_batch": dt,
                "geometry_stages_per_s": stt["inner_stages"] / dt, "status_max": int(st.max())}

    log("c3 sample mixed")
    out["mixed"] = run(pkg.PREC_MIXED, sample, stages, 6)
    out["mixed"]["note"] = f"{sample} prior geometries, every evaluation stopped after {stages} inner stages"
    cmp = {}
    for name, prec in (("mixed", pkg.PREC_MIXED), ("fp64", pkg.PREC_FP64)):
        log(f"c3 comparison {name}")
        cmp[name] = run(prec, cmp_sample, cmp_stages, 7)
    out["comparison"] = {"note": f"the first {cmp_sample} geometries in both precisions, every evaluation stopped "
                                 f"after {cmp_stages} inner stage(s); the largest mesh sets the wall time",
                         **cmp, "mixed_speedup_vs_fp64": cmp["fp64"]["s_per_batch"] / cmp["mixed"]["s_per_batch"]}
    return out


def cpu_nested_rate(w, obs, rg, target_s=15.0):
    """Oracle (timing build) nested evaluations of prior-box geometries on all
    host threads (one geometry per thread, as the reference's MPI ranks);
    outer particles per second = evaluations per second / 2."""
    from oracle import pyoracle
    pyoracle.build()
    o = pyoracle.Oracle(w.settings, obs)
    nthreads = os.cpu_count() or 1
    rng = np.random.default_rng(5)
    th = rg[:, 0] + rng.uniform(0, 1, (4 * nthreads, len(rg))) * (rg[:, 1] - rg[:, 0])
    t0 = time.perf_counter()
    o.fault_likelihood_batch(th[:nthreads], 1, np.arange(nthreads, dtype=np.uint64), nthreads=nthreads)
    t1 = time.perf_counter() - t0
    n = int(min(len(th), max(nthreads, nthreads * round(target_s / max(t1, 1e-3)))))
    t0 = time.perf_counter()
    o.fault_likelihood_batch(th[:n], 1, np.arange(n, dtype=np.uint64), nthreads=nthreads)
    dt = time.perf_counter() - t0
    return {"value": n / dt / 2.0, "unit": "outer particles/s", "cores": nthreads, "kind": "port",
            "sample": f"{n} nested evaluations of prior-box geometries, {dt:.1f} s wall"}


def gb300_arm(args):
    import torch
    import torch.distributed as tdist

    rank, world, local = dist_env()
    if world > 1 and not tdist.is_initialized():
        tdist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    import smc_inversion_fort_gb300 as pkg
    from smc_inversion_fort_gb300 import build as b
    from oracle import pyoracle
    pyoracle.use_timing_build()   # the CPU baseline legs time the -O3 build of the oracle
    b.build()
    if args.equal_error_study:
        equal_error_study(pkg, torch, args)
        return
    if args.equal_error_points:
        equal_error_points(pkg, args.equal_error_points)
        return
    w, obs, th = workload(args.n_theta)
    g = pkg.SmcGpu(w.settings, device=local)
    g.set_data(obs)
    dm = g.dims()
    D, nobs, n = dm["D"], dm["nobs"], args.n_theta
    entries = n * nobs * D
    # a dedicated (non-default) stream: the library launches on it and the
    # CUDA events below are recorded on it
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    g.set_stream(stream.cuda_stream)
    dth = torch.from_numpy(th).to(dev)
    out = torch.empty((n, D, nobs), dtype=torch.float64, device=dev)

    def step():
        g.greens_dev(n, dth.data_ptr(), out.data_ptr(), pkg.PREC_FP64)

    log("c1 Green's build")
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    clk = ClockSampler(local)
    if world > 1:
        tdist.barrier()
    torch.cuda.synchronize()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    t_start, t_end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t_start.record(stream)
    for a, e in evs:
        a.record(stream)
        step()
        e.record(stream)
    t_end.record(stream)
    torch.cuda.synchronize()
    if world > 1:
        tdist.barrier()
    clocks = clk.stop()
    total_ms = max_over_ranks(t_start.elapsed_time(t_end), world, dev)
    ms = total_ms / args.steps
    kern_ms = statistics.mean(a.elapsed_time(e) for a, e in evs)
    value = entries * world / (ms * 1e-3)
    evals = n * w.settings.dims()["npatch"] * w.settings.nquad ** 2 * 400
    ach_tflops = evals * FLOPS_PER_EVAL / (kern_ms * 1e-3) / 1e12
    alg_bytes = entries * 8 + th.nbytes + 400 * 8 * 7
    ach_gbs = alg_bytes / (kern_ms * 1e-3) / 1e9
    peaks = {}
    mp = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(mp):
        with open(mp) as f:
            peaks = json.load(f)
    PEAKS.update(peaks)
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    fp64_peak = measured_peak_fp64_tflops(torch, dev)

    # FP32 variant of the same build
    out32 = torch.empty((n, D, nobs), dtype=torch.float32, device=dev)
    for _ in range(2):
        g.greens_dev(n, dth.data_ptr(), out32.data_ptr(), pkg.PREC_FP32)
    torch.cuda.synchronize()
    a32, e32 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a32.record(stream)
    for _ in range(args.steps):
        g.greens_dev(n, dth.data_ptr(), out32.data_ptr(), pkg.PREC_FP32)
    e32.record(stream)
    torch.cuda.synchronize()
    ms32 = a32.elapsed_time(e32) / args.steps
    # FP32 error against the FP64 build on a slice
    sl = slice(0, min(n, 64))
    ref = out[sl]
    scale = ref.abs().amax(dim=-1, keepdim=True).clamp_min(1e-300)
    err32 = float(((out32[sl].double() - ref).abs() / scale).max().item())
    del out32

    # end to end through the C ABI with host buffers (pinned), FP64
    th_host = torch.from_numpy(th).pin_memory()
    out_host = torch.empty((n, D, nobs), dtype=torch.float64).pin_memory()
    g.set_stream(None)
    g.calc_greens_func(th_host.numpy(), pkg.PREC_FP64, out=out_host.numpy())
    if world > 1:
        tdist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        g.calc_greens_func(th_host.numpy(), pkg.PREC_FP64, out=out_host.numpy())
    e2e_s = max_over_ranks((time.perf_counter() - t0) / args.steps, world, dev)
    same = bool(torch.equal(out_host[:4], out[:4].cpu()))
    del out_host

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded stations, prior-box geometries)",
            "config": c1_config(n, nobs, D),
            "gpu_launches": 2 * args.steps,
            "roofline": {"bound": "hbm", "achieved": ach_gbs, "peak": hbm_peak, "unit": "GB/s",
                         "frac": ach_gbs / hbm_peak, "traffic": None,
                         "note": "ALU-bound kernel; the binding roofline is roofline_alu (FP64 pipe)"},
            "roofline_alu": {"bound": "fp64", "achieved": ach_tflops, "peak": fp64_peak, "unit": "TFLOP/s",
                             "frac": ach_tflops / fp64_peak, "flops_per_eval": FLOPS_PER_EVAL,
                             "evals_per_launch": evals, "peak_source": "measured cuBLAS DGEMM 4096^3 in this run"},
            "kernel_ms": kern_ms,
            "fp32": {"value": entries * world / (ms32 * 1e-3), "ms_per_step": ms32, "col_rel_err_vs_fp64": err32},
            "e2e": {"value": entries * world / e2e_s, "unit": UNIT, "h2d_bytes_per_step": th.nbytes,
                    "d2h_bytes_per_step": entries * 8, "bitwise_equal_to_device_path": same},
            "clocks": clocks}
    tr = load_traffic()
    if tr:
        line["roofline"]["traffic"] = tr.get("traffic_bytes_per_launch")
        line["roofline"]["traffic_source"] = tr.get("source")
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_greens_rate(w, obs, th)
        line["cpu_baseline"].pop("wall_s", None)
    if not args.no_nested:
        g.close()
        del out, dth
        torch.cuda.empty_cache()
        cpu = rank == 0 and not args.no_cpu_baseline
        line["nested_smc"] = nested_bench(pkg, torch, peaks, fp64_peak, cpu=cpu, fp64_stages=args.fp64_stages)
        if not args.no_c2:
            line["nested_smc_c2"] = nested_c2_bench(pkg, torch, cpu=cpu)
        if not args.no_c3:
            line["nested_smc_c3"] = nested_c3_bench(pkg, torch)
        if not args.no_c4:
            line["nested_smc_c4"] = nested_c4_bench(pkg, torch, stages=0 if args.c4_full else 2)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        tdist.destroy_process_group()


def equal_error_study(pkg, torch, args):
    """Full c0 outer-SMC runs (fault_smc_exec to gamma = 1) over several
    seeds in MIXED and FP64: posterior mean and std of every geometry
    parameter, evidence, stage counts and per-stage timing, written as JSON."""
    km, kf = (int(x) for x in args.study_seeds.split(","))
    om, of = (int(x) for x in args.study_seed0.split(","))
    w, obs, rg, th_true, s_true = nested_workload(pkg, "c0")
    runs = {"mixed": [], "fp64": []}
    for name, prec, k, off in (("mixed", pkg.PREC_MIXED, km, om), ("fp64", pkg.PREC_FP64, kf, of)):
        for seed in range(off + 1, off + k + 1):
            t0 = time.perf_counter()
            r = timed_outer_run(pkg, w, obs, rg, prec, seed)
            p = r["parts"]
            runs[name].append({"seed": seed, "evidence": r["evidence"], "nstage": r["nstage"],
                               "wall_s": time.perf_counter() - t0, "mean": p.mean(0).tolist(),
                               "std": p.std(0).tolist(), "stage_s": [round(float(x), 4) for x in r["stage_s"]],
                               "stats": r["stats"]})
            print(name, seed, r["nstage"], r["evidence"], round(time.perf_counter() - t0, 1), flush=True)
    summ = {}
    for name in runs:
        if not runs[name]:
            continue
        m = np.array([x["mean"] for x in runs[name]])
        sd = np.array([x["std"] for x in runs[name]])
        ev = np.array([x["evidence"] for x in runs[name]])
        summ[name] = {"seeds": len(m), "mean_of_means": m.mean(0).tolist(),
                      "se_of_means": (m.std(0, ddof=1) / np.sqrt(len(m))).tolist() if len(m) > 1 else None,
                      "mean_of_stds": sd.mean(0).tolist(), "evidence_mean": float(ev.mean()),
                      "evidence_se": float(ev.std(ddof=1) / np.sqrt(len(ev))) if len(ev) > 1 else None}
    width = rg[:, 1] - rg[:, 0]
    ee = None
    if not args.study_no_evidence:
        log("evidence and slip posterior, 512 streams per geometry")
        ee = equal_error_c0(pkg, w, obs, rg, th_true, reps=512)
    res = {"workload": "c0 (8x4 patches, D = 64, 60 GNSS stations, 500 outer x 500 inner particles, ntau 50)",
           "evidence_and_slip": ee,
           "parameters": ["x", "y", "top", "length", "width", "strike", "dip", "log_alpha2"],
           "true_theta": th_true.tolist(), "prior_range": rg.tolist(), "runs": runs, "summary": summ}
    if "mixed" in summ and "fp64" in summ:
        mm, mf = np.array(summ["mixed"]["mean_of_means"]), np.array(summ["fp64"]["mean_of_means"])
        sdm, sdf = np.array(summ["mixed"]["mean_of_stds"]), np.array(summ["fp64"]["mean_of_stds"])
        res.update({"posterior_mean_rel_diff": ((mm - mf) / np.abs(mf)).tolist(),
                    "posterior_mean_diff_rel_prior_width": ((mm - mf) / width).tolist(),
                    "posterior_std_rel_diff": ((sdm - sdf) / sdf).tolist(),
                    "evidence_diff": summ["mixed"]["evidence_mean"] - summ["fp64"]["evidence_mean"]})
    with open(args.equal_error_study, "w") as f:
        json.dump(res, f, indent=1)
    print(json.dumps({k: res[k] for k in ("posterior_mean_rel_diff", "posterior_std_rel_diff", "evidence_diff")
                      if k in res}))


def equal_error_points(pkg, spec, reps=512):
    """-log Z of the c0 nested evaluation in MIXED and FP64 at given
    geometries, `reps` independent streams each: mean, spread, median,
    minimum and the log of the mean evidence per precision."""
    w, obs, rg, th_true, s_true = nested_workload(pkg, "c0")
    ths = np.array([[float(v) for v in t.split(",")] for t in spec.split(";")])
    thr = np.repeat(ths, reps, axis=0)
    st = np.arange(len(thr), dtype=np.uint64)
    res = {}
    for name, prec in (("mixed", pkg.PREC_MIXED), ("fp64", pkg.PREC_FP64)):
        g = pkg.SmcGpu(w.settings, prec)
        g.set_data(obs)
        v, s = g.fault_calc_likelihood(thr, 99, st + (0 if name == "fp64" else 10**6))
        res[name] = v.reshape(len(ths), reps)
        print(name, "status max", int(s.max()), flush=True)
        g.close()
    for i in range(len(ths)):
        a, b = res["mixed"][i], res["fp64"][i]
        se = np.sqrt((a.var(ddof=1) + b.var(ddof=1)) / reps)
        print(f"theta {i}: mixed {a.mean():.4f} (sd {a.std():.3f}, med {np.median(a):.3f}, min {a.min():.3f}) "
              f"fp64 {b.mean():.4f} (sd {b.std():.3f}, med {np.median(b):.3f}, min {b.min():.3f})  "
              f"diff {a.mean() - b.mean():+.4f} se {se:.4f}")


def main():
    args = parse()
    if args.impl == "reference":
        reference_arm(args)
    else:
        gb300_arm(args)


if __name__ == "__main__":
    main()
