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
    p.add_argument("--no-c2", action="store_true", help="skip the c2 (D = 256) nested sample")
    p.add_argument("--c2-cpu-baseline", action="store_true",
                   help="also time the oracle on c2 (16 geometries, one per host thread: about 2.5 minutes, the "
                        "slowest geometry sets the wall time)")
    p.add_argument("--outer-stages", type=int, default=1)
    return p.parse_args()


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def workload(n_theta):
    from smc_inversion_fort_gb300.configs import make_stations, preset, random_thetas
    w = preset("c1")
    obs = make_stations(w, np.random.default_rng(2024))
    obs["dvec"] = np.zeros(len(obs["obs_sigma"]))
    th = random_thetas(w, n_theta, seed=7)
    return w, obs, th


def cpu_greens_rate(w, obs, th, target_s=15.0, max_theta=512):
    """Oracle Green's build on all host threads over a bounded sample."""
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
            "sample": f"{n} of {len(th)} geometries, full 1200x256 matrices, {dt:.1f} s wall"}


def reference_arm(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    w, obs, th = workload(args.n_theta)
    vals = []
    cb = None
    for k in range(args.warmup + args.steps):
        r = cpu_greens_rate(w, obs, th, target_s=8.0 if k >= args.warmup else 2.0, max_theta=256)
        if k >= args.warmup:
            vals.append(r["value"])
            cb = r
    v = statistics.median(vals)
    D = w.settings.dims()["D"]
    nobs = 3 * 400
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": args.n_theta * nobs * D / v * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": "c1: 8192 geometries x 16x8 patches x 5x5 Gauss points x 400 stations (3-comp)",
                       "n_theta": args.n_theta, "nobs": nobs, "D": D},
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


def nested_workload(seed=2024):
    """c0: 8x4 patches x 2 components (D = 64), 60 three-component GNSS
    stations, 500 inner and 500 outer particles; data from the known fault."""
    from smc_inversion_fort_gb300.configs import make_stations, preset, prior_range, true_slip, true_theta
    w = preset("c0")
    rng = np.random.default_rng(seed)
    obs = make_stations(w, rng)
    return w, obs, rng, prior_range(w), true_theta(w), true_slip(w)


def nested_bench(pkg, torch, stages=1, cpu=True):
    """Outer particles/s of the nested SMC on c0, FP64 and MIXED, and the
    MIXED-vs-FP64 evidence difference."""
    import dataclasses
    w, obs, rng, rg, th_true, s_true = nested_workload()
    obs["dvec"] = np.zeros(len(obs["obs_sigma"]))
    g = pkg.SmcGpu(w.settings)
    g.set_data(obs)
    G = g.calc_greens_func(th_true[None])[0]
    obs["dvec"] = G.T @ s_true + rng.standard_normal(G.shape[1]) * obs["obs_sigma"]
    out = {"workload": "c0: 8x4 patches (D=64), 60 GNSS stations (180 obs), 500 inner x 500 outer particles, "
                       "ntau 50, CV 2 / 0.2", "n_outer": w.n_outer, "timed_outer_stages": stages}
    for name, prec in (("mixed", pkg.PREC_MIXED), ("fp64", pkg.PREC_FP64)):
        times = {}
        for k in (-1, stages):
            s2 = dataclasses.replace(w.settings, max_outer_stages=k)
            gg = pkg.SmcGpu(s2, prec)
            gg.set_data(obs)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            _, _, ev, ns = gg.fault_smc_exec(rg, w.n_outer, 17)
            torch.cuda.synchronize()
            times[k] = time.perf_counter() - t0
            gg.close()
        per_stage = (times[stages] - times[-1]) / stages
        out[name] = {"outer_particles_per_s": w.n_outer / per_stage, "s_per_outer_stage": per_stage,
                     "nested_evals_per_s": 2 * w.n_outer / per_stage, "init_eval_s": times[-1]}
    # evidence agreement on the true geometry over independent streams
    # (1024 per precision: standard error about 0.03 nat)
    reps = 1024
    thr = np.repeat(th_true[None], reps, 0)
    st = np.arange(reps, dtype=np.uint64)
    res = {}
    for name, prec in (("mixed", pkg.PREC_MIXED), ("fp64", pkg.PREC_FP64)):
        gg = pkg.SmcGpu(w.settings, prec)
        gg.set_data(obs)
        res[name], _ = gg.fault_calc_likelihood(thr, 99, st + (0 if name == "fp64" else 10**6))
        gg.close()
    d = res["mixed"].mean() - res["fp64"].mean()
    se = float(np.sqrt((res["mixed"].var(ddof=1) + res["fp64"].var(ddof=1)) / reps))
    out["mixed_vs_fp64"] = {"delta_neglog_evidence": float(d), "standard_error": se, "reps": reps,
                            "fp64_mean": float(res["fp64"].mean()), "fp64_std": float(res["fp64"].std())}
    out["mixed_speedup_vs_fp64"] = out["mixed"]["outer_particles_per_s"] / out["fp64"]["outer_particles_per_s"]
    if cpu:
        out["cpu_baseline"] = cpu_nested_rate(w, obs, rg)
        out["mixed_speedup_vs_cpu"] = out["mixed"]["outer_particles_per_s"] / out["cpu_baseline"]["value"]
    return out


def nested_c2_bench(pkg, torch, cpu=True):
    """Nested evaluations/s on c2 (16x8 patches x 2 components, D = 256; 400
    GNSS stations and 2000 InSAR points in two paths with a 5 km exponential
    covariance, 3200 observations; 2048 inner particles, ntau 50), MIXED.
    Sample: four waves of prior geometries (the inner kernel runs one geometry
    per CTA at this size, so CTAs that finish early take the next geometries;
    one wave would time only the slowest geometry), after a small warm-up batch."""
    from smc_inversion_fort_gb300.configs import make_stations, preset, random_thetas, true_slip, true_theta
    w = preset("c2")
    rng = np.random.default_rng(2024)
    obs = make_stations(w, rng)
    obs["dvec"] = np.zeros(len(obs["obs_sigma"]))
    g = pkg.SmcGpu(w.settings, pkg.PREC_MIXED)
    g.set_data(obs)
    G = g.calc_greens_func(true_theta(w)[None])[0]
    obs["dvec"] = G.T @ true_slip(w) + rng.standard_normal(G.shape[1]) * obs["obs_sigma"]
    g.set_data(obs)
    nsm = torch.cuda.get_device_properties(0).multi_processor_count
    g.fault_calc_likelihood(random_thetas(w, 8, seed=11), 5, np.arange(8, dtype=np.uint64))
    n = 4 * nsm
    th = random_thetas(w, n, seed=12)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    nl, st = g.fault_calc_likelihood(th, 6, np.arange(n, dtype=np.uint64) + 100)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    g.close()
    out = {} if cpu else {"cpu_baseline": None,
                          "cpu_baseline_note": "off by default (about 2.5 minutes); bench.py --c2-cpu-baseline"}
    if cpu:
        # the oracle on all host threads, one geometry per thread, on the first
        # geometries of the same sample (the oracle's covariance set-up, like
        # set_data on the GPU, is outside the timed region)
        from oracle import pyoracle
        pyoracle.build()
        o = pyoracle.Oracle(w.settings, obs)
        nthreads = os.cpu_count() or 1
        t0 = time.perf_counter()
        o.fault_likelihood_batch(th[:nthreads], 6, np.arange(nthreads, dtype=np.uint64) + 100, nthreads=nthreads)
        tc = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": nthreads / tc / 2.0, "unit": "outer particles/s", "cores": nthreads,
                               "kind": "port", "sample": f"the first {nthreads} geometries of the GPU sample, one "
                                                         f"per thread, {tc:.1f} s wall"}
        out["mixed_speedup_vs_cpu"] = (n / dt / 2.0) / out["cpu_baseline"]["value"]
    return {"workload": "c2: 16x8 patches (D=256), 400 GNSS + 2000 InSAR points (3200 obs, 5 km exponential "
                        "covariance), 2048 inner particles, ntau 50, MIXED",
            "sample": f"{n} prior geometries in one batch (four waves of one geometry per SM)",
            "nested_evals_per_s": n / dt, "outer_particles_per_s": n / dt / 2, "s_per_batch": dt,
            "status_max": int(st.max()), "neglog_median": float(np.median(nl)), **out}


def cpu_nested_rate(w, obs, rg, target_s=15.0):
    """Oracle nested evaluations of prior-box geometries on all host threads
    (one geometry per thread, as the reference's MPI ranks); outer particles
    per second = evaluations per second / 2."""
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
    b.build()
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
    total_ms = t_start.elapsed_time(t_end)
    if world > 1:
        t = torch.tensor([total_ms], device=dev)
        tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
        total_ms = float(t.item())
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
    e2e_s = (time.perf_counter() - t0) / args.steps
    if world > 1:
        t = torch.tensor([e2e_s], device=dev)
        tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
        e2e_s = float(t.item())
    same = bool(torch.equal(out_host[:4], out[:4].cpu()))
    del out_host

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded stations, prior-box geometries)",
            "config": {"workload": "c1: 8192 geometries x 16x8 patches x 5x5 Gauss points x 400 stations (3-comp), "
                                   "patch-constant basis, FP64",
                       "n_theta": n, "nobs": nobs, "D": D, "entries_per_step": entries,
                       "l2": "output 20.1 GB per step, larger than L2; no flush needed"},
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
    if not args.no_nested:
        g.close()
        del out, dth
        torch.cuda.empty_cache()
        line["nested_smc"] = nested_bench(pkg, torch, stages=args.outer_stages,
                                          cpu=(rank == 0 and not args.no_cpu_baseline))
        if not args.no_c2:
            line["nested_smc_c2"] = nested_c2_bench(pkg, torch, cpu=(rank == 0 and args.c2_cpu_baseline))
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        tdist.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        reference_arm(args)
    else:
        gb300_arm(args)


if __name__ == "__main__":
    main()
