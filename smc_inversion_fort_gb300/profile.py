"""Fixed small workloads for profiling one kernel family at a time.

    python -m smc_inversion_fort_gb300.profile greens [--n-theta 256] [--fp32] [--reps 2]
    python -m smc_inversion_fort_gb300.profile nested [--n-theta 16] [--mixed] [--reps 1] [--warps 0]
        [--engine mma|cuda|tcgen05|global|auto] [--workload c0] [--max-stages K]

`greens` runs the Green's build of the 16x8-patch, 5x5-Gauss-point,
400-station workload on n geometries; `nested` runs nested evaluations of the
8x4-patch, 60-station, 500-particle workload.  Each rep is one batch.
"""
from __future__ import annotations

import argparse
import time

import numpy as np


def main(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("what", choices=["greens", "nested", "outer"])
    p.add_argument("--stages", type=int, default=1, help="outer: outer SMC stages after the initial evaluation")
    p.add_argument("--n-theta", type=int, default=0)
    p.add_argument("--fp32", action="store_true")
    p.add_argument("--mixed", action="store_true")
    p.add_argument("--reps", type=int, default=2)
    p.add_argument("--warps", type=int, default=0, help="inner kernel warps per geometry (0: by batch size)")
    p.add_argument("--engine", choices=["mma", "cuda", "tcgen05", "global", "auto"], default="mma",
                   help="inner step engine")
    p.add_argument("--max-stages", type=int, default=0, help="nested: stop every evaluation after K inner stages")
    p.add_argument("--workload", default="c0", help="nested: named workload (c0, c2, d160, d256, ...)")
    a = p.parse_args(argv)
    import torch

    import smc_inversion_fort_gb300 as pkg
    from smc_inversion_fort_gb300.configs import make_stations, preset, random_thetas, true_slip, true_theta

    if a.what == "greens":
        w = preset("c1")
        n = a.n_theta or 256
        obs = make_stations(w, np.random.default_rng(2024))
        obs["dvec"] = np.zeros(len(obs["obs_sigma"]))
        g = pkg.SmcGpu(w.settings)
        g.set_data(obs)
        dm = g.dims()
        th = torch.from_numpy(random_thetas(w, n, seed=7)).cuda()
        prec = pkg.PREC_FP32 if a.fp32 else pkg.PREC_FP64
        out = torch.empty((n, dm["D"], dm["nobs"]), dtype=torch.float32 if a.fp32 else torch.float64, device="cuda")
        for _ in range(a.reps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            g.greens_dev(n, th.data_ptr(), out.data_ptr(), prec)
            torch.cuda.synchronize()
            print(f"greens n_theta={n} {'fp32' if a.fp32 else 'fp64'}: {1e3 * (time.perf_counter() - t0):.2f} ms")
    elif a.what == "outer":
        # fault_smc_exec on the workload's outer population, a few stages
        from smc_inversion_fort_gb300.configs import prior_range
        import dataclasses
        w = preset(a.workload)
        rng = np.random.default_rng(2024)
        obs = make_stations(w, rng)
        obs["dvec"] = np.zeros(len(obs["obs_sigma"]))
        prec = pkg.PREC_MIXED if a.mixed else pkg.PREC_FP64
        g = pkg.SmcGpu(w.settings, prec)
        g.set_data(obs)
        G = g.calc_greens_func(true_theta(w)[None])[0]
        obs["dvec"] = G.T @ true_slip(w) + rng.standard_normal(G.shape[1]) * obs["obs_sigma"]
        g.close()
        g = pkg.SmcGpu(dataclasses.replace(w.settings, max_outer_stages=a.stages), prec)
        g.set_data(obs)
        t0 = time.perf_counter()
        _, _, ev, ns = g.fault_smc_exec(prior_range(w), w.n_outer, 17)
        print(f"outer {a.workload} {'mixed' if a.mixed else 'fp64'} {ns} stages: {time.perf_counter() - t0:.3f} s, "
              f"evidence {ev:.4f}")
    else:
        from smc_inversion_fort_gb300.configs import fixed_mesh
        w = preset(a.workload)
        w.settings.inner_warps = a.warps
        w.settings.inner_engine = {"mma": 0, "cuda": 1, "tcgen05": 2, "global": 3, "auto": 4}[a.engine]
        if a.max_stages:
            w.settings.max_stages = a.max_stages
        n = a.n_theta or 16
        rng = np.random.default_rng(2024)
        obs = make_stations(w, rng)
        obs["dvec"] = np.zeros(len(obs["obs_sigma"]))
        prec = pkg.PREC_MIXED if a.mixed else pkg.PREC_FP64
        # data from the true geometry on its own mesh (per-geometry mesh workloads)
        wf = fixed_mesh(w, true_theta(w))
        g0 = pkg.SmcGpu(wf.settings)
        g0.set_data(obs)
        G = g0.calc_greens_func(true_theta(w)[None])[0]
        g0.close()
        obs["dvec"] = G.T @ true_slip(wf) + rng.standard_normal(G.shape[1]) * obs["obs_sigma"]
        g = pkg.SmcGpu(w.settings, prec)
        g.set_data(obs)
        th = np.vstack([true_theta(w)[None], random_thetas(w, n - 1, seed=3)])
        for r in range(a.reps):
            t0 = time.perf_counter()
            nl, st = g.fault_calc_likelihood(th, 1, np.arange(n, dtype=np.uint64) + 1000 * r)
            print(f"nested {a.workload} n_theta={n} warps={a.warps} {a.engine} {'mixed' if a.mixed else 'fp64'}: "
                  f"{time.perf_counter() - t0:.3f} s, "
                  f"-logZ[0] {nl[0]:.4f}, status {int(st.max())}")


if __name__ == "__main__":
    main()
