"""Autotuner of the inner SMC step engine per slip dimension.

For each slip-dimension bucket of the per-geometry meshes (2.5 km patches on
a 10-60 km x 5-30 km rectangle: 4x2 ... 24x12 patches, D = 16 ... 576) and
for MIXED and FP64, every engine configuration that takes the size is timed
on the device on one batch of prior geometries with the c2/c3 observations
(400 GNSS stations, 2000 InSAR points, 2048 inner particles), stopped after a
few inner stages so that a candidate costs seconds (sizes that only one
engine takes are not timed).  The fastest configuration of each bucket goes
into the engine table that
SMCGPU_ENGINE_AUTO reads (smcgpu_set_engine_table; SmcGpu loads
engine_table.json next to this file).

    python -m smc_inversion_fort_gb300.autotune [--out PATH] [--stages K] [--batch N]

Candidates (warps per geometry for the CUDA-core engine):
  MIXED: warp MMA (D <= 256), CUDA cores with 2, 4 or 8 warps (D <= 192),
         tcgen05 (D <= 128), global matrix (any D);
  FP64:  CUDA cores with 2, 4 or 8 warps (D <= 128), global matrix (any D).
"""
from __future__ import annotations

import argparse
import dataclasses
import json
import os
import time

import numpy as np

# (nxi, neta) of each bucket's representative mesh; the bucket covers the
# slip dimensions above the previous bucket's up to its own D = 2 nxi neta
BUCKETS = [(4, 2), (4, 4), (8, 4), (8, 6), (8, 8), (12, 8), (16, 8), (16, 12), (24, 12)]


def candidates(pkg, mixed: bool, D: int):
    out = []
    if mixed:
        if D <= 256:
            out.append((pkg.ENGINE_MMA, 0))
        if D <= 192:
            out += [(pkg.ENGINE_CUDA, w) for w in (2, 4, 8)]
        if D <= 128:
            out.append((pkg.ENGINE_TCGEN05, 0))
    elif D <= 128:
        out += [(pkg.ENGINE_CUDA, w) for w in (2, 4, 8)]
    out.append((pkg.ENGINE_GLOBAL, 0))
    return out


def time_candidate(pkg, settings, prec, engine, warps, obs, th, reps=2):
    s = dataclasses.replace(settings, inner_engine=engine, inner_warps=warps)
    g = pkg.SmcGpu(s, prec)
    g.set_data(obs)
    st = np.arange(len(th), dtype=np.uint64)
    g.fault_calc_likelihood(th[:2], 1, st[:2])   # warm-up: allocations, module load
    best = float("inf")
    for r in range(reps):
        t0 = time.perf_counter()
        g.fault_calc_likelihood(th, 2 + r, st)
        best = min(best, time.perf_counter() - t0)
    g.close()
    return best


def tune(stages: int = 2, batch: int = 0, out: str | None = None, verbose: bool = True):
    import torch

    import smc_inversion_fort_gb300 as pkg
    from smc_inversion_fort_gb300.configs import make_stations, preset, random_thetas

    w = preset("c3")
    obs = make_stations(w, np.random.default_rng(2024))
    obs["dvec"] = np.random.default_rng(1).standard_normal(len(obs["obs_sigma"])) * obs["obs_sigma"]
    nsm = torch.cuda.get_device_properties(0).multi_processor_count
    n = batch or 2 * nsm
    th = random_thetas(w, n, seed=21)
    table = {"fp64": [], "mixed": []}
    timings = []
    for prec, key in ((pkg.PREC_MIXED, "mixed"), (pkg.PREC_FP64, "fp64")):
        for nxi, neta in BUCKETS:
            s = dataclasses.replace(w.settings, nxi=(nxi,), neta=(neta,), patch_km=0.0, max_stages=stages)
            D = 2 * nxi * neta
            res = []
            cands = candidates(pkg, prec == pkg.PREC_MIXED, D)
            if len(cands) == 1:   # only the global-matrix engine takes this size
                table[key].append([D, cands[0][0], cands[0][1]])
                continue
            for eng, wp in cands:
                t = time_candidate(pkg, s, prec, eng, wp, obs, th)
                res.append((t, eng, wp))
                timings.append({"precision": key, "D": D, "engine": eng, "warps": wp, "seconds": t})
                if verbose:
                    print(f"{key} D={D:4d} engine {eng} warps {wp}: {t:.3f} s", flush=True)
            t, eng, wp = min(res)
            table[key].append([D, eng, wp])
    table["measured"] = {"batch": n, "inner_stages": stages, "inner_particles": w.settings.nparticle_slip,
                         "observations": "400 GNSS + 2000 InSAR (c2/c3)", "timings": timings}
    path = out or pkg.ENGINE_TABLE_PATH
    with open(path, "w") as f:
        json.dump(table, f, indent=1)
    return table


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--out", default=None)
    p.add_argument("--stages", type=int, default=2)
    p.add_argument("--batch", type=int, default=0, help="geometries per timed batch (default: 2 x SM count)")
    a = p.parse_args()
    from smc_inversion_fort_gb300 import build
    build.build()
    t = tune(a.stages, a.batch, a.out)
    print(json.dumps({k: t[k] for k in ("mixed", "fp64")}))


if __name__ == "__main__":
    main()
