"""Nested likelihood above 128 slip dimensions, warp-MMA engine (MIXED).

Beyond 128 dimensions the stage matrix of the inner HMC step no longer fits in
shared memory; the warp-MMA engine then streams it from global memory in
fragment order.  Its results are checked against the FP64 oracle (D = 256)
and against the independent FP32 CUDA-core engine (D = 160), statistically
over independent
streams: the mean and the median -log Z agree within 4 standard errors (the
median of n draws has standard error about 1.2533 sd / sqrt(n)).
"""
import dataclasses

import numpy as np
import pytest

from smc_inversion_fort_gb300.configs import make_stations, preset, random_thetas, true_slip, true_theta

pytestmark = pytest.mark.gpu


def setup_case(name, orc, seed=2024):
    w = preset(name)
    rng = np.random.default_rng(seed)
    obs = make_stations(w, rng)
    o0 = orc.Oracle(w.settings, obs)
    d = o0.greens(true_theta(w)).T @ true_slip(w)
    obs["dvec"] = d + rng.standard_normal(len(d)) * obs["obs_sigma"]
    return w, obs, orc.Oracle(w.settings, obs)


def _agree(a, b):
    a, b = np.atleast_2d(a), np.atleast_2d(b)
    n = a.shape[1]
    se = np.sqrt((a.var(1, ddof=1) + b.var(1, ddof=1)) / n)
    print("a mean/median", a.mean(1), np.median(a, 1), "\nb mean/median", b.mean(1), np.median(b, 1), "\nse", se)
    assert np.all(np.abs(a.mean(1) - b.mean(1)) < 4 * se + 1e-9)
    assert np.all(np.abs(np.median(a, 1) - np.median(b, 1)) < 4 * 1.2533 * se + 1e-9)


def test_d256_mixed_matches_oracle(smcgpu, orc):
    """D = 256 (16 x 8 patches, the c2 slip size): streamed-matrix MMA engine
    against the FP64 oracle on the true geometry and one prior draw."""
    w, obs, o = setup_case("d256", orc)
    assert w.settings.dims()["D"] == 256
    th = np.vstack([true_theta(w)[None], random_thetas(w, 1, seed=5)])
    reps = 64
    th_rep = np.repeat(th, reps, axis=0)
    streams = np.arange(len(th_rep), dtype=np.uint64) + 9100
    g = smcgpu.SmcGpu(w.settings, smcgpu.PREC_MIXED)
    g.set_data(obs)
    a, sa = g.fault_calc_likelihood(th_rep, 41, streams)
    b, sb = o.fault_likelihood_batch(th_rep, 41, streams + 10**6)
    assert np.all(sa == 0) and np.all(sb == 0)
    _agree(a.reshape(-1, reps), b.reshape(-1, reps))


def test_d160_mma_matches_cuda_cores(smcgpu, orc):
    """D = 160: the streamed-matrix MMA engine against the FP32 CUDA-core
    engine (shared-memory matrix), two independent MIXED implementations."""
    w, obs, o = setup_case("d160", orc)
    assert w.settings.dims()["D"] == 160
    th = np.vstack([true_theta(w)[None], random_thetas(w, 2, seed=6)])
    reps = 64
    th_rep = np.repeat(th, reps, axis=0)
    streams = np.arange(len(th_rep), dtype=np.uint64) + 9300
    res = []
    for eng in (smcgpu.ENGINE_MMA, smcgpu.ENGINE_CUDA):
        g = smcgpu.SmcGpu(dataclasses.replace(w.settings, inner_engine=eng), smcgpu.PREC_MIXED)
        g.set_data(obs)
        v, st = g.fault_calc_likelihood(th_rep, 43, streams + (0 if eng == smcgpu.ENGINE_MMA else 10**6))
        assert np.all(st == 0)
        res.append(v.reshape(-1, reps))
        g.close()
    _agree(res[0], res[1])


def test_d256_posterior_mean_matches_oracle(smcgpu, orc):
    """Posterior mean slip of the final inner population at D = 256 against
    the oracle's, averaged over independent streams: within 4 standard errors
    per patch, or 2% of the peak slip."""
    w, obs, o = setup_case("d256", orc)
    th = true_theta(w)
    g = smcgpu.SmcGpu(w.settings, smcgpu.PREC_MIXED)
    g.set_data(obs)
    n = 16
    mg = np.array([g.fault_likelihood_posterior(th, 51, 300 + k)["particles"].mean(0) for k in range(n)])
    mr = np.array([o.fault_likelihood(th, 51, 500 + k)["particles"].mean(0) for k in range(n)])
    se = np.sqrt((mg.var(0, ddof=1) + mr.var(0, ddof=1)) / n)
    diff = np.abs(mg.mean(0) - mr.mean(0))
    print("max |diff|", diff.max(), "max se", se.max())
    assert np.all(diff < 4 * se + 0.02 * true_slip(w).max())
