"""The global-matrix inner engine (SMCGPU_ENGINE_GLOBAL) against the oracle.

This engine keeps the stage matrix M = gamma A + L^T L / alpha^2 of each
geometry in global memory and streams it once per leapfrog step, so it runs
any slip dimension up to 1024 in both precisions: the FP64 path above 128
dimensions, the c2 slip size in FP64 and the c4 slip size (32 x 16 patches x
2 components = 1024).  It is also selectable at any size, which lets its
FP64 arithmetic be pinned exactly against the oracle on the small cases.

FP64 follows the reference's algebra with the same Philox draws as the
oracle: with short trajectories (ntau = 1, 3) the tempering schedules agree
to 1e-12 and -log Z to 1e-9; at longer trajectories the comparison is
statistical (mean and median -log Z within 4 standard errors over
independent streams; the median of n draws has standard error about
1.2533 sd / sqrt(n)).
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


def _agree(a, b, k=4.0):
    a, b = np.atleast_2d(a), np.atleast_2d(b)
    n = a.shape[1]
    se = np.sqrt((a.var(1, ddof=1) + b.var(1, ddof=1)) / n)
    print("a mean/median", a.mean(1), np.median(a, 1), "\nb mean/median", b.mean(1), np.median(b, 1), "\nse", se)
    assert np.all(np.abs(a.mean(1) - b.mean(1)) < k * se + 1e-9)
    assert np.all(np.abs(np.median(a, 1) - np.median(b, 1)) < k * 1.2533 * se + 1e-9)


@pytest.mark.parametrize("name", ["tiny", "tiny-nodal", "tiny-sar", "tiny-2plane"])
@pytest.mark.parametrize("ntau", [1, 3])
def test_global_fp64_schedule_short_trajectories(smcgpu, orc, name, ntau):
    w, obs, o = setup_case(name, orc)
    s = dataclasses.replace(w.settings, ntau=ntau, inner_engine=smcgpu.ENGINE_GLOBAL)
    o = orc.Oracle(s, obs)
    th = np.vstack([true_theta(w)[None], random_thetas(w, 5, seed=3)])
    streams = np.arange(100, 100 + len(th), dtype=np.uint64)
    g = smcgpu.SmcGpu(s, smcgpu.PREC_FP64)
    g.set_data(obs)
    got = g.fault_likelihood_trace(th, seed=11, streams=streams)
    for i in range(len(th)):
        ref = o.fault_likelihood(th[i], 11, int(streams[i]), trace=True)
        a, b = got["neglog"][i], ref["neglog"]
        rel = abs(a - b) / max(1.0, abs(b))
        nst = len(got["gamma"][i])
        dg = float(np.abs(got["gamma"][i] - ref["gamma"]).max()) if nst == len(ref["gamma"]) else np.inf
        print(f"{name} ntau {ntau} theta {i}: gpu {a:.10f} oracle {b:.10f} rel {rel:.2e} max |dgamma| {dg:.1e}")
        assert got["status"][i] == 0 and ref["status"] == 0
        assert dg <= (1e-9 if "sar" in name else 1e-12) and rel < 1e-9


def test_global_fp64_statistics_match_oracle(smcgpu, orc):
    """Reference trajectory length (ntau = 50): mean and median -log Z over
    24 streams against the oracle's, at the true geometry."""
    w, obs, o = setup_case("tiny", orc)
    s = dataclasses.replace(w.settings, inner_engine=smcgpu.ENGINE_GLOBAL)
    n = 24
    th = np.repeat(true_theta(w)[None], n, 0)
    streams = np.arange(7000, 7000 + n, dtype=np.uint64)
    g = smcgpu.SmcGpu(s, smcgpu.PREC_FP64)
    g.set_data(obs)
    a, sa = g.fault_calc_likelihood(th, 31, streams)
    b, sb = o.fault_likelihood_batch(th, 31, streams)
    assert np.all(sa == 0) and np.all(sb == 0)
    _agree(a, b)


def test_global_mixed_matches_fp64(smcgpu, orc):
    """MIXED global-matrix engine against the FP64 CUDA-core engine: 48
    streams at each of 4 geometries."""
    w, obs, o = setup_case("tiny", orc)
    th = np.vstack([true_theta(w)[None], random_thetas(w, 3, seed=4)])
    reps = 48
    th_rep = np.repeat(th, reps, axis=0)
    streams = np.arange(len(th_rep), dtype=np.uint64) + 5000
    g64 = smcgpu.SmcGpu(w.settings, smcgpu.PREC_FP64)
    g64.set_data(obs)
    g32 = smcgpu.SmcGpu(dataclasses.replace(w.settings, inner_engine=smcgpu.ENGINE_GLOBAL), smcgpu.PREC_MIXED)
    g32.set_data(obs)
    a, sa = g64.fault_calc_likelihood(th_rep, 21, streams)
    b, sb = g32.fault_calc_likelihood(th_rep, 21, streams + 10**6)
    assert np.all(sa == 0) and np.all(sb == 0)
    _agree(a.reshape(-1, reps), b.reshape(-1, reps))


def test_global_mixed_matches_mma_c0(smcgpu, orc):
    """c0 (D = 64, 500 inner particles): the global-matrix engine against the
    warp-MMA engine, both MIXED, 64 streams at the true geometry."""
    w, obs, o = setup_case("c0", orc)
    th = np.repeat(true_theta(w)[None], 64, 0)
    st = np.arange(64, dtype=np.uint64) + 700
    res = []
    for eng in (smcgpu.ENGINE_MMA, smcgpu.ENGINE_GLOBAL):
        g = smcgpu.SmcGpu(dataclasses.replace(w.settings, inner_engine=eng), smcgpu.PREC_MIXED)
        g.set_data(obs)
        v, s = g.fault_calc_likelihood(th, 17, st + (0 if eng == smcgpu.ENGINE_MMA else 10**6))
        assert np.all(s == 0)
        res.append(v)
        g.close()
    _agree(res[0], res[1])


@pytest.mark.parametrize("name", ["d256", "d512", "d1024"])
def test_fp64_large_d_matches_oracle(smcgpu, orc, name):
    """FP64 above 128 slip dimensions (global-matrix engine) against the
    oracle: -log Z over 16 streams at the true geometry."""
    w, obs, o = setup_case(name, orc)
    n = 16
    th = np.repeat(true_theta(w)[None], n, 0)
    streams = np.arange(n, dtype=np.uint64) + 9500
    g = smcgpu.SmcGpu(w.settings, smcgpu.PREC_FP64)
    g.set_data(obs)
    a, sa = g.fault_calc_likelihood(th, 47, streams)
    b, sb = o.fault_likelihood_batch(th, 47, streams + 10**6)
    assert np.all(sa == 0) and np.all(sb == 0)
    _agree(a, b)


def test_fp64_large_d_short_trajectories_exact(smcgpu, orc):
    """D = 512 in FP64 with ntau = 1: the tempering schedule and -log Z equal
    the oracle's (same draws, FP64 rounding differences only)."""
    w, obs, o = setup_case("d512", orc)
    s = dataclasses.replace(w.settings, ntau=1)
    o = orc.Oracle(s, obs)
    g = smcgpu.SmcGpu(s, smcgpu.PREC_FP64)
    g.set_data(obs)
    th = np.vstack([true_theta(w)[None], random_thetas(w, 1, seed=2)])
    streams = np.array([31, 32], np.uint64)
    got = g.fault_likelihood_trace(th, seed=5, streams=streams)
    for i in range(2):
        ref = o.fault_likelihood(th[i], 5, int(streams[i]), trace=True)
        rel = abs(got["neglog"][i] - ref["neglog"]) / max(1.0, abs(ref["neglog"]))
        print("d512 ntau 1", got["neglog"][i], ref["neglog"], rel, got["nstage"][i], len(ref["gamma"]))
        assert got["nstage"][i] == len(ref["gamma"])
        assert np.abs(got["gamma"][i] - ref["gamma"]).max() <= 1e-9 and rel < 1e-9


@pytest.mark.parametrize("name", ["d512", "d1024"])
def test_mixed_large_d_matches_oracle(smcgpu, orc, name):
    """MIXED at 512 and 1024 slip dimensions (32 x 16 patches: the c4 slip
    size) against the FP64 oracle: -log Z over 16 streams at the true geometry."""
    w, obs, o = setup_case(name, orc)
    assert w.settings.dims()["D"] == {"d512": 512, "d1024": 1024}[name]
    n = 16
    th = np.repeat(true_theta(w)[None], n, 0)
    streams = np.arange(n, dtype=np.uint64) + 9700
    g = smcgpu.SmcGpu(w.settings, smcgpu.PREC_MIXED)
    g.set_data(obs)
    a, sa = g.fault_calc_likelihood(th, 53, streams)
    b, sb = o.fault_likelihood_batch(th, 53, streams + 10**6)
    assert np.all(sa == 0) and np.all(sb == 0)
    _agree(a, b)


def test_size_limits_are_errors(smcgpu, orc):
    """Beyond 1024 slip dimensions (33 x 16 patches x 2) the call fails with a
    clear message in both precisions, before any launch; no fallback."""
    w, obs, o = setup_case("d1056", orc)
    for prec, name in ((smcgpu.PREC_FP64, "FP64"), (smcgpu.PREC_MIXED, "MIXED")):
        g = smcgpu.SmcGpu(w.settings, prec)
        g.set_data(obs)
        with pytest.raises(smcgpu.SmcError, match=f"{name} inner kernel \\(D <= 1024\\)"):
            g.fault_calc_likelihood(true_theta(w)[None], 1, np.zeros(1, np.uint64))
