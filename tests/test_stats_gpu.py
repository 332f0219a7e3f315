"""Run statistics (smcgpu_stats_*) and per-stage outer timing
(smcgpu_outer_stage_times) through the C ABI: the counters agree with what
the calls return, and recording off costs nothing and records nothing."""
import dataclasses

import numpy as np
import pytest

from smc_inversion_fort_gb300.configs import make_stations, preset, prior_range, random_thetas, true_slip, true_theta

pytestmark = pytest.mark.gpu


def _case(orc):
    w = preset("tiny")
    rng = np.random.default_rng(5)
    obs = make_stations(w, rng)
    d = orc.Oracle(w.settings, obs).greens(true_theta(w)).T @ true_slip(w)
    obs["dvec"] = d + rng.standard_normal(len(d)) * obs["obs_sigma"]
    return w, obs


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_stats_count_stages_and_trajectories(smcgpu, orc, prec):
    w, obs = _case(orc)
    w.settings.ntau = 3
    p = smcgpu.PREC_FP64 if prec == "fp64" else smcgpu.PREC_MIXED
    g = smcgpu.SmcGpu(w.settings, p)
    g.set_data(obs)
    th = np.vstack([true_theta(w)[None], random_thetas(w, 7, seed=2)])
    g.fault_calc_likelihood(th, 3, np.arange(8, dtype=np.uint64))
    assert g.stats()["nested_evals"] == 0          # off until reset
    g.stats_reset(True)
    got = g.fault_likelihood_trace(th, seed=3, streams=np.arange(8, dtype=np.uint64))
    st = g.stats()
    assert st["nested_evals"] == 8
    assert st["inner_stages"] == int(got["nstage"].sum())
    N = w.settings.nparticle_slip
    # every stage moves each of the N particles once (sampling), plus the
    # tuning pass's children of every fifth parent
    assert int(got["nstage"].sum()) * N <= st["inner_trajectories"] <= int(got["nstage"].sum()) * 2 * N
    assert 0 < st["inner_kernel_ms"] <= st["nested_ms"]
    g.stats_reset(False)
    g.fault_calc_likelihood(th, 3, np.arange(8, dtype=np.uint64))
    assert g.stats()["nested_evals"] == 0


def test_outer_stage_times(smcgpu, orc):
    w, obs = _case(orc)
    s = dataclasses.replace(w.settings, ntau=1, cv_outer=1.0, nparticle_slip=32)
    g = smcgpu.SmcGpu(s, smcgpu.PREC_MIXED)
    g.set_data(obs)
    rg = prior_range(w)
    parts, lik, ev, ns = g.fault_smc_exec(rg, 24, 5)
    sec, evals = g.outer_stage_times()
    assert len(sec) == len(evals) == ns + 1
    assert np.all(sec > 0)
    assert evals[0] == 24                     # the initial population
    assert np.all(evals[1:] >= 1)
