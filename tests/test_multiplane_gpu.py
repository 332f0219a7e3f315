"""The reference's own fault geometry on the GPU: a bent multi-plane trace
with the nodal slip basis, against the oracle.

The reference parametrises the fault as a surface trace from (xmin, ymin)
to (xmax, ymax) through bend points, one dipping plane per segment
(get_geometry, init.f90:121-173): free bends (x_i, y_i) in theta when
fix_xbend = .false., bends at fixed x with their y in theta when
fix_xbend = .true.  Each plane carries its own node grid; DOFs sit on every
node except the bottom edge and the outer ends of the two end planes
(discretize_fault, init.f90:248-265); the smoothing Laplacian is built per
plane (gen_laplacian, init.f90:295-474).

Checked on two-plane (free bend, GNSS only and GNSS + two InSAR paths) and
three-plane (fixed bends, uneven patch counts along strike) cases:
  * Green's build: FP64 within 1e-12 of each column's scale, FP32 within 2e-4;
  * Gram products A = G^T Sigma^-1 G, b, d^T Sigma^-1 d within 1e-12;
  * the Gibbs initial population (max_stages = 0) within 1e-10;
  * nested evaluations with short trajectories (ntau = 1, 3): the same
    tempering schedule (stage count equal, exponents within 1e-9; the InSAR
    case's bisection is steeper, 1e-12 holds for the GNSS cases) and -log Z
    to 1e-9;
  * the outer SMC end to end: same stages, evidence to 1e-8, population 1e-9.
"""
import numpy as np
import pytest

from smc_inversion_fort_gb300.configs import make_stations, preset, prior_range, random_thetas, true_slip, true_theta

pytestmark = pytest.mark.gpu

CASES = ["tiny-2plane", "tiny-3plane-fix", "tiny-2plane-sar"]


def setup_case(name, orc, seed=2024):
    w = preset(name)
    rng = np.random.default_rng(seed)
    obs = make_stations(w, rng)
    o0 = orc.Oracle(w.settings, obs)
    d = o0.greens(true_theta(w)).T @ true_slip(w)
    obs["dvec"] = d + rng.standard_normal(len(d)) * obs["obs_sigma"]
    return w, obs, orc.Oracle(w.settings, obs)


def colwise_rel(a, b):
    scale = np.abs(b).max(axis=-1, keepdims=True)
    scale = np.where(scale == 0, 1.0, scale)
    return float((np.abs(a - b) / scale).max())


@pytest.mark.parametrize("name", CASES)
def test_multiplane_dims_match_oracle(smcgpu, orc, name):
    w, obs, o = setup_case(name, orc)
    g = smcgpu.SmcGpu(w.settings)
    g.set_data(obs)
    dm = g.dims()
    assert dm["D"] == o.dims["D"] == w.settings.dims()["D"]
    assert dm["ndim_fault"] == o.dims["ndim_fault"] == len(true_theta(w))


@pytest.mark.parametrize("name", CASES)
def test_multiplane_greens_matches_oracle(smcgpu, orc, name):
    w, obs, o = setup_case(name, orc)
    th = np.vstack([true_theta(w)[None], random_thetas(w, 5, seed=5)])
    ref = o.greens_batch(th)
    g = smcgpu.SmcGpu(w.settings)
    g.set_data(obs)
    got = g.calc_greens_func(th, smcgpu.PREC_FP64)
    err = colwise_rel(got, ref)
    err32 = colwise_rel(g.calc_greens_func(th, smcgpu.PREC_FP32).astype(np.float64), ref)
    print(f"{name}: fp64 col-rel {err:.2e}  fp32 col-rel {err32:.2e}")
    assert err <= 1e-12
    assert err32 <= 2e-4


@pytest.mark.parametrize("name", CASES)
def test_multiplane_gram_matches_oracle(smcgpu, orc, name):
    w, obs, o = setup_case(name, orc)
    th = np.vstack([true_theta(w)[None], random_thetas(w, 3, seed=8)])
    g = smcgpu.SmcGpu(w.settings, smcgpu.PREC_FP64)
    g.set_data(obs)
    A, b, dsd = g.gram(th)
    for t in range(len(th)):
        _, lsar, lgnss = o.hyper(th[t])
        Ar, br, dr = o.gram(o.greens(th[t]), np.exp(lsar), np.exp(lgnss))
        ea = np.abs(A[t].T - Ar).max() / np.abs(Ar).max()
        eb = np.abs(b[t] - br).max() / np.abs(br).max()
        ed = abs(dsd[t] - dr) / abs(dr)
        assert ea < 1e-12 and eb < 1e-12 and ed < 1e-12, (ea, eb, ed)


@pytest.mark.parametrize("name", CASES)
def test_multiplane_gibbs_initial_population(smcgpu, orc, name):
    w, obs, o = setup_case(name, orc)
    w.settings.max_stages = 0
    o = orc.Oracle(w.settings, obs)
    g = smcgpu.SmcGpu(w.settings, smcgpu.PREC_FP64)
    g.set_data(obs)
    for th in (true_theta(w), random_thetas(w, 1, seed=8)[0]):
        got = g.fault_likelihood_posterior(th, 3, 9)
        ref = o.fault_likelihood(th, 3, 9)
        assert got["neglog"] == 1e10 and ref["neglog"] == 1e10
        scale = np.abs(ref["particles"]).max()
        assert np.abs(got["particles"] - ref["particles"]).max() <= 1e-10 * scale
        np.testing.assert_allclose(got["likelihood"], ref["likelihood"], rtol=1e-9)
        np.testing.assert_allclose(got["prior"], ref["prior"], rtol=1e-9, atol=1e-12)


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("ntau", [1, 3])
def test_multiplane_nested_schedule_short_trajectories(smcgpu, orc, name, ntau):
    w, obs, o = setup_case(name, orc)
    w.settings.ntau = ntau
    o = orc.Oracle(w.settings, obs)
    th = np.vstack([true_theta(w)[None], random_thetas(w, 5, seed=3)])
    streams = np.arange(100, 100 + len(th), dtype=np.uint64)
    g = smcgpu.SmcGpu(w.settings, smcgpu.PREC_FP64)
    g.set_data(obs)
    got = g.fault_likelihood_trace(th, seed=11, streams=streams)
    for i in range(len(th)):
        ref = o.fault_likelihood(th[i], 11, int(streams[i]), trace=True)
        a, b = got["neglog"][i], ref["neglog"]
        rel = abs(a - b) / max(1.0, abs(b))
        nst = len(got["gamma"][i])
        dg = float(np.abs(got["gamma"][i] - ref["gamma"]).max()) if nst == len(ref["gamma"]) else np.inf
        print(f"{name} ntau {ntau} theta {i}: gpu {a:.10f} oracle {b:.10f} rel {rel:.2e} stages {nst}/"
              f"{len(ref['gamma'])} max |dgamma| {dg:.1e}")
        assert got["status"][i] == 0 and ref["status"] == 0
        assert dg <= 1e-9 and rel < 1e-9


@pytest.mark.parametrize("name", ["tiny-2plane", "tiny-3plane-fix"])
def test_multiplane_mixed_matches_fp64(smcgpu, orc, name):
    """MIXED against FP64 on the bent traces (warp-MMA engine): mean -log Z
    over 64 streams within 4 standard errors, at the true geometry."""
    w, obs, o = setup_case(name, orc)
    th = np.repeat(true_theta(w)[None], 64, 0)
    st = np.arange(64, dtype=np.uint64) + 900
    g64 = smcgpu.SmcGpu(w.settings, smcgpu.PREC_FP64)
    g64.set_data(obs)
    g32 = smcgpu.SmcGpu(w.settings, smcgpu.PREC_MIXED)
    g32.set_data(obs)
    a, sa = g64.fault_calc_likelihood(th, 41, st)
    b, sb = g32.fault_calc_likelihood(th, 41, st + 10**6)
    assert np.all(sa == 0) and np.all(sb == 0)
    se = np.sqrt((a.var(ddof=1) + b.var(ddof=1)) / len(a))
    print(name, "fp64", a.mean(), "mixed", b.mean(), "se", se)
    assert abs(a.mean() - b.mean()) < 4 * se + 1e-9


@pytest.mark.parametrize("name", ["tiny-2plane", "tiny-3plane-fix"])
def test_multiplane_outer_smc_matches_oracle(smcgpu, orc, name):
    w, obs, o = setup_case(name, orc)
    w.settings.nparticle_slip = 32
    w.settings.ntau = 1
    w.settings.cv_outer = 1.0
    o = orc.Oracle(w.settings, obs)
    rg = prior_range(w)
    # the GNSS-only cases fix log sigma2_sar and log sigma2_gnss at 0; open
    # them slightly so that the proposal covariance (smc_fault.f90:522-570)
    # has full rank and its Cholesky factor is not decided by rounding
    rg[-2:] = [[-0.5, 0.5], [-0.5, 0.5]]
    g = smcgpu.SmcGpu(w.settings, smcgpu.PREC_FP64)
    g.set_data(obs)
    parts, lik, ev, ns = g.fault_smc_exec(rg, 24, 5)
    ref = o.fault_smc(rg, 24, 5)
    print(name, "gpu evidence", ev, "stages", ns, "oracle", ref["evidence"], ref["nstage"])
    assert ns == ref["nstage"]
    assert abs(ev - ref["evidence"]) <= 1e-8 * max(1.0, abs(ref["evidence"]))
    np.testing.assert_allclose(parts, ref["particles"], rtol=1e-9, atol=1e-9)
