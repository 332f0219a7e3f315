"""Failure paths through the C ABI, injected on the host: bad observations,
degenerate or non-finite geometries, and settings that drive the inner SMC
into its caps.  Every call must return normally with the documented status
code or per-geometry status bits, and the context must stay usable.

Reference behaviour kept: the stage cap returns neglog = 1e10
(smc_slip.f90:1557-1560); the reflection loop (smc_slip.f90:787-799), which
the reference runs without a bound, stops after 10^6 reflections with
SMCGPU_ST_REFLECT_CAP (the oracle has the same cap); the gamma bisection,
which the reference also runs without a bound (smc_slip.f90:333-365), stops
after 2000 steps with SMCGPU_ST_BISECT_CAP.  No GPU fault is provoked: every
case is a valid launch on valid memory.
"""
import dataclasses

import numpy as np
import pytest

from smc_inversion_fort_gb300.configs import make_stations, preset, random_thetas, true_slip, true_theta

pytestmark = pytest.mark.gpu


def _case(orc, name="tiny", seed=2024):
    w = preset(name)
    rng = np.random.default_rng(seed)
    obs = make_stations(w, rng)
    o0 = orc.Oracle(w.settings, obs)
    d = o0.greens(true_theta(w)).T @ true_slip(w)
    obs["dvec"] = d + rng.standard_normal(len(d)) * obs["obs_sigma"]
    return w, obs


@pytest.mark.parametrize("field,row,value", [("dvec", 3, np.nan), ("dvec", 0, np.inf), ("obs_sigma", 5, 0.0),
                                             ("obs_sigma", 2, -1.0), ("obs_points", 4, np.nan),
                                             ("obs_unitvec", 7, np.inf)])
def test_set_data_rejects_bad_observations(smcgpu, orc, field, row, value):
    w, obs = _case(orc)
    g = smcgpu.SmcGpu(w.settings)
    bad = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in obs.items()}
    a = bad[field]
    if a.ndim == 2:
        a[row, 0] = value
    else:
        a[row] = value
    with pytest.raises(smcgpu.SmcError) as ei:
        g.set_data(bad)
    assert f"row {row + 1}" in str(ei.value)
    # the context is still usable with good data
    g.set_data(obs)
    nl, st = g.fault_calc_likelihood(true_theta(w)[None], 3, np.array([1], np.uint64))
    assert st[0] == 0 and np.isfinite(nl[0])


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_nonfinite_theta_sets_status_and_spares_the_batch(smcgpu, orc, prec):
    """A NaN entry in one geometry gives that geometry SMCGPU_ST_NONFINITE and
    neglog = NaN; the other geometries of the batch equal their values when
    evaluated alone."""
    w, obs = _case(orc)
    w.settings.ntau = 3
    p = smcgpu.PREC_FP64 if prec == "fp64" else smcgpu.PREC_MIXED
    g = smcgpu.SmcGpu(w.settings, p)
    g.set_data(obs)
    th = np.vstack([true_theta(w)[None], random_thetas(w, 3, seed=2)])
    st = np.arange(4, dtype=np.uint64) + 40
    ref, sref = g.fault_calc_likelihood(th, 7, st)
    bad = th.copy()
    bad[1, 3] = np.nan          # length of geometry 1
    nl, stat = g.fault_calc_likelihood(bad, 7, st)
    assert stat[1] & smcgpu.ST_NONFINITE and np.isnan(nl[1])
    for i in (0, 2, 3):
        assert stat[i] == sref[i] == 0
        assert nl[i] == ref[i]
    # Green's columns of the NaN geometry are NaN, the others unchanged
    G = g.calc_greens_func(bad)
    G0 = g.calc_greens_func(th)
    assert np.isnan(G[1]).any()
    np.testing.assert_array_equal(G[[0, 2, 3]], G0[[0, 2, 3]])


def test_zero_length_plane_is_nonfinite(smcgpu, orc):
    """A two-plane trace whose bend point sits on the trace start: the first
    plane has zero length, its patch width and Laplacian weights 1/dxi^2 are
    infinite, and the evaluation returns SMCGPU_ST_NONFINITE."""
    w, obs = _case(orc, "tiny-2plane")
    w.settings.ntau = 3
    g = smcgpu.SmcGpu(w.settings)
    g.set_data(obs)
    th = true_theta(w).copy()
    th[2], th[3] = w.settings.xmin, th[0]     # bend (x, y) = (xmin, ymin)
    nl, stat = g.fault_calc_likelihood(np.vstack([th, true_theta(w)]), 5, np.array([1, 2], np.uint64))
    assert stat[0] & smcgpu.ST_NONFINITE
    assert stat[1] == 0 and np.isfinite(nl[1])


def test_source_above_surface_gives_zero_columns(smcgpu, orc):
    """A rectangle whose top edge is above the surface (top depth -6 km):
    DC3D0 returns zeros for sources above the half-space (depth < 0,
    DC3Dfortran.f90:66-69), so the columns of the patches whose Gauss points
    are all above the surface are exactly zero, as in the oracle, and the
    nested evaluation is finite."""
    w, obs = _case(orc)
    g = smcgpu.SmcGpu(w.settings)
    g.set_data(obs)
    th = true_theta(w).copy()
    th[2] = -6.0                 # top depth
    o = orc.Oracle(w.settings, obs)
    ref = o.greens(th)
    got = g.calc_greens_func(th[None])[0]
    zero_ref = np.all(ref == 0.0, axis=1)
    assert zero_ref.any()
    assert np.array_equal(np.all(got == 0.0, axis=1), zero_ref)
    scale = np.abs(ref).max(axis=-1, keepdims=True)
    scale = np.where(scale == 0, 1.0, scale)
    assert float((np.abs(got - ref) / scale).max()) <= 1e-12
    w.settings.ntau = 3
    g2 = smcgpu.SmcGpu(w.settings)
    g2.set_data(obs)
    nl, stat = g2.fault_calc_likelihood(th[None], 5, np.array([3], np.uint64))
    assert stat[0] == 0 and np.isfinite(nl[0])


def test_stage_cap_sentinel(smcgpu, orc):
    """max_stages = 2: every evaluation stops at the cap with neglog = 1e10
    and SMCGPU_ST_STAGE_CAP (smc_slip.f90:1557-1560, which caps at 200)."""
    w, obs = _case(orc)
    for p in (smcgpu.PREC_FP64, smcgpu.PREC_MIXED):
        s = dataclasses.replace(w.settings, max_stages=2, ntau=3)
        g = smcgpu.SmcGpu(s, p)
        g.set_data(obs)
        # a geometry far from the truth needs many stages
        th = random_thetas(w, 8, seed=31)
        nl, stat = g.fault_calc_likelihood(th, 9, np.arange(8, dtype=np.uint64))
        capped = (stat & smcgpu.ST_STAGE_CAP) != 0
        assert capped.any()
        assert np.all(nl[capped] == 1e10)
        assert np.all(stat[~capped] == 0)


def test_unreachable_cv_target_hits_bisection_cap(smcgpu, orc):
    """A negative CV target cannot be met by any tempering step (the weights'
    CV is never negative), so the FP64 bisection stops at its 2000-step cap
    in every stage, gamma stays put, and the stage cap ends the evaluation:
    SMCGPU_ST_BISECT_CAP | SMCGPU_ST_STAGE_CAP, neglog = 1e10."""
    w, obs = _case(orc)
    s = dataclasses.replace(w.settings, cv_inner=-1.0, max_stages=3, ntau=1)
    g = smcgpu.SmcGpu(s, smcgpu.PREC_FP64)
    g.set_data(obs)
    nl, stat = g.fault_calc_likelihood(true_theta(w)[None], 2, np.array([5], np.uint64))
    assert stat[0] & smcgpu.ST_BISECT_CAP
    assert stat[0] & smcgpu.ST_STAGE_CAP
    assert nl[0] == 1e10


def test_reflection_cap(smcgpu, orc):
    """max_slip = 1e-9 m: a tuning step of size up to 1 carries an entry 10^7
    box widths out, so the FP64 reflection loop (smc_slip.f90:787-799) stops
    at its 10^6 cap with SMCGPU_ST_REFLECT_CAP, as the oracle does on the same
    draws; the evaluation still returns."""
    w, obs = _case(orc)
    s = dataclasses.replace(w.settings, max_slip=1e-9, max_stages=1, ntau=1)
    g = smcgpu.SmcGpu(s, smcgpu.PREC_FP64)
    g.set_data(obs)
    nl, stat = g.fault_calc_likelihood(true_theta(w)[None], 3, np.array([9], np.uint64))
    ref = orc.Oracle(s, obs).fault_likelihood(true_theta(w), 3, 9)
    assert ref["status"] & smcgpu.ST_REFLECT_CAP
    assert stat[0] & smcgpu.ST_REFLECT_CAP
    assert np.isfinite(nl[0])
