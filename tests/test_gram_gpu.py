"""Gram products of slip_calc_gsd_gsg (smc_slip.f90:1347-1443) on the GPU
against the oracle, which follows the reference's dense Sigma_SAR^-1 products
in the reference's loop order; the GPU applies the whitening factor of
Sigma_SAR^-1 and tiles the products, so the two agree to FP64 rounding
(1e-12 of the largest entry)."""
import dataclasses

import numpy as np
import pytest

from smc_inversion_fort_gb300.configs import make_stations, preset, random_thetas, true_slip, true_theta

pytestmark = pytest.mark.gpu


def _case(w, orc, seed=2024):
    rng = np.random.default_rng(seed)
    obs = make_stations(w, rng)
    o0 = orc.Oracle(w.settings, obs)
    d = o0.greens(true_theta(w)).T @ true_slip(w)
    obs["dvec"] = d + rng.standard_normal(len(d)) * obs["obs_sigma"]
    return obs, orc.Oracle(w.settings, obs)


@pytest.mark.parametrize("name", ["tiny", "tiny-sar", "d256-sar"])
def test_gram_matches_oracle(smcgpu, orc, name):
    if name == "d256-sar":
        # 256 slip dimensions (4 x 4 column tiles) and two InSAR paths of 150
        # points (several whitening row tiles each)
        w = dataclasses.replace(preset("d256"), n_sar=300, npath=2)
    else:
        w = preset(name)
    obs, o = _case(w, orc)
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
        print(f"{name} theta {t}: A {ea:.2e} b {eb:.2e} dsd {ed:.2e}")
        assert ea < 1e-12 and eb < 1e-12 and ed < 1e-12
        assert np.array_equal(A[t], A[t].T)   # mirrored, not recomputed
