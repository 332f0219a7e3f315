"""The sweep schedule of the Gibbs initialisation (built on the host from the
L^T L pattern; the inner kernel's start runs it level by level) against the
oracle's dense L^T L: every slip component appears exactly once, and for every
coupled pair the earlier component sits in a strictly lower level (so no two
components of a level are coupled and a level-by-level sweep equals the
sequential sweep of slip_gen_init_particles, smc_slip.f90:207-263).  Reference
layout (nodal basis) and the rectangle (patch basis, c0 and D = 256)."""
import numpy as np
import pytest

from smc_inversion_fort_gb300.configs import make_stations, preset, true_theta


@pytest.mark.parametrize("name", ["tiny", "tiny-nodal", "c0", "c0-nodal", "d256"])
def test_gibbs_levels_reproduce_the_sequential_sweep(smcgpu, orc, name):
    w = preset(name)
    levels = smcgpu.gibbs_levels(w.settings)
    D = w.settings.dims()["D"]
    assert sorted(i for lv in levels for i in lv) == list(range(D))
    obs = make_stations(w, np.random.default_rng(1))
    obs["dvec"] = np.zeros(len(obs["obs_sigma"]))
    LL = orc.Oracle(w.settings, obs).laplacian(true_theta(w))[4]
    lvl = np.empty(D, int)
    for k, lv in enumerate(levels):
        lvl[lv] = k
    ii, jj = np.nonzero(LL)
    off = ii != jj
    lo, hi = np.minimum(ii[off], jj[off]), np.maximum(ii[off], jj[off])
    assert np.all(lvl[lo] < lvl[hi])
    print(name, "D", D, "levels", len(levels), "widest", max(len(lv) for lv in levels))
    assert len(levels) < D
