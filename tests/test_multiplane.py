"""Oracle geometry of the reference's multi-plane trace (CPU): plane records
(get_geometry, init.f90:121-173, and the fault centre of calc_greens_func,
gfunc.f90:283-296), DOF counts (main.f90:209-238) and the per-plane
Laplacian (gen_laplacian, init.f90:295-474) on the multi-plane workloads the
GPU tests use."""
import numpy as np
import pytest

from smc_inversion_fort_gb300.configs import make_stations, preset, random_thetas, true_theta

CASES = ["tiny-2plane", "tiny-3plane-fix", "tiny-2plane-sar"]


def _oracle(orc, name):
    w = preset(name)
    obs = make_stations(w, np.random.default_rng(1))
    obs["dvec"] = np.zeros(len(obs["obs_sigma"]))
    return w, orc.Oracle(w.settings, obs)


def _trace(w, th):
    """Trace vertices (x, y) from theta, as get_geometry reads them."""
    s = w.settings
    n = s.nplane
    xs, ys = [s.xmin], [th[0]]
    for k in range(1, n):
        if s.layout == 0:
            xs.append(th[2 * k]); ys.append(th[2 * k + 1])
        else:
            xs.append(s.xbend[k - 1]); ys.append(th[k + 1])
    xs.append(s.xmax); ys.append(th[1])
    dips = th[2 * n + 1 - 1: 3 * n] if s.layout == 0 else th[n + 1: 2 * n + 1]
    return np.array(xs), np.array(ys), np.array(dips)


@pytest.mark.parametrize("name", CASES)
def test_plane_records_follow_the_trace(orc, name):
    w, o = _oracle(orc, name)
    s = w.settings
    for th in np.vstack([true_theta(w)[None], random_thetas(w, 4, seed=3)]):
        xs, ys, dips = _trace(w, th)
        pl = o.plane_params(th)          # xf, yf, zf, strike, dip, lxi, leta per plane
        for p in range(s.nplane):
            dx, dy = xs[p + 1] - xs[p], ys[p + 1] - ys[p]
            assert pl[p, 5] == pytest.approx(np.hypot(dx, dy), rel=1e-14)
            assert pl[p, 3] == pytest.approx(np.degrees(np.arctan2(dx, dy)), abs=1e-12)
            assert pl[p, 4] == pytest.approx(dips[p], abs=1e-12)
            assert pl[p, 6] == pytest.approx(-s.zmin / np.sin(np.radians(dips[p])), rel=1e-14)
            assert pl[p, 2] == pytest.approx(s.zmin / 2.0, abs=1e-14)


@pytest.mark.parametrize("name", CASES)
def test_dof_counts_and_per_plane_laplacian(orc, name):
    w, o = _oracle(orc, name)
    s = w.settings
    # DOF rule of discretize_fault: no DOF on the bottom node row of any
    # plane, nor on the outer end columns of the first and last plane
    nd = 0
    for p in range(s.nplane):
        c = (s.nxi[p] + 1) * s.neta[p]
        if p == 0:
            c -= s.neta[p]
        if p == s.nplane - 1:
            c -= s.neta[p]
        nd += c
    assert o.dims["ndof"] == nd == w.settings.dims()["ndof"]
    assert o.dims["D"] == 2 * nd
    li, lv, lti, ltv, ll = o.laplacian(true_theta(w))
    # rows of L are node components, columns DOF components; a plane's rows
    # only reach DOFs of the same plane (the Laplacian is built per plane)
    node_plane = np.concatenate([[p] * ((s.nxi[p] + 1) * (s.neta[p] + 1)) for p in range(s.nplane)])
    dof_plane = []
    for p in range(s.nplane):
        for j in range(s.neta[p] + 1):
            for i in range(s.nxi[p] + 1):
                if j == 0 or (p == 0 and i == 0) or (p == s.nplane - 1 and i == s.nxi[p]):
                    continue
                dof_plane.append(p)
    dof_plane = np.array(dof_plane)
    for r in range(li.shape[0]):
        for q in range(9):
            c = li[r, q]
            if c >= 0 and lv[r, q] != 0.0:
                assert dof_plane[c // 2] == node_plane[r // 2]
    assert np.allclose(ll, ll.T, rtol=0, atol=1e-12 * np.abs(ll).max())
