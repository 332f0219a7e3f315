"""Post-processing of sampled geometries (main.f90:553-830): calc_slip_map
(mean inner slip per geometry) and point_cloud (sub-patch points in global
coordinates with interpolated slip), GPU against the oracle."""
import os

import numpy as np
import pytest

from smc_inversion_fort_gb300.configs import make_stations, preset, random_thetas, true_slip, true_theta


def _case(orc, name):
    w = preset(name)
    rng = np.random.default_rng(3)
    obs = make_stations(w, rng)
    o0 = orc.Oracle(w.settings, obs)
    obs["dvec"] = o0.greens(true_theta(w)).T @ true_slip(w) + rng.standard_normal(len(obs["obs_sigma"])) * obs["obs_sigma"]
    return w, obs, orc.Oracle(w.settings, obs)


def test_oracle_point_cloud_geometry(orc):
    """Sub-point centres of a plane average to the plane centre; a uniform
    slip interpolates to itself; |u| is the norm of (uxi, ueta)."""
    w, obs, o = _case(orc, "tiny-nodal")
    th = true_theta(w)
    nn = o.dims["nnode"]
    slip = np.tile([0.3, -1.2], nn)
    pts = o.point_cloud(th, slip, 4)
    assert pts.shape == (o.dims["npatch"], 4, 4, 6)
    np.testing.assert_allclose(pts[..., 3], 0.3, atol=1e-15)
    np.testing.assert_allclose(pts[..., 4], -1.2, atol=1e-15)
    np.testing.assert_allclose(pts[..., 5], np.hypot(0.3, 1.2), rtol=1e-15)
    plane = o.plane_params(th)[0, :3]
    np.testing.assert_allclose(pts[..., :3].reshape(-1, 3).mean(0), plane, atol=1e-10)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["tiny-nodal", "tiny"])
def test_point_cloud_matches_oracle(smcgpu, orc, name, tmp_path):
    w, obs, o = _case(orc, name)
    g = smcgpu.SmcGpu(w.settings)
    g.set_data(obs)
    th = np.vstack([true_theta(w)[None], random_thetas(w, 4, seed=9)])
    rng = np.random.default_rng(4)
    D = g.dims()["D"]
    slip_dof = rng.uniform(0, w.settings.max_slip, (len(th), D))
    nodes = g.slip_to_nodes(slip_dof)
    pts = g.point_cloud(th, nodes, 8)
    for i in range(len(th)):
        ref = o.point_cloud(th[i], nodes[i], 8)
        np.testing.assert_allclose(pts[i], ref, rtol=1e-12, atol=1e-12)
    # point_cloud's files: one per plane, 6 x f12.5 per record
    g.write_point_cloud(str(tmp_path / "points_"), pts)
    lines = open(tmp_path / "points_1").read().splitlines()
    assert len(lines) == len(th) * g.mesh_counts()["npatch"] * 64
    assert all(len(ln) == 72 for ln in lines)
    v = [float(lines[0][k:k + 12]) for k in range(0, 72, 12)]
    np.testing.assert_allclose(v, pts[0, 0, 0, 0], atol=6e-6)


@pytest.mark.gpu
def test_slip_map_matches_oracle(smcgpu, orc, tmp_path):
    """calc_slip_map: the mean of the final inner population; with short
    trajectories the GPU population equals the oracle's, so the means do."""
    w, obs, o = _case(orc, "tiny-nodal")
    w.settings.ntau = 1
    o = orc.Oracle(w.settings, obs)
    g = smcgpu.SmcGpu(w.settings)
    g.set_data(obs)
    th = np.vstack([true_theta(w)[None], random_thetas(w, 3, seed=2)])
    streams = np.arange(40, 40 + len(th), dtype=np.uint64)
    mean, nl, st = g.slip_map(th, 8, streams)
    assert np.all(st == 0)
    for i in range(len(th)):
        ref = o.fault_likelihood(th[i], 8, int(streams[i]))
        np.testing.assert_allclose(mean[i], ref["particles"].mean(0), rtol=1e-9, atol=1e-12)
        assert abs(nl[i] - ref["neglog"]) <= 1e-9 * abs(ref["neglog"])
    path = str(tmp_path / "mapslip.dat")
    g.write_slip_map(path, mean)
    lines = open(path).read().splitlines()
    nn = g.mesh_counts()["nnode"]
    assert len(lines) == len(th) and all(len(ln) == 12 * 2 * nn for ln in lines)
    first = np.array([float(lines[0][k:k + 12]) for k in range(0, 24 * nn, 12)])
    np.testing.assert_allclose(first, g.slip_to_nodes(mean[:1])[0], atol=6e-6)
