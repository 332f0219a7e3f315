"""Green's-function build on the GPU against the oracle's restatement of
calc_greens_func (gfunc.f90:242-348) + DC3D0.

FP64 tolerance: per basis column, max |G_gpu - G_oracle| <= 1e-12 *
max |G_oracle column| (the same entries summed in a different order).
FP32 tolerance: 2e-4 of the column scale (reported alongside)."""
import numpy as np
import pytest

from smc_inversion_fort_gb300.configs import make_stations, preset, random_thetas, true_theta

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
FP32_TOL = 2e-4


def colwise_rel(a, b):
    scale = np.abs(b).max(axis=-1, keepdims=True)
    scale = np.where(scale == 0, 1.0, scale)
    return float((np.abs(a - b) / scale).max())


@pytest.mark.parametrize("name,nth", [("tiny-nodal", 6), ("tiny", 6), ("tiny-sar", 4), ("c0", 3), ("c0-nodal", 3)])
def test_greens_fp64_matches_oracle(smcgpu, orc, name, nth):
    w = preset(name)
    obs = make_stations(w, np.random.default_rng(11))
    obs["dvec"] = np.zeros(len(obs["obs_sigma"]))
    th = np.vstack([true_theta(w)[None], random_thetas(w, nth - 1, seed=5)])
    o = orc.Oracle(w.settings, obs)
    ref = o.greens_batch(th)
    g = smcgpu.SmcGpu(w.settings)
    g.set_data(obs)
    got = g.calc_greens_func(th, smcgpu.PREC_FP64)
    assert got.shape == ref.shape
    err = colwise_rel(got, ref)
    assert err <= FP64_TOL, err
    got32 = g.calc_greens_func(th, smcgpu.PREC_FP32)
    err32 = colwise_rel(got32.astype(np.float64), ref)
    print(f"{name}: fp64 col-rel {err:.2e}  fp32 col-rel {err32:.2e}")
    assert err32 <= FP32_TOL, err32


def test_greens_c1_geometry_5x5(smcgpu, orc):
    """16x8 patches, 5x5 Gauss points, 400 three-component stations, some
    within 1 km of the trace (the Green's benchmark workload, 2 geometries)."""
    w = preset("c1")
    obs = make_stations(w, np.random.default_rng(3))
    obs["dvec"] = np.zeros(len(obs["obs_sigma"]))
    th = random_thetas(w, 2, seed=9)
    o = orc.Oracle(w.settings, obs)
    ref = o.greens_batch(th)
    g = smcgpu.SmcGpu(w.settings)
    g.set_data(obs)
    got = g.calc_greens_func(th, smcgpu.PREC_FP64)
    assert colwise_rel(got, ref) <= FP64_TOL
    got32 = g.calc_greens_func(th, smcgpu.PREC_FP32)
    assert colwise_rel(got32.astype(np.float64), ref) <= FP32_TOL


def test_greens_chunked_host_path_matches_device_path(smcgpu):
    """The host-buffer entry point (chunked, double-buffered D2H) returns the
    same bytes as the device-pointer entry point."""
    import torch
    w = preset("c0")
    obs = make_stations(w, np.random.default_rng(1))
    obs["dvec"] = np.zeros(len(obs["obs_sigma"]))
    g = smcgpu.SmcGpu(w.settings)
    g.set_data(obs)
    th = random_thetas(w, 37, seed=2)
    host = g.calc_greens_func(th)
    dth = torch.from_numpy(th).cuda()
    dm = g.dims()
    out = torch.empty((37, dm["D"], dm["nobs"]), dtype=torch.float64, device="cuda")
    g.set_stream(torch.cuda.current_stream().cuda_stream)
    g.greens_dev(37, dth.data_ptr(), out.data_ptr())
    torch.cuda.synchronize()
    np.testing.assert_array_equal(out.cpu().numpy(), host)
