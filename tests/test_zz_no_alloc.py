"""The allocation-free Green's build entry point, through the C ABI.

smcgpu_greens_batch_noalloc serves callers that cannot allocate device
memory while they run: applications that hand the whole GPU memory to their
own pool at start-up, and stage loops that must not pay cudaMalloc's
device-wide synchronisation.  Its scratch (the per-plane geometry records)
lives in a fixed device array instead of a buffer grown with cudaMalloc.
This test checks, on two calls in a row with different geometries, that its
output equals smcgpu_greens_batch_dev's (the tolerance of the Green's tests,
1e-12 of the column scale; the two share the kernels, so it is exact in
practice), that repeated calls change neither the device's free memory nor
torch's allocator statistics, and that a batch larger than the fixed array is
refused.

The file is named so that pytest collects it after every other test.
"""
import ctypes as C

import numpy as np
import pytest

from smc_inversion_fort_gb300.configs import make_stations, preset, random_thetas

pytestmark = pytest.mark.gpu

MAX_RECORDS = 16384


def _colwise_rel(a, b):
    scale = np.abs(b).max(axis=-1, keepdims=True)
    scale = np.where(scale == 0, 1.0, scale)
    return float((np.abs(a - b) / scale).max())


def test_noalloc_greens_matches_allocating_path(smcgpu):
    import torch
    lib = smcgpu.load_library()
    f = lib.smcgpu_greens_batch_noalloc
    f.restype = C.c_int32
    f.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.c_void_p]
    w = preset("c0")
    obs = make_stations(w, np.random.default_rng(21))
    obs["dvec"] = np.zeros(len(obs["obs_sigma"]))
    g = smcgpu.SmcGpu(w.settings)
    g.set_data(obs)
    dm = g.dims()
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    g.set_stream(stream.cuda_stream)
    for call, (n, seed) in enumerate(((300, 1), (117, 2))):
        for prec, dt in ((smcgpu.PREC_FP64, torch.float64), (smcgpu.PREC_FP32, torch.float32)):
            th = torch.from_numpy(random_thetas(w, n, seed=seed + 10 * call)).cuda()
            ref = torch.empty((n, dm["D"], dm["nobs"]), dtype=dt, device="cuda")
            out = torch.full((n, dm["D"], dm["nobs"]), float("nan"), dtype=dt, device="cuda")
            g.greens_dev(n, th.data_ptr(), ref.data_ptr(), prec)
            rc = f(g.h, n, th.data_ptr(), prec, out.data_ptr())
            assert rc == 0, lib.smcgpu_last_error(g.h).decode()
            stream.synchronize()
            a, b = out.double().cpu().numpy(), ref.double().cpu().numpy()
            assert np.isfinite(a).all()
            assert _colwise_rel(a, b) <= 1e-12
    # the point of the entry point: after a warm-up call, further calls leave
    # the device's free memory (cudaMemGetInfo) and torch's allocator untouched
    n = 300
    th = torch.from_numpy(random_thetas(w, n, seed=77)).cuda()
    out = torch.empty((n, dm["D"], dm["nobs"]), dtype=torch.float64, device="cuda")
    assert f(g.h, n, th.data_ptr(), smcgpu.PREC_FP64, out.data_ptr()) == 0
    stream.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    stats0 = torch.cuda.memory_stats()
    for _ in range(3):
        assert f(g.h, n, th.data_ptr(), smcgpu.PREC_FP64, out.data_ptr()) == 0
    stream.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    stats1 = torch.cuda.memory_stats()
    assert free1 == free0, (free0, free1)
    for k in ("allocation.all.allocated", "segment.all.allocated", "reserved_bytes.all.current"):
        assert stats1.get(k) == stats0.get(k), k
    # batches beyond the fixed array are refused with a clear error
    big = torch.zeros((MAX_RECORDS + 1, dm["ndim_fault"]), dtype=torch.float64, device="cuda")
    rc = f(g.h, MAX_RECORDS + 1, big.data_ptr(), smcgpu.PREC_FP64, big.data_ptr())
    assert rc == -1   # SMCGPU_ERR_ARG
    assert "16384" in lib.smcgpu_last_error(g.h).decode()
    torch.cuda.set_stream(torch.cuda.default_stream())
