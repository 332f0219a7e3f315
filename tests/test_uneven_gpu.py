"""Per-geometry meshes (smcgpu_config.patch_km > 0): one batch of geometries
whose patch counts differ (the uneven slip dimensions of the benchmark plan's
c3), against the oracle run on each geometry's own fixed mesh.

The reference discretises every geometry inside fault_calc_likelihood
(smc_fault.f90:116-147 -> discretize_fault, init.f90:198-293), so a
geometry's mesh may differ from its neighbour's; here the patch counts are
round(length / patch_km) x round(width / patch_km).  The library splits a
batch by mesh and runs each part in the mesh's own context, all parts in
flight together, so the results must equal the fixed-mesh evaluation of each
geometry: to rounding in FP64 against the oracle (short trajectories, the
same Philox draws), and bit for bit against the library's own fixed-mesh
contexts.
"""
import dataclasses

import numpy as np
import pytest

from smc_inversion_fort_gb300.configs import (fixed_mesh, make_stations, mesh_of, preset, prior_range, random_thetas,
                                              true_slip, true_theta)

pytestmark = pytest.mark.gpu


def setup_case(orc, seed=2024):
    w = preset("tiny-uneven")
    rng = np.random.default_rng(seed)
    obs = make_stations(w, rng)
    wf = fixed_mesh(w, true_theta(w))
    d = orc.Oracle(wf.settings, obs).greens(true_theta(w)).T @ true_slip(wf)
    obs["dvec"] = d + rng.standard_normal(len(d)) * obs["obs_sigma"]
    return w, obs


def _batch(w, n=10, seed=3):
    th = np.vstack([true_theta(w)[None], random_thetas(w, n - 1, seed=seed)])
    meshes = {mesh_of(w.settings, t) for t in th}
    assert len(meshes) >= 3, meshes   # several buckets in one batch
    return th


@pytest.mark.parametrize("ntau", [1, 3])
def test_uneven_batch_matches_oracle_per_mesh(smcgpu, orc, ntau):
    w, obs = setup_case(orc)
    w.settings.ntau = ntau
    th = _batch(w)
    streams = np.arange(200, 200 + len(th), dtype=np.uint64)
    g = smcgpu.SmcGpu(w.settings, smcgpu.PREC_FP64)
    g.set_data(obs)
    got = g.fault_likelihood_trace(th, seed=13, streams=streams)
    for i in range(len(th)):
        wf = fixed_mesh(w, th[i])
        ref = orc.Oracle(wf.settings, obs).fault_likelihood(th[i], 13, int(streams[i]), trace=True)
        a, b = got["neglog"][i], ref["neglog"]
        rel = abs(a - b) / max(1.0, abs(b))
        nst = len(got["gamma"][i])
        dg = float(np.abs(got["gamma"][i] - ref["gamma"]).max()) if nst == len(ref["gamma"]) else np.inf
        print(f"theta {i} mesh {mesh_of(w.settings, th[i])}: gpu {a:.10f} oracle {b:.10f} rel {rel:.1e} "
              f"max |dgamma| {dg:.1e}")
        assert got["status"][i] == 0 and ref["status"] == 0
        assert dg <= 1e-12 and rel < 1e-9


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_uneven_batch_equals_fixed_mesh_contexts(smcgpu, orc, prec):
    """Reference trajectory length: the uneven batch equals, bit for bit, each
    geometry evaluated alone in a context of its own fixed mesh."""
    w, obs = setup_case(orc)
    p = smcgpu.PREC_FP64 if prec == "fp64" else smcgpu.PREC_MIXED
    # fixed warps per geometry: the CUDA-core engine otherwise picks them from
    # the batch size, which changes the order of its group sums
    s = dataclasses.replace(w.settings, inner_engine=smcgpu.ENGINE_MMA if prec == "mixed" else smcgpu.ENGINE_CUDA,
                            inner_warps=4)
    th = _batch(w, 12, seed=4)
    streams = np.arange(300, 300 + len(th), dtype=np.uint64)
    g = smcgpu.SmcGpu(s, p)
    g.set_data(obs)
    nl, st = g.fault_calc_likelihood(th, 17, streams)
    assert np.all(st == 0)
    for i in range(len(th)):
        nx, ne = mesh_of(s, th[i])
        gf = smcgpu.SmcGpu(dataclasses.replace(s, nxi=(nx,), neta=(ne,), patch_km=0.0), p)
        gf.set_data(obs)
        v, sv = gf.fault_calc_likelihood(th[i:i + 1], 17, streams[i:i + 1])
        gf.close()
        assert sv[0] == 0 and v[0] == nl[i], (i, v[0], nl[i])


def test_uneven_outer_smc(smcgpu, orc):
    """fault_smc_exec over a prior whose geometries span several meshes: it
    runs to gamma = 1 with every stage's batch split by mesh, and a second
    run with the same seed gives the same result."""
    w, obs = setup_case(orc)
    s = dataclasses.replace(w.settings, ntau=3, cv_outer=1.0, nparticle_slip=32)
    rg = prior_range(w)
    g = smcgpu.SmcGpu(s, smcgpu.PREC_MIXED)
    g.set_data(obs)
    parts, lik, ev, ns = g.fault_smc_exec(rg, 32, 9)
    assert ns >= 1 and np.isfinite(ev)
    assert len({mesh_of(s, t) for t in parts}) >= 1
    p2, l2, ev2, ns2 = g.fault_smc_exec(rg, 32, 9)
    assert ns2 == ns and ev2 == ev
    np.testing.assert_array_equal(p2, parts)


def test_engine_table_selects_engines(smcgpu, orc):
    """SMCGPU_ENGINE_AUTO with a table that sends every slip dimension to the
    global-matrix engine gives the same bits as that engine chosen directly;
    a table entry for another engine changes the draws' consumer and so the
    results (the table is live)."""
    w, obs = setup_case(orc)
    th = _batch(w, 8, seed=5)
    st = np.arange(8, dtype=np.uint64) + 40
    res = {}
    for name, eng, table in (("direct", smcgpu.ENGINE_GLOBAL, None),
                             ("auto", smcgpu.ENGINE_AUTO, [(1024, smcgpu.ENGINE_GLOBAL, 0)]),
                             ("auto-mma", smcgpu.ENGINE_AUTO, [(256, smcgpu.ENGINE_MMA, 0),
                                                               (1024, smcgpu.ENGINE_GLOBAL, 0)])):
        g = smcgpu.SmcGpu(dataclasses.replace(w.settings, inner_engine=eng), smcgpu.PREC_MIXED)
        if table:
            g.set_engine_table(smcgpu.PREC_MIXED, table)
        g.set_data(obs)
        res[name], s2 = g.fault_calc_likelihood(th, 3, st)
        assert np.all(s2 == 0)
        g.close()
    np.testing.assert_array_equal(res["auto"], res["direct"])
    assert not np.array_equal(res["auto-mma"], res["direct"])
    with pytest.raises(smcgpu.SmcError, match="ascend"):
        g = smcgpu.SmcGpu(w.settings, smcgpu.PREC_MIXED)
        g.set_engine_table(smcgpu.PREC_MIXED, [(64, 0, 0), (32, 3, 0)])
