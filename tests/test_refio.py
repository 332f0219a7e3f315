"""Readers of the reference's input files (io.cpp via refio.py).

The files are written here in the reference's formats (setting.dat as read
by main.f90:107-157, observation rows as read by init.f90:24-80, range.dat as
read by main.f90:497-502) and must come back exactly; Fortran list-directed
forms (commas, blank records, r*v repeats, D exponents, quoted strings, the
"/" terminator, .true./F logicals) are covered.  The GPU test runs main.f90's
shipped mode from such a directory.
"""
import os

import numpy as np
import pytest

from smc_inversion_fort_gb300.configs import make_stations, preset, prior_range, true_slip, true_theta

SETTING = """# number of fault planes
{nplane}
# fix-xbend
{fix}
# xbend
{xbend}

# number of samples for fault
{nfault}
# number of samples for slip
{nslip}

# observation path
{obs}
# number of SAR paths
{npath}
# output directory path
{out}

# max slip(m)
{max_slip}

# nxi
{nxi}
# neta
{neta}

# xmin
{xmin}
# xmax
{xmax}
# zmin
{zmin}

# GSMC
{gsmc}
"""


def write_setting(path, **kw):
    d = dict(nplane=1, fix=".false.", xbend="", nfault=16, nslip=64, obs="data/observation.dat", npath=2,
             out="output/", max_slip="4.0d0", nxi="4", neta="3", xmin="-10.0", xmax="10.0", zmin="-10.0",
             gsmc=".false.")
    d.update(kw)
    with open(path, "w") as f:
        f.write(SETTING.format(**d))


def write_observation(path, obs, npath, blank_every=0):
    nsar = int(obs["nsar_index"][-1] - 1) if npath else 0
    idx = obs["nsar_index"]
    with open(path, "w") as f:
        f.write("x y ex ey ez dlos sigma type\n")
        for i in range(len(obs["dvec"])):
            if i < nsar:
                p = int(np.searchsorted(idx, i + 1, side="right")) - 1
                typ = f"InSAR_path{p + 1}"
            else:
                typ = "GNSS"
            v = [obs["obs_points"][i, 0], obs["obs_points"][i, 1], *obs["obs_unitvec"][i], obs["dvec"][i],
                 obs["obs_sigma"][i]]
            f.write(" ".join(repr(float(x)) for x in v) + f" {typ}\n")
            if blank_every and i % blank_every == 0:
                f.write("\n")


def tiny_sar_obs(seed=2024):
    w = preset("tiny-sar")
    obs = make_stations(w, np.random.default_rng(seed))
    obs["dvec"] = np.random.default_rng(seed + 1).standard_normal(len(obs["obs_sigma"])) * obs["obs_sigma"]
    return w, obs


def test_read_settings(smcgpu, tmp_path):
    from smc_inversion_fort_gb300 import refio
    p = str(tmp_path / "setting.dat")
    write_setting(p)
    st = refio.read_settings(p)
    assert st["nplane"] == 1 and st["fix_xbend"] is False and st["xbend"] == []
    assert st["nparticle_fault"] == 16 and st["nparticle_slip"] == 64
    assert st["observation_path"] == "data/observation.dat" and st["output_dir"] == "output/"
    assert st["npath"] == 2 and st["max_slip"] == 4.0
    assert st["nxi"] == [4] and st["neta"] == [3]
    assert (st["xmin"], st["xmax"], st["zmin"]) == (-10.0, 10.0, -10.0)
    assert st["gsmc"] is False
    # three planes, fixed bends, list-directed forms
    write_setting(p, nplane="3", fix="T", xbend="-3.5d0, 4.25", nxi="3*5", neta="2 2,\n 3", gsmc=".TRUE.",
                  max_slip="2.5E0")
    st = refio.read_settings(p)
    assert st["nplane"] == 3 and st["fix_xbend"] is True and st["xbend"] == [-3.5, 4.25]
    assert st["nxi"] == [5, 5, 5] and st["gsmc"] is True and st["max_slip"] == 2.5
    # the neta list continues on the next record; that READ consumes both
    # records, so the fields after it still line up
    assert st["neta"] == [2, 2, 3] and st["zmin"] == -10.0


def test_settings_to_config(smcgpu, tmp_path):
    from smc_inversion_fort_gb300 import refio
    p = str(tmp_path / "setting.dat")
    write_setting(p, nplane="2", fix="F", xbend="1.5", nxi="4 5", neta="3 3")
    s = refio.settings_to_smc(refio.read_settings(p))
    assert (s.layout, s.basis, s.nplane, s.nxi, s.neta, s.xbend) == (0, 0, 2, (4, 5), (3, 3), (1.5,))
    assert s.ndim_fault() == 3 * 2 + 3
    write_setting(p, nplane="2", fix="T", xbend="1.5", nxi="4 5", neta="3 3")
    s = refio.settings_to_smc(refio.read_settings(p))
    assert s.layout == 1 and s.ndim_fault() == 2 * 2 + 4
    # the C-side mapping agrees
    lib = smcgpu.load_library()
    import ctypes as C
    stf, cfg = smcgpu.SettingsFile(), smcgpu.SmcConfig()
    assert lib.smcgpu_read_settings(p.encode(), C.byref(stf)) == 0
    assert lib.smcgpu_settings_to_config(C.byref(stf), C.byref(cfg)) == 0
    assert (cfg.layout, cfg.basis, cfg.nplane, cfg.nxi[1], cfg.xbend[0]) == (1, 0, 2, 5, 1.5)


@pytest.mark.parametrize("blank_every", [0, 7])
def test_read_observation_roundtrip(smcgpu, tmp_path, blank_every):
    from smc_inversion_fort_gb300 import refio
    w, obs = tiny_sar_obs()
    p = str(tmp_path / "obs.dat")
    write_observation(p, obs, w.npath, blank_every)
    got = refio.read_observation(p, w.npath)
    for k in ("obs_points", "obs_unitvec", "obs_sigma", "dvec"):
        np.testing.assert_array_equal(got[k], obs[k])
    np.testing.assert_array_equal(got["nsar_index"], obs["nsar_index"])
    assert got["ngnss"] == obs["ngnss"] and got["nsar_total"] == w.n_sar


def test_reader_list_directed_forms(smcgpu, tmp_path):
    from smc_inversion_fort_gb300 import refio
    p = str(tmp_path / "obs.dat")
    with open(p, "w") as f:
        f.write("header\n")
        f.write("1.0, 2.0, 0.5, 0.5, 0.7071d0, 1.25D-1, 0.1 'InSAR a'\n")
        f.write("\n")
        # read_observation1 counts records, so every row sits on one record
        f.write("3.0 4.0 0.0 0.0 1.0 2*0.5 \"InSAR a\"\n")
        f.write("5.0 6.0 1 0 0 0.3 0.2 GNSS / trailing text is ignored\n")
        f.write("5.0 6.0 0 1 0 0.4 0.2 GNSS\n5.0 6.0 0 0 1 0.5 0.3 GNSS\n\n")
    got = refio.read_observation(p, 1)
    assert len(got["dvec"]) == 5
    np.testing.assert_array_equal(got["obs_points"][:2], [[1.0, 2.0], [3.0, 4.0]])
    assert got["obs_unitvec"][0, 2] == 0.7071 and got["dvec"][0] == 0.125
    assert got["dvec"][1] == 0.5 and got["obs_sigma"][1] == 0.5
    np.testing.assert_array_equal(got["nsar_index"], [1, 3])
    assert got["ngnss"] == 1
    r = str(tmp_path / "range.dat")
    with open(r, "w") as f:
        f.write("ymin\n-10 2\nymax\n-2, 10\ndip\n 2*45.0\n")
    np.testing.assert_array_equal(refio.read_range(r, 3), [[-10, 2], [-2, 10], [45, 45]])
    v = str(tmp_path / "peak.dat")
    with open(v, "w") as f:
        f.write("1.5\n-2d0 ignored\n3\n")
    np.testing.assert_array_equal(refio.read_values(v, 3), [1.5, -2.0, 3.0])
    with open(v, "w") as f:
        f.write("1 2\n3*4.0\n")
    np.testing.assert_array_equal(refio.read_values(v, 5, one_per_record=False), [1, 2, 4, 4, 4])


def test_reader_errors(smcgpu, tmp_path):
    from smc_inversion_fort_gb300 import refio
    with pytest.raises(smcgpu.SmcError, match="cannot open"):
        refio.read_settings(str(tmp_path / "missing.dat"))
    p = str(tmp_path / "obs.dat")
    with open(p, "w") as f:
        f.write("h\n1 2 0 0 1 0.1 0.1 InSAR_a\n1 2 0 0 1 0.1 0.1 InSAR_b\n")
    with pytest.raises(smcgpu.SmcError, match="more InSAR paths"):
        refio.read_observation(p, 1)
    with open(p, "w") as f:
        f.write("h\n1 2 0 0 1 0.1 GNSS\n")   # one value short: the READ runs into the end of file
    with pytest.raises(smcgpu.SmcError, match="row 1: unexpected end of file"):
        refio.read_observation(p, 0)
    with open(p, "w") as f:
        f.write("h\n1 2 0 0 1 x 0.1 GNSS\n")
    with pytest.raises(smcgpu.SmcError, match="bad value 'x'"):
        refio.read_observation(p, 0)
    r = str(tmp_path / "range.dat")
    with open(r, "w") as f:
        f.write("a\n1 2\nb\n")
    with pytest.raises(smcgpu.SmcError, match="parameter 2"):
        refio.read_range(r, 2)


def make_run_dir(root, w, obs, theta, rg, nfault=16):
    os.makedirs(os.path.join(root, "data"), exist_ok=True)
    s = w.settings
    write_setting(os.path.join(root, "data", "setting.dat"), nplane=s.nplane, nfault=nfault,
                  nslip=s.nparticle_slip, npath=w.npath, nxi=" ".join(map(str, s.nxi)),
                  neta=" ".join(map(str, s.neta)), xmin=repr(s.xmin), xmax=repr(s.xmax), zmin=repr(s.zmin),
                  max_slip=repr(s.max_slip))
    write_observation(os.path.join(root, "data", "observation.dat"), obs, w.npath)
    with open(os.path.join(root, "peak_fault.dat"), "w") as f:
        f.write("".join(f"{repr(float(v))}\n" for v in theta))
    with open(os.path.join(root, "data", "range.dat"), "w") as f:
        for i, (lo, hi) in enumerate(rg):
            f.write(f"param {i + 1}\n{repr(float(lo))} {repr(float(hi))}\n")


@pytest.mark.gpu
def test_run_main_from_reference_directory(smcgpu, orc, tmp_path):
    """main.f90's shipped mode from a reference-format directory: identical to
    the API call on the same arrays, the oracle's first tempering exponent,
    and the slip dump in slip_smc_exec's layout."""
    from smc_inversion_fort_gb300 import refio
    w, obs = tiny_sar_obs()
    o0 = orc.Oracle(w.settings, obs)
    th = true_theta(w)
    obs["dvec"] = o0.greens(th).T @ true_slip(w) + np.random.default_rng(5).standard_normal(
        len(obs["dvec"])) * obs["obs_sigma"]
    root = str(tmp_path / "run")
    make_run_dir(root, w, obs, th, prior_range(w))
    post = refio.run_main(root, seed=3, stream=9)
    g = smcgpu.SmcGpu(w.settings)
    g.set_data(obs)
    ref = g.fault_likelihood_posterior(th, 3, 9)
    assert post["status"] == 0 and post["neglog"] == ref["neglog"]
    np.testing.assert_array_equal(post["particles"], ref["particles"])
    assert post["abic"] == 2 * ref["neglog"] + 2 * len(th)
    oref = orc.Oracle(w.settings, obs).fault_likelihood(th, 3, 9, trace=True)
    tr = g.fault_likelihood_trace(th[None], seed=3, streams=np.array([9], np.uint64))
    assert tr["gamma"][0][0] == pytest.approx(oref["gamma"][0], abs=1e-12)
    lines = open(os.path.join(root, "output", "slip_from_mean_fault.dat")).read().splitlines()
    assert len(lines) == w.settings.nparticle_slip
    nnode = (w.settings.nxi[0] + 1) * (w.settings.neta[0] + 1)
    assert all(len(ln) == 12 * (2 * nnode + 2) for ln in lines)
    first = [float(ln[i:i + 12]) for ln in lines[:1] for i in range(0, len(ln), 12)]
    np.testing.assert_allclose(first[-2:], [ref["likelihood"][0], ref["prior"][0]], atol=6e-6)
    assert max(first[:-2]) <= w.settings.max_slip + 1e-5 and min(first[:-2]) >= 0.0
