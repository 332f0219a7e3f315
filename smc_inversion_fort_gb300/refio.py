"""The reference's input files and run modes, over the C ABI readers.

An unchanged reference run directory (``data/setting.dat``, the observation
file it names, ``peak_fault.dat``, ``data/range.dat``) drives the GPU path:

* :func:`run_main` is ``main.f90``'s shipped mode (main.f90:418-482): one
  nested evaluation of the geometry in ``peak_fault.dat``, its slip posterior
  written like ``slip_smc_exec`` does (smc_slip.f90:1632-1660), and the ABIC
  ``2 neglog + 2 ndim_fault``;
* :func:`run_fault_smc` is the outer SMC over the ``data/range.dat`` box
  (main.f90:490-545) with the per-stage CSV files in ``output_dir``.

The file formats are read by ``smcgpu_read_*`` (io.cpp) with Fortran
list-directed semantics; paths inside setting.dat are relative to the run
directory, as for the reference run from that directory.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import PREC_FP64, SettingsFile, SmcError, SmcGpu, _ptr, load_library
from .configs import SmcSettings


def _err(lib, what, rc):
    if rc != 0:
        raise SmcError(f"{what} failed ({rc}): {lib.smcgpu_last_error(None).decode()}")


def read_settings(path: str) -> dict:
    """data/setting.dat (main.f90:107-157) as a dict of its values."""
    lib = load_library()
    st = SettingsFile()
    _err(lib, "read_settings", lib.smcgpu_read_settings(path.encode(), C.byref(st)))
    n = st.nplane
    return {
        "nplane": n, "fix_xbend": bool(st.fix_xbend), "xbend": [st.xbend[i] for i in range(n - 1)],
        "nparticle_fault": st.nparticle_fault, "nparticle_slip": st.nparticle_slip,
        "observation_path": st.observation_path.decode(), "npath": st.npath, "output_dir": st.output_dir.decode(),
        "max_slip": st.max_slip, "nxi": [st.nxi[i] for i in range(n)], "neta": [st.neta[i] for i in range(n)],
        "xmin": st.xmin, "xmax": st.xmax, "zmin": st.zmin, "gsmc": bool(st.gsmc),
    }


def settings_to_smc(st: dict) -> SmcSettings:
    """The reference's discretisation for these settings: nodal basis, trace
    layout (fixed bends when fix_xbend), reference SMC constants."""
    return SmcSettings(
        layout=1 if st["fix_xbend"] else 0, basis=0, nplane=st["nplane"], nxi=tuple(st["nxi"]),
        neta=tuple(st["neta"]), xbend=tuple(st["xbend"]), xmin=st["xmin"], xmax=st["xmax"], zmin=st["zmin"],
        max_slip=st["max_slip"], nparticle_slip=st["nparticle_slip"])


def read_observation(path: str, npath: int) -> dict:
    """read_observation1 + read_observation2 (init.f90:5-80): the arrays that
    SmcGpu.set_data takes."""
    lib = load_library()
    nobs = C.c_int32()
    _err(lib, "count_observations", lib.smcgpu_count_observations(path.encode(), C.byref(nobs)))
    n = nobs.value
    pts, e = np.zeros((n, 2)), np.zeros((n, 3))
    sg, dv = np.zeros(n), np.zeros(n)
    idx = np.zeros(npath + 1, np.int32)
    nsar, ngnss = C.c_int32(), C.c_int32()
    _err(lib, "read_observations",
         lib.smcgpu_read_observations(path.encode(), n, npath, _ptr(pts), _ptr(e), _ptr(sg), _ptr(dv), _ptr(idx),
                                      C.byref(nsar), C.byref(ngnss)))
    return {"obs_points": pts, "obs_unitvec": e, "obs_sigma": sg, "dvec": dv, "nsar_index": idx,
            "nsar_total": nsar.value, "ngnss": ngnss.value}


def read_range(path: str, ndim: int) -> np.ndarray:
    """data/range.dat: (ndim, 2) lower / upper bounds."""
    lib = load_library()
    out = np.zeros((ndim, 2))
    _err(lib, "read_range", lib.smcgpu_read_range(path.encode(), ndim, _ptr(out)))
    return out


def read_values(path: str, n: int, one_per_record: bool = True) -> np.ndarray:
    lib = load_library()
    out = np.zeros(n)
    _err(lib, "read_values", lib.smcgpu_read_values(path.encode(), n, int(one_per_record), _ptr(out)))
    return out


def load_run(workdir: str, precision: int = PREC_FP64):
    """Settings, observations and a GPU context with the data resident."""
    st = read_settings(os.path.join(workdir, "data", "setting.dat"))
    obs = read_observation(os.path.join(workdir, st["observation_path"]), st["npath"])
    s = settings_to_smc(st)
    g = SmcGpu(s, precision)
    g.set_data(obs)
    return st, obs, g


def run_main(workdir: str, precision: int = PREC_FP64, seed: int = 1, stream: int = 0,
             slip_path: str = "output/slip_from_mean_fault.dat") -> dict:
    """main.f90's shipped mode: nested evaluation of peak_fault.dat's geometry."""
    st, obs, g = load_run(workdir, precision)
    nd = g.dims()["ndim_fault"]
    theta = read_values(os.path.join(workdir, "peak_fault.dat"), nd)
    post = g.fault_likelihood_posterior(theta, seed, stream)
    if slip_path:
        out = os.path.join(workdir, slip_path)
        os.makedirs(os.path.dirname(out) or ".", exist_ok=True)
        g.write_slip(out, post["particles"], post["likelihood"], post["prior"])
    post["abic"] = 2.0 * post["neglog"] + 2.0 * nd
    post["theta"] = theta
    g.close()
    return post


def read_gsmc(workdir: str, nd: int) -> dict:
    """GSMC reference distribution files (main.f90:313-332): data/qmean.dat,
    qcov.dat, qcov_inv.dat (column-major lists), log_qcov_det.dat; qcov is
    factored like dpotrf('L')."""
    d = os.path.join(workdir, "data")
    qmean = read_values(os.path.join(d, "qmean.dat"), nd, one_per_record=False)
    qcov = read_values(os.path.join(d, "qcov.dat"), nd * nd, one_per_record=False).reshape(nd, nd).T
    qinv = read_values(os.path.join(d, "qcov_inv.dat"), nd * nd, one_per_record=False).reshape(nd, nd).T
    ld = read_values(os.path.join(d, "log_qcov_det.dat"), 1)[0]
    return {"qmean": qmean, "qcov_chol": np.linalg.cholesky(qcov), "qcov_inv": qinv, "log_qcov_det": ld}


def run_fault_smc(workdir: str, precision: int = PREC_FP64, seed: int = 1) -> dict:
    """fault_smc_exec over data/range.dat with nparticle_fault outer particles
    (GSMC when setting.dat says so); stage CSVs go to output_dir (relative to
    the run directory)."""
    st, obs, g = load_run(workdir, precision)
    nd = g.dims()["ndim_fault"]
    rg = read_range(os.path.join(workdir, "data", "range.dat"), nd)
    od = os.path.join(workdir, st["output_dir"]) if st["output_dir"] else None
    gq = read_gsmc(workdir, nd) if st["gsmc"] else None
    parts, lik, ev, ns = g.fault_smc_exec(rg, st["nparticle_fault"], seed, od, gsmc=gq)
    g.close()
    return {"particles": parts, "likelihood": lik, "evidence": ev, "nstage": ns, "range": rg}


def read_stage_samples(path: str, nparticle: int, offset: int, stride: int, nd: int) -> np.ndarray:
    """The geometry samples that calc_slip_map / point_cloud read from an
    outer-stage file (main.f90:575-587, 705-716): skip `offset` records,
    then keep the last of every `stride` records; columns 1..nd of each."""
    rows = np.loadtxt(path, ndmin=2)
    need = offset + nparticle * stride
    if rows.shape[0] < need:
        raise SmcError(f"{path}: {rows.shape[0]} records, {need} needed")
    idx = offset + stride * np.arange(1, nparticle + 1) - 1
    return np.ascontiguousarray(rows[idx, :nd])


def run_slip_map(workdir: str, fault_path: str, out_path: str, nparticle: int | None = None, offset: int = 10,
                 stride: int = 2, precision: int = PREC_FP64, seed: int = 1) -> dict:
    """calc_slip_map (main.f90:553-664) from a run directory: the mean inner
    slip of each sampled geometry, written to out_path."""
    st, obs, g = load_run(workdir, precision)
    nd = g.dims()["ndim_fault"]
    n = nparticle or st["nparticle_fault"]
    th = read_stage_samples(os.path.join(workdir, fault_path), n, offset, stride, nd)
    mean, nl, stat = g.slip_map(th, seed, np.arange(n, dtype=np.uint64))
    out = os.path.join(workdir, out_path)
    os.makedirs(os.path.dirname(out) or ".", exist_ok=True)
    g.write_slip_map(out, mean)
    g.close()
    return {"theta": th, "mean_slip": mean, "neglog": nl, "status": stat}


def run_point_cloud(workdir: str, fault_path: str, slip_path: str, out_prefix: str, nparticle: int | None = None,
                    offset: int = 10, stride: int = 100, nr: int = 8) -> np.ndarray:
    """point_cloud (main.f90:666-806): geometry samples from an outer-stage
    file and their node slips from a calc_slip_map file; one output file per
    plane, out_prefix//iplane."""
    st, obs, g = load_run(workdir)
    nd = g.dims()["ndim_fault"]
    n = nparticle or st["nparticle_fault"]
    th = read_stage_samples(os.path.join(workdir, fault_path), n, offset, stride, nd)
    slip = np.loadtxt(os.path.join(workdir, slip_path), ndmin=2)[:n]
    pts = g.point_cloud(th, slip, nr)
    out = os.path.join(workdir, out_prefix)
    os.makedirs(os.path.dirname(out) or ".", exist_ok=True)
    g.write_point_cloud(out, pts)
    g.close()
    return pts
