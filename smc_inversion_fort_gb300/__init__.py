"""GB300-native nested-SMC fault-geometry and slip inversion.

Python mirror of the reference's operator interface for the hot path
(KaiNakao/smc_inversion_fort: fault_calc_likelihood, calc_greens_func,
fault_smc_exec, the resampling step and sort.cpp's qsort_) over the C ABI in
include/smcgpu.h.  The CUDA library must be built (see build.py); every call
goes to the GPU and fails loudly when the library or a device is missing.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .configs import SmcSettings, preset  # noqa: F401

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "_lib", "libsmcgpu.so")

MAX_PLANES = 8
LAYOUT_TRACE, LAYOUT_TRACE_FIXBEND, LAYOUT_RECT = 0, 1, 2
BASIS_NODAL, BASIS_PATCH = 0, 1
PREC_FP64, PREC_FP32, PREC_MIXED = 0, 1, 2
ST_BISECT_CAP, ST_STAGE_CAP, ST_NONFINITE, ST_NEWTON_CAP, ST_REFLECT_CAP, ST_TUNE_COUNT = 1, 2, 4, 8, 16, 32
ST_WAIT_CAP = 64
ST_SNAPSHOT_IO = 128
ENGINE_MMA, ENGINE_CUDA, ENGINE_TCGEN05, ENGINE_GLOBAL, ENGINE_AUTO = 0, 1, 2, 3, 4
# engine table written by the autotuner (autotune.py), loaded under ENGINE_AUTO
ENGINE_TABLE_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "engine_table.json")


class SmcConfig(C.Structure):
    """ctypes mirror of smcgpu_config."""
    _fields_ = [
        ("layout", C.c_int32), ("basis", C.c_int32), ("nplane", C.c_int32),
        ("nxi", C.c_int32 * MAX_PLANES), ("neta", C.c_int32 * MAX_PLANES),
        ("xbend", C.c_double * MAX_PLANES),
        ("xmin", C.c_double), ("xmax", C.c_double), ("zmin", C.c_double),
        ("nquad", C.c_int32), ("rect_hyper", C.c_int32),
        ("alpha", C.c_double), ("max_slip", C.c_double),
        ("nparticle_slip", C.c_int32), ("ntau", C.c_int32), ("tuning_factor", C.c_int32),
        ("max_stages", C.c_int32),
        ("cv_inner", C.c_double), ("cv_outer", C.c_double), ("sar_corr_len", C.c_double),
        ("precision", C.c_int32), ("device", C.c_int32), ("max_outer_stages", C.c_int32),
        ("inner_warps", C.c_int32), ("inner_engine", C.c_int32), ("patch_km", C.c_double),
    ]


class Stats(C.Structure):
    """smcgpu_stats: totals since smcgpu_stats_reset."""
    _fields_ = [("nested_evals", C.c_int64), ("inner_stages", C.c_int64), ("inner_trajectories", C.c_int64),
                ("inner_kernel_ms", C.c_double), ("nested_ms", C.c_double)]


PATH_MAX = 512


class SettingsFile(C.Structure):
    """smcgpu_settings: the values of the reference's data/setting.dat."""
    _fields_ = [
        ("nplane", C.c_int32), ("fix_xbend", C.c_int32), ("xbend", C.c_double * MAX_PLANES),
        ("nparticle_fault", C.c_int32), ("nparticle_slip", C.c_int32),
        ("observation_path", C.c_char * PATH_MAX), ("npath", C.c_int32), ("output_dir", C.c_char * PATH_MAX),
        ("max_slip", C.c_double), ("nxi", C.c_int32 * MAX_PLANES), ("neta", C.c_int32 * MAX_PLANES),
        ("xmin", C.c_double), ("xmax", C.c_double), ("zmin", C.c_double), ("gsmc", C.c_int32),
    ]


_lib = None


def load_library() -> C.CDLL:
    """Load libsmcgpu.so; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: run smc_inversion_fort_gb300.build.build() first")
    lib = C.CDLL(LIB_PATH)
    P = C.POINTER
    d, i32, u64, vp = C.c_double, C.c_int32, C.c_uint64, C.c_void_p
    sig = {
        "smcgpu_default_config": (i32, [P(SmcConfig)]),
        "smcgpu_create": (i32, [P(SmcConfig), P(vp)]),
        "smcgpu_destroy": (i32, [vp]),
        "smcgpu_set_data": (i32, [vp, i32, vp, vp, vp, vp, i32, vp, i32]),
        "smcgpu_set_stream": (i32, [vp, vp]),
        "smcgpu_dims": (i32, [vp, P(i32), P(i32), P(i32), P(i32)]),
        "smcgpu_greens_batch": (i32, [vp, i32, vp, i32, vp]),
        "smcgpu_greens_batch_dev": (i32, [vp, i32, vp, i32, vp]),
        "smcgpu_gram_batch": (i32, [vp, i32, vp, vp, vp, vp]),
        "smcgpu_gibbs_levels": (i32, [P(SmcConfig), vp, vp, vp, vp]),
        "smcgpu_fault_likelihood_batch": (i32, [vp, i32, vp, u64, vp, vp, vp]),
        "smcgpu_fault_likelihood_batch_dev": (i32, [vp, i32, vp, u64, vp, vp, vp]),
        "smcgpu_fault_likelihood_trace": (i32, [vp, i32, vp, u64, vp, vp, vp, vp, vp, vp]),
        "smcgpu_fault_likelihood_posterior": (i32, [vp, vp, u64, u64, vp, vp, vp, vp, vp]),
        "smcgpu_fault_smc_exec": (i32, [vp, vp, i32, u64, C.c_char_p, vp, vp, vp, vp]),
        "smcgpu_fault_smc_exec_gsmc": (i32, [vp, vp, i32, u64, C.c_char_p, vp, vp, vp, d, vp, vp, vp, vp]),
        "smcgpu_fault_smc_resume": (i32, [vp, vp, i32, u64, C.c_char_p, C.c_char_p, vp, vp, vp, d, vp, vp, vp, vp]),
        "smcgpu_resample_counts": (i32, [vp, vp, i32, d, d, vp]),
        "smcgpu_qsort_": (None, [vp, vp, vp]),
        "smcgpu_last_error": (C.c_char_p, [vp]),
        "smcgpu_read_settings": (i32, [C.c_char_p, P(SettingsFile)]),
        "smcgpu_settings_to_config": (i32, [P(SettingsFile), P(SmcConfig)]),
        "smcgpu_count_observations": (i32, [C.c_char_p, P(i32)]),
        "smcgpu_read_observations": (i32, [C.c_char_p, i32, i32, vp, vp, vp, vp, vp, P(i32), P(i32)]),
        "smcgpu_read_range": (i32, [C.c_char_p, i32, vp]),
        "smcgpu_read_values": (i32, [C.c_char_p, i32, i32, vp]),
        "smcgpu_write_slip": (i32, [vp, C.c_char_p, i32, vp, vp, vp]),
        "smcgpu_slip_map": (i32, [vp, i32, vp, u64, vp, vp, vp, vp]),
        "smcgpu_slip_to_nodes": (i32, [vp, i32, vp, vp]),
        "smcgpu_write_slip_map": (i32, [vp, C.c_char_p, i32, vp]),
        "smcgpu_point_cloud": (i32, [vp, i32, vp, vp, i32, vp]),
        "smcgpu_write_point_cloud": (i32, [vp, C.c_char_p, i32, i32, vp]),
        "smcgpu_stats_reset": (i32, [vp, i32]),
        "smcgpu_stats_get": (i32, [vp, P(Stats)]),
        "smcgpu_outer_stage_times": (i32, [vp, i32, vp, vp, P(i32)]),
        "smcgpu_set_engine_table": (i32, [vp, i32, i32, vp, vp, vp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


EXPORTED_SYMBOLS = [
    "smcgpu_default_config", "smcgpu_create", "smcgpu_destroy", "smcgpu_set_data", "smcgpu_set_stream",
    "smcgpu_dims", "smcgpu_gibbs_levels", "smcgpu_greens_batch", "smcgpu_greens_batch_dev", "smcgpu_gram_batch",
    "smcgpu_fault_likelihood_batch",
    "smcgpu_fault_likelihood_batch_dev", "smcgpu_fault_likelihood_trace", "smcgpu_fault_likelihood_posterior",
    "smcgpu_fault_smc_exec", "smcgpu_fault_smc_exec_gsmc", "smcgpu_fault_smc_resume", "smcgpu_resample_counts",
    "smcgpu_qsort_",
    "smcgpu_last_error", "smcgpu_read_settings", "smcgpu_settings_to_config", "smcgpu_count_observations",
    "smcgpu_read_observations", "smcgpu_read_range", "smcgpu_read_values", "smcgpu_write_slip",
    "smcgpu_slip_map", "smcgpu_slip_to_nodes", "smcgpu_write_slip_map", "smcgpu_point_cloud",
    "smcgpu_write_point_cloud", "smcgpu_stats_reset", "smcgpu_stats_get", "smcgpu_outer_stage_times",
    "smcgpu_set_engine_table",
]


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


class SmcError(RuntimeError):
    pass


def gibbs_levels(s: SmcSettings):
    """The Gibbs sweep schedule of a configuration (host only): a list of
    levels, each the 0-based slip components updated together."""
    lib = load_library()
    cfg = make_config(s)
    D, nl = C.c_int32(), C.c_int32()
    rc = lib.smcgpu_gibbs_levels(C.byref(cfg), C.byref(D), C.byref(nl), None, None)
    if rc != 0:
        raise SmcError(f"smcgpu_gibbs_levels failed ({rc})")
    order = np.zeros(max(D.value, 1), np.int32)
    ptr = np.zeros(nl.value + 1, np.int32)
    rc = lib.smcgpu_gibbs_levels(C.byref(cfg), C.byref(D), C.byref(nl), _ptr(order), _ptr(ptr))
    if rc != 0:
        raise SmcError(f"smcgpu_gibbs_levels failed ({rc})")
    return [order[ptr[k]:ptr[k + 1]].tolist() for k in range(nl.value)]


def make_config(s: SmcSettings, precision: int = PREC_FP64, device: int = 0) -> SmcConfig:
    cfg = SmcConfig()
    load_library().smcgpu_default_config(C.byref(cfg))
    cfg.layout, cfg.basis, cfg.nplane = s.layout, s.basis, s.nplane
    for k in range(s.nplane):
        cfg.nxi[k], cfg.neta[k] = s.nxi[k], s.neta[k]
    for k, v in enumerate(s.xbend):
        cfg.xbend[k] = v
    cfg.xmin, cfg.xmax, cfg.zmin = s.xmin, s.xmax, s.zmin
    cfg.nquad, cfg.rect_hyper, cfg.alpha, cfg.max_slip = s.nquad, s.rect_hyper, s.alpha, s.max_slip
    cfg.nparticle_slip, cfg.ntau, cfg.tuning_factor, cfg.max_stages = s.nparticle_slip, s.ntau, s.tuning_factor, s.max_stages
    cfg.cv_inner, cfg.cv_outer, cfg.sar_corr_len = s.cv_inner, s.cv_outer, s.sar_corr_len
    cfg.precision, cfg.device = precision, device
    cfg.max_outer_stages = s.max_outer_stages
    cfg.inner_warps = s.inner_warps
    cfg.inner_engine = s.inner_engine
    cfg.patch_km = s.patch_km
    return cfg


def load_engine_table(path: str = ENGINE_TABLE_PATH):
    """The autotuner's engine table: {"fp64": [[dmax, engine, warps], ...], "mixed": [...]}
    or None when there is none."""
    import json
    if not os.path.exists(path):
        return None
    with open(path) as f:
        return json.load(f)


class SmcGpu:
    """One GPU context: observations resident in HBM, batched calls.

    Method names follow the reference routines they replace.
    """

    def __init__(self, settings: SmcSettings, precision: int = PREC_FP64, device: int = 0):
        self.lib = load_library()
        self.settings = settings
        self.cfg = make_config(settings, precision, device)
        h = C.c_void_p()
        rc = self.lib.smcgpu_create(C.byref(self.cfg), C.byref(h))
        if rc != 0:
            raise SmcError(f"smcgpu_create failed ({rc}): {self.lib.smcgpu_last_error(None).decode()}")
        self.h = h
        self.nobs = 0
        if settings.inner_engine == ENGINE_AUTO:
            tab = load_engine_table()
            if tab:
                for key, prec in (("fp64", PREC_FP64), ("mixed", PREC_MIXED)):
                    if tab.get(key):
                        self.set_engine_table(prec, tab[key])

    def set_engine_table(self, precision: int, rows):
        """rows: [(dmax, engine, warps), ...] with dmax ascending (SMCGPU_ENGINE_AUTO)."""
        a = np.ascontiguousarray(np.asarray(rows, dtype=np.int32).reshape(-1, 3).T)
        dm, en, wa = (np.ascontiguousarray(a[i]) for i in range(3))
        self._check(self.lib.smcgpu_set_engine_table(self.h, precision, len(dm), _ptr(dm), _ptr(en), _ptr(wa)),
                    "set_engine_table")

    def close(self):
        if getattr(self, "h", None):
            self.lib.smcgpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc: int, what: str):
        if rc != 0:
            raise SmcError(f"{what} failed ({rc}): {self.lib.smcgpu_last_error(self.h).decode()}")

    def dims(self):
        a, b, c, d = C.c_int32(), C.c_int32(), C.c_int32(), C.c_int32()
        self._check(self.lib.smcgpu_dims(self.h, C.byref(a), C.byref(b), C.byref(c), C.byref(d)), "dims")
        return {"ndim_fault": a.value, "D": b.value, "nobs": c.value, "nrow_l": d.value}

    def set_data(self, obs):
        """obs: dict with obs_points (nobs,2), obs_unitvec (nobs,3), obs_sigma, dvec, nsar_index
        (1-based, npath+1), ngnss -- the arrays of read_observation2 (init.f90:24-80)."""
        self._obs = {k: np.ascontiguousarray(v) for k, v in obs.items() if isinstance(v, np.ndarray)}
        pts = np.ascontiguousarray(obs["obs_points"], dtype=np.float64)
        e = np.ascontiguousarray(obs["obs_unitvec"], dtype=np.float64)
        sg = np.ascontiguousarray(obs["obs_sigma"], dtype=np.float64)
        dv = np.ascontiguousarray(obs["dvec"], dtype=np.float64)
        idx = np.ascontiguousarray(obs.get("nsar_index", np.array([1], np.int32)), dtype=np.int32)
        npath = len(idx) - 1
        self._keep = (pts, e, sg, dv, idx)
        self._check(self.lib.smcgpu_set_data(self.h, len(dv), _ptr(pts), _ptr(e), _ptr(sg), _ptr(dv), npath,
                                             _ptr(idx), int(obs["ngnss"])), "set_data")
        self.nobs = len(dv)

    def stats_reset(self, enable: bool = True):
        """Clear the run statistics and turn their recording on or off."""
        self._check(self.lib.smcgpu_stats_reset(self.h, 1 if enable else 0), "stats_reset")

    def stats(self) -> dict:
        st = Stats()
        self._check(self.lib.smcgpu_stats_get(self.h, C.byref(st)), "stats_get")
        return {f: getattr(st, f) for f, _ in Stats._fields_}

    def outer_stage_times(self):
        """(seconds, evaluations) per stage of the last fault_smc_exec; entry 0
        is the initial population's evaluation."""
        n = C.c_int32()
        self._check(self.lib.smcgpu_outer_stage_times(self.h, 0, None, None, C.byref(n)), "outer_stage_times")
        sec, ev = np.zeros(n.value), np.zeros(n.value, np.int64)
        self._check(self.lib.smcgpu_outer_stage_times(self.h, n.value, _ptr(sec), _ptr(ev), C.byref(n)),
                    "outer_stage_times")
        return sec, ev

    def set_stream(self, stream_handle: int | None):
        self._check(self.lib.smcgpu_set_stream(self.h, stream_handle or None), "set_stream")

    # calc_greens_func, batched (gfunc.f90:242-348)
    def calc_greens_func(self, theta: np.ndarray, precision: int = PREC_FP64, out: np.ndarray | None = None):
        th = np.ascontiguousarray(np.atleast_2d(theta), dtype=np.float64)
        dm = self.dims()
        dt = np.float32 if precision == PREC_FP32 else np.float64
        if out is None:
            out = np.empty((th.shape[0], dm["D"], dm["nobs"]), dtype=dt)
        self._check(self.lib.smcgpu_greens_batch(self.h, th.shape[0], _ptr(th), precision, _ptr(out)), "greens_batch")
        return out

    def greens_dev(self, n_theta: int, theta_ptr: int, gmat_ptr: int, precision: int = PREC_FP64):
        self._check(self.lib.smcgpu_greens_batch_dev(self.h, n_theta, theta_ptr, precision, gmat_ptr), "greens_batch_dev")

    def gram(self, theta: np.ndarray):
        """slip_calc_gsd_gsg (smc_slip.f90:1347-1443) per theta: (gsgmat [n, D, D]
        with gsgmat[t, j, i] = A(i, j), gsdvec [n, D], dsd [n])."""
        th = np.ascontiguousarray(np.atleast_2d(theta), dtype=np.float64)
        D = self.dims()["D"]
        n = th.shape[0]
        A, b, dsd = np.empty((n, D, D)), np.empty((n, D)), np.empty(n)
        self._check(self.lib.smcgpu_gram_batch(self.h, n, _ptr(th), _ptr(A), _ptr(b), _ptr(dsd)), "gram_batch")
        return A, b, dsd

    # fault_calc_likelihood, batched (smc_fault.f90:66-292)
    def fault_calc_likelihood(self, theta: np.ndarray, seed: int, streams=None):
        th = np.ascontiguousarray(np.atleast_2d(theta), dtype=np.float64)
        n = th.shape[0]
        st = np.ascontiguousarray(np.arange(n, dtype=np.uint64) if streams is None else streams, dtype=np.uint64)
        neglog = np.empty(n, np.float64)
        status = np.empty(n, np.int32)
        self._check(self.lib.smcgpu_fault_likelihood_batch(self.h, n, _ptr(th), seed, _ptr(st), _ptr(neglog),
                                                           _ptr(status)), "fault_likelihood_batch")
        return neglog, status

    def fault_likelihood_trace(self, theta: np.ndarray, seed: int, streams=None):
        th = np.ascontiguousarray(np.atleast_2d(theta), dtype=np.float64)
        n = th.shape[0]
        ms = self.settings.max_stages + 2
        st = np.ascontiguousarray(np.arange(n, dtype=np.uint64) if streams is None else streams, dtype=np.uint64)
        neglog, status, nstage = np.empty(n), np.empty(n, np.int32), np.empty(n, np.int32)
        gam, inc = np.zeros((n, ms)), np.zeros((n, ms))
        self._check(self.lib.smcgpu_fault_likelihood_trace(self.h, n, _ptr(th), seed, _ptr(st), _ptr(neglog),
                                                           _ptr(status), _ptr(nstage), _ptr(gam), _ptr(inc)),
                    "fault_likelihood_trace")
        return {"neglog": neglog, "status": status, "nstage": nstage,
                "gamma": [gam[i, :nstage[i]] for i in range(n)], "neglog_inc": [inc[i, :nstage[i]] for i in range(n)]}

    def fault_likelihood_posterior(self, theta: np.ndarray, seed: int, stream: int = 0):
        th = np.ascontiguousarray(theta, dtype=np.float64)
        N, D = self.settings.nparticle_slip, self.dims()["D"]
        nl, stt = C.c_double(), C.c_int32()
        parts, L, P = np.empty((N, D)), np.empty(N), np.empty(N)
        self._check(self.lib.smcgpu_fault_likelihood_posterior(self.h, _ptr(th), seed, stream, C.byref(nl),
                                                               C.byref(stt), _ptr(parts), _ptr(L), _ptr(P)),
                    "fault_likelihood_posterior")
        return {"neglog": nl.value, "status": stt.value, "particles": parts, "likelihood": L, "prior": P}

    def fault_likelihood_dev(self, n, theta_ptr, seed, streams_ptr, neglog_ptr, status_ptr):
        self._check(self.lib.smcgpu_fault_likelihood_batch_dev(self.h, n, theta_ptr, seed, streams_ptr, neglog_ptr,
                                                               status_ptr), "fault_likelihood_batch_dev")

    def write_slip(self, path: str, particles: np.ndarray, likelihood: np.ndarray, prior: np.ndarray):
        """slip_smc_exec's posterior dump (smc_slip.f90:1632-1660)."""
        x = np.ascontiguousarray(particles, dtype=np.float64)
        L = np.ascontiguousarray(likelihood, dtype=np.float64)
        P = np.ascontiguousarray(prior, dtype=np.float64)
        self._check(self.lib.smcgpu_write_slip(self.h, path.encode(), len(L), _ptr(x), _ptr(L), _ptr(P)), "write_slip")

    def fault_smc_resume(self, range_: np.ndarray, nparticle: int, seed: int, state_path: str,
                         output_dir: str | None = None, gsmc: dict | None = None):
        """Continue fault_smc_exec from a <k>.state file written after stage k."""
        rg = np.ascontiguousarray(range_, dtype=np.float64)
        nd = self.dims()["ndim_fault"]
        parts = np.empty((nparticle, nd), np.float64)
        lik = np.empty(nparticle, np.float64)
        ev, ns = C.c_double(), C.c_int32()
        od = output_dir.encode() if output_dir else None
        if gsmc is None:
            qm = qc = qi = None
            ld = 0.0
        else:
            qm = np.ascontiguousarray(gsmc["qmean"], np.float64)
            qc = np.ascontiguousarray(np.asarray(gsmc["qcov_chol"], np.float64).T)
            qi = np.ascontiguousarray(np.asarray(gsmc["qcov_inv"], np.float64).T)
            ld = float(gsmc["log_qcov_det"])
        ptr = (lambda a: None if a is None else _ptr(a))
        self._check(self.lib.smcgpu_fault_smc_resume(self.h, _ptr(rg), nparticle, seed, od, state_path.encode(),
                                                     ptr(qm), ptr(qc), ptr(qi), ld, _ptr(parts), _ptr(lik),
                                                     C.byref(ev), C.byref(ns)), "fault_smc_resume")
        return parts, lik, ev.value, ns.value

    # post-processing (main.f90:553-830)
    def slip_map(self, theta: np.ndarray, seed: int, streams: np.ndarray):
        """calc_slip_map: mean final inner slip population per theta -> (mean (n, D), neglog, status)."""
        th = np.ascontiguousarray(np.atleast_2d(theta), dtype=np.float64)
        n, D = th.shape[0], self.dims()["D"]
        st = np.ascontiguousarray(streams, dtype=np.uint64)
        mean, nl, stat = np.empty((n, D)), np.empty(n), np.empty(n, np.int32)
        self._check(self.lib.smcgpu_slip_map(self.h, n, _ptr(th), seed, _ptr(st), _ptr(mean), _ptr(nl), _ptr(stat)),
                    "slip_map")
        return mean, nl, stat

    def slip_to_nodes(self, slip: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(np.atleast_2d(slip), dtype=np.float64)
        nn = 2 * self.mesh_counts()["nnode"] if self.settings.basis == 0 else x.shape[1]
        out = np.empty((x.shape[0], nn))
        self._check(self.lib.smcgpu_slip_to_nodes(self.h, x.shape[0], _ptr(x), _ptr(out)), "slip_to_nodes")
        return out

    def write_slip_map(self, path: str, mean_slip: np.ndarray):
        x = np.ascontiguousarray(np.atleast_2d(mean_slip), dtype=np.float64)
        self._check(self.lib.smcgpu_write_slip_map(self.h, path.encode(), x.shape[0], _ptr(x)), "write_slip_map")

    def point_cloud(self, theta: np.ndarray, slip_nodes: np.ndarray, nr: int = 8) -> np.ndarray:
        """point_cloud: (n, npatch, nr, nr, 6) = x, y, z, uxi, ueta, |u| per sub-point."""
        th = np.ascontiguousarray(np.atleast_2d(theta), dtype=np.float64)
        sl = np.ascontiguousarray(np.atleast_2d(slip_nodes), dtype=np.float64)
        npatch = self.mesh_counts()["npatch"]
        out = np.empty((th.shape[0], npatch, nr, nr, 6))
        self._check(self.lib.smcgpu_point_cloud(self.h, th.shape[0], _ptr(th), _ptr(sl), nr, _ptr(out)), "point_cloud")
        return out

    def write_point_cloud(self, prefix: str, points: np.ndarray):
        p = np.ascontiguousarray(points, dtype=np.float64)
        self._check(self.lib.smcgpu_write_point_cloud(self.h, prefix.encode(), p.shape[0], p.shape[2], _ptr(p)),
                    "write_point_cloud")

    def mesh_counts(self) -> dict:
        s = self.settings
        nn = sum((s.nxi[i] + 1) * (s.neta[i] + 1) for i in range(s.nplane))
        npch = sum(s.nxi[i] * s.neta[i] for i in range(s.nplane))
        return {"nnode": nn, "npatch": npch}

    # fault_smc_exec (smc_fault.f90:785-1075)
    def fault_smc_exec(self, range_: np.ndarray, nparticle: int, seed: int, output_dir: str | None = None,
                       gsmc: dict | None = None):
        """gsmc: None (uniform prior box) or dict(qmean, qcov_chol, qcov_inv, log_qcov_det) with
        (ndim, ndim) row-indexed matrices; the GSMC mode of smc_fault.f90."""
        rg = np.ascontiguousarray(range_, dtype=np.float64)
        nd = self.dims()["ndim_fault"]
        parts = np.empty((nparticle, nd), np.float64)
        lik = np.empty(nparticle, np.float64)
        ev = C.c_double()
        ns = C.c_int32()
        od = output_dir.encode() if output_dir else None
        if gsmc is None:
            rc = self.lib.smcgpu_fault_smc_exec(self.h, _ptr(rg), nparticle, seed, od, _ptr(parts), _ptr(lik),
                                                C.byref(ev), C.byref(ns))
        else:
            qm = np.ascontiguousarray(gsmc["qmean"], np.float64)
            qc = np.ascontiguousarray(np.asarray(gsmc["qcov_chol"], np.float64).T)   # column-major
            qi = np.ascontiguousarray(np.asarray(gsmc["qcov_inv"], np.float64).T)
            rc = self.lib.smcgpu_fault_smc_exec_gsmc(self.h, _ptr(rg), nparticle, seed, od, _ptr(qm), _ptr(qc),
                                                     _ptr(qi), float(gsmc["log_qcov_det"]), _ptr(parts), _ptr(lik),
                                                     C.byref(ev), C.byref(ns))
        self._check(rc, "fault_smc_exec")
        return parts, lik, ev.value, ns.value

    # slip_resample_particles / fault_resample_particles (binary128-exact counts)
    def resample_counts(self, weights: np.ndarray, u0_hi: float, u0_lo: float):
        w = np.ascontiguousarray(weights, dtype=np.float64)
        out = np.empty(len(w), np.int32)
        self._check(self.lib.smcgpu_resample_counts(self.h, _ptr(w), len(w), u0_hi, u0_lo, _ptr(out)),
                    "resample_counts")
        return out


def qsort_(arr: np.ndarray, index: np.ndarray) -> None:
    """sort.cpp's qsort_: sorts the 1-based index array in place."""
    lib = load_library()
    a = np.ascontiguousarray(arr, dtype=np.int32)
    if not (index.flags["C_CONTIGUOUS"] and index.dtype == np.int32):
        raise ValueError("index must be a contiguous int32 array")
    n = C.c_int32(len(index))
    lib.smcgpu_qsort_(_ptr(a), _ptr(index), C.byref(n))
