"""ctypes binding of the CPU oracle (oracle.cpp).

TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the
CPU-baseline / reference legs of bench.py as the checker and the timed CPU
restatement of the reference.  Never used by the product path.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
# timing build (-O3, FMA contraction allowed): the CPU baseline only, never a
# parity check; select it with use_timing_build() before the first call
FAST_LIB_PATH = os.path.join(HERE, "_build", "liboracle_fast.so")
MAXP = 8
_use_fast = False


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "oracle.cpp")
    newest = max(os.path.getmtime(src), os.path.getmtime(os.path.join(HERE, "oracle.h")))
    if force or any(not os.path.exists(p) or os.path.getmtime(p) < newest for p in (LIB_PATH, FAST_LIB_PATH)):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def use_timing_build() -> None:
    """Load the -O3 timing build instead of the parity build (bench.py's CPU
    baseline); must be called before any oracle call in the process."""
    global _use_fast
    if _lib is not None and not _use_fast:
        raise RuntimeError("the parity build is already loaded in this process")
    _use_fast = True


class OrcSetup(C.Structure):
    _fields_ = [
        ("layout", C.c_int32), ("basis", C.c_int32), ("nplane", C.c_int32),
        ("nxi", C.c_int32 * MAXP), ("neta", C.c_int32 * MAXP), ("xbend", C.c_double * MAXP),
        ("xmin", C.c_double), ("xmax", C.c_double), ("zmin", C.c_double),
        ("nquad", C.c_int32), ("rect_hyper", C.c_int32), ("alpha", C.c_double), ("max_slip", C.c_double),
        ("nparticle_slip", C.c_int32), ("ntau", C.c_int32), ("tuning_factor", C.c_int32), ("max_stages", C.c_int32),
        ("cv_inner", C.c_double), ("cv_outer", C.c_double),
        ("nobs", C.c_int32), ("nsar_total", C.c_int32), ("ngnss", C.c_int32), ("npath", C.c_int32),
        ("nsar_index", C.c_void_p), ("obs_points", C.c_void_p), ("obs_unitvec", C.c_void_p),
        ("obs_sigma", C.c_void_p), ("dvec", C.c_void_p), ("sigma_sar_inv", C.c_void_p),
        ("max_outer_stages", C.c_int32),
    ]


class OrcDims(C.Structure):
    _fields_ = [("ndim_fault", C.c_int32), ("D", C.c_int32), ("nnode", C.c_int32), ("ndof", C.c_int32),
                ("npatch", C.c_int32), ("nrow_l", C.c_int32)]


class OrcTrace(C.Structure):
    _fields_ = [("nstage", C.c_int32), ("gamma", C.c_void_p), ("neglog_inc", C.c_void_p), ("assigned", C.c_void_p)]


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(FAST_LIB_PATH if _use_fast else LIB_PATH)
        vp, d, i32, u64, u32 = C.c_void_p, C.c_double, C.c_int32, C.c_uint64, C.c_uint32
        L.orc_philox4x64.argtypes = [vp, vp, vp]
        L.orc_uniform.argtypes = [u64, u64, u32, u32, u64, u64]
        L.orc_uniform.restype = d
        L.orc_normal.argtypes = [u64, u64, u32, u32, u64, u64]
        L.orc_normal.restype = d
        L.orc_quad_uniform.argtypes = [u64, u64, u32, u32, vp, vp]
        L.orc_dims.argtypes = [vp, vp]
        L.orc_dc3d0.argtypes = [d] * 10 + [vp, vp]
        L.orc_plane_params.argtypes = [vp, vp, vp]
        L.orc_greens.argtypes = [vp, vp, vp]
        L.orc_greens_batch.argtypes = [vp, i32, vp, vp, i32]
        L.orc_laplacian.argtypes = [vp, vp, vp, vp, vp, vp, vp]
        L.orc_laplacian.restype = i32
        L.orc_sigma_sar_inv.argtypes = [i32, i32, vp, vp, vp, d, vp]
        L.orc_gram.argtypes = [vp, vp, d, d, vp, vp, vp]
        L.orc_hyper.argtypes = [vp, vp, vp, vp, vp]
        L.orc_fault_likelihood.argtypes = [vp, vp, u64, u64, vp, vp, vp, vp, vp]
        L.orc_fault_likelihood.restype = i32
        L.orc_fault_likelihood_batch.argtypes = [vp, i32, vp, u64, vp, vp, vp, i32]
        L.orc_slip_energy.argtypes = [vp, vp, d, vp, vp, vp, vp]
        L.orc_slip_energy.restype = i32
        L.orc_resample.argtypes = [vp, i32, d, d, vp]
        L.orc_qsort_.argtypes = [vp, vp, vp]
        L.orc_fault_smc.argtypes = [vp, vp, i32, i32, u64, i32, vp, vp, vp, vp, vp, vp]
        L.orc_fault_smc.restype = i32
        L.orc_point_cloud.argtypes = [vp, vp, vp, i32, vp]
        L.orc_point_cloud.restype = i32
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data


class Oracle:
    """Oracle view of one settings + observation set."""

    def __init__(self, settings, obs):
        s = settings
        self.settings = s
        self.obs = {k: (np.ascontiguousarray(v) if isinstance(v, np.ndarray) else v) for k, v in obs.items()}
        o = self.obs
        self.pts = np.ascontiguousarray(o["obs_points"], np.float64)
        self.e = np.ascontiguousarray(o["obs_unitvec"], np.float64)
        self.sig = np.ascontiguousarray(o["obs_sigma"], np.float64)
        self.d = np.ascontiguousarray(o.get("dvec", np.zeros(len(self.sig))), np.float64)
        idx1 = np.asarray(o.get("nsar_index", np.array([1])), np.int32)
        self.npath = len(idx1) - 1
        self.idx0 = np.ascontiguousarray(idx1 - 1, np.int32)
        nsar = int(self.idx0[-1]) if self.npath > 0 else 0
        self.nsar = nsar
        self.ngnss = int(o["ngnss"])
        nobs = len(self.sig)
        blocks = []
        if self.npath > 0:
            tot = sum(int(self.idx0[p + 1] - self.idx0[p]) ** 2 for p in range(self.npath))
            self.sinv = np.zeros(max(tot, 1))
            lib().orc_sigma_sar_inv(nobs, self.npath, _p(self.idx0), _p(self.pts), _p(self.sig), s.sar_corr_len,
                                    _p(self.sinv))
        else:
            self.sinv = np.zeros(1)
        del blocks
        st = OrcSetup()
        st.layout, st.basis, st.nplane = s.layout, s.basis, s.nplane
        for k in range(s.nplane):
            st.nxi[k], st.neta[k] = s.nxi[k], s.neta[k]
        for k, v in enumerate(s.xbend):
            st.xbend[k] = v
        st.xmin, st.xmax, st.zmin = s.xmin, s.xmax, s.zmin
        st.nquad, st.rect_hyper, st.alpha, st.max_slip = s.nquad, s.rect_hyper, s.alpha, s.max_slip
        st.nparticle_slip, st.ntau, st.tuning_factor, st.max_stages = s.nparticle_slip, s.ntau, s.tuning_factor, s.max_stages
        st.cv_inner, st.cv_outer = s.cv_inner, s.cv_outer
        st.nobs, st.nsar_total, st.ngnss, st.npath = nobs, nsar, self.ngnss, self.npath
        st.nsar_index, st.obs_points, st.obs_unitvec = _p(self.idx0), _p(self.pts), _p(self.e)
        st.obs_sigma, st.dvec, st.sigma_sar_inv = _p(self.sig), _p(self.d), _p(self.sinv)
        st.max_outer_stages = getattr(s, "max_outer_stages", 0)
        self.st = st
        dm = OrcDims()
        lib().orc_dims(C.byref(st), C.byref(dm))
        self.dims = {f: getattr(dm, f) for f, _ in OrcDims._fields_}
        self.nobs = nobs

    def greens(self, theta):
        th = np.ascontiguousarray(theta, np.float64)
        g = np.zeros((self.dims["D"], self.nobs))
        lib().orc_greens(C.byref(self.st), _p(th), _p(g))
        return g

    def greens_batch(self, thetas, nthreads=0):
        th = np.ascontiguousarray(thetas, np.float64)
        g = np.zeros((th.shape[0], self.dims["D"], self.nobs))
        lib().orc_greens_batch(C.byref(self.st), th.shape[0], _p(th), _p(g), nthreads)
        return g

    def plane_params(self, theta):
        th = np.ascontiguousarray(theta, np.float64)
        out = np.zeros(7 * self.settings.nplane)
        lib().orc_plane_params(C.byref(self.st), _p(th), _p(out))
        return out.reshape(-1, 7)

    def laplacian(self, theta):
        th = np.ascontiguousarray(theta, np.float64)
        D, nrow = self.dims["D"], self.dims["nrow_l"]
        li, lv = np.zeros(nrow * 9, np.int32), np.zeros(nrow * 9)
        lti, ltv = np.zeros(D * 9, np.int32), np.zeros(D * 9)
        ll = np.zeros(D * D)
        lib().orc_laplacian(C.byref(self.st), _p(th), _p(li), _p(lv), _p(lti), _p(ltv), _p(ll))
        return li.reshape(nrow, 9), lv.reshape(nrow, 9), lti.reshape(D, 9), ltv.reshape(D, 9), ll.reshape(D, D).T

    def hyper(self, theta):
        th = np.ascontiguousarray(theta, np.float64)
        a, b, c = C.c_double(), C.c_double(), C.c_double()
        lib().orc_hyper(C.byref(self.st), _p(th), C.byref(a), C.byref(b), C.byref(c))
        return a.value, b.value, c.value

    def gram(self, gmat, sigma_sar2, sigma_gnss2):
        D = self.dims["D"]
        g = np.ascontiguousarray(gmat, np.float64)
        A, b, dsd = np.zeros(D * D), np.zeros(D), C.c_double()
        lib().orc_gram(C.byref(self.st), _p(g), sigma_sar2, sigma_gnss2, _p(A), _p(b), C.byref(dsd))
        return A.reshape(D, D).T, b, dsd.value

    def fault_likelihood(self, theta, seed, stream, trace=False):
        th = np.ascontiguousarray(theta, np.float64)
        N, D = self.settings.nparticle_slip, self.dims["D"]
        nl = C.c_double()
        parts, L, P = np.zeros((N, D)), np.zeros(N), np.zeros(N)
        tr = None
        if trace:
            ms = self.settings.max_stages + 2
            gam, inc, asg = np.zeros(ms), np.zeros(ms), np.zeros((ms, N), np.int32)
            tr = OrcTrace(0, _p(gam), _p(inc), _p(asg))
        status = lib().orc_fault_likelihood(C.byref(self.st), _p(th), seed, stream, C.byref(nl), _p(parts), _p(L),
                                            _p(P), C.byref(tr) if tr is not None else None)
        out = {"neglog": nl.value, "status": status, "particles": parts, "likelihood": L, "prior": P}
        if trace:
            n = tr.nstage
            out.update(gamma=gam[:n].copy(), neglog_inc=inc[:n].copy(), assigned=asg[:n].copy())
        return out

    def slip_energy(self, theta, gamma, x):
        """Likelihood, prior and the tempered gradient gamma dL/dx + dP/dx at slip x."""
        th = np.ascontiguousarray(theta, np.float64)
        xv = np.ascontiguousarray(x, np.float64)
        grad = np.zeros(self.dims["D"])
        lik, pri = C.c_double(), C.c_double()
        lib().orc_slip_energy(C.byref(self.st), _p(th), float(gamma), _p(xv), C.byref(lik), C.byref(pri), _p(grad))
        return lik.value, pri.value, grad

    def fault_likelihood_batch(self, thetas, seed, streams, nthreads=0):
        th = np.ascontiguousarray(thetas, np.float64)
        st = np.ascontiguousarray(streams, np.uint64)
        nl = np.zeros(th.shape[0])
        stat = np.zeros(th.shape[0], np.int32)
        lib().orc_fault_likelihood_batch(C.byref(self.st), th.shape[0], _p(th), seed, _p(st), _p(nl), _p(stat),
                                         nthreads)
        return nl, stat

    def point_cloud(self, theta, slip, nr):
        """slip: slip_dist(2, nnode) as a flat array (nodal) or the D patch values."""
        th = np.ascontiguousarray(theta, np.float64)
        sl = np.ascontiguousarray(slip, np.float64)
        out = np.zeros((self.dims["npatch"], nr, nr, 6))
        lib().orc_point_cloud(C.byref(self.st), _p(th), _p(sl), nr, _p(out))
        return out

    def fault_smc(self, range_, nparticle, seed, numprocs=1, nthreads=0, gsmc=None):
        """gsmc: None (uniform prior box) or dict(qmean, qcov_chol, qcov_inv, log_qcov_det)."""
        rg = np.ascontiguousarray(range_, np.float64)
        nd = self.dims["ndim_fault"]
        parts, L = np.zeros((nparticle, nd)), np.zeros(nparticle)
        ev, ns = C.c_double(), C.c_int32()
        gam = np.zeros(1024)
        gp = None
        if gsmc is not None:
            keep = [np.ascontiguousarray(gsmc[k], np.float64) for k in ("qmean", "qcov_chol", "qcov_inv")]
            # column-major matrices: pass the transpose of a row-major (nd, nd) array
            keep[1] = np.ascontiguousarray(keep[1].T)
            keep[2] = np.ascontiguousarray(keep[2].T)
            g = OrcGsmc(_p(keep[0]), _p(keep[1]), _p(keep[2]), float(gsmc["log_qcov_det"]))
            gp = C.byref(g)
        status = lib().orc_fault_smc(C.byref(self.st), _p(rg), nparticle, numprocs, seed, nthreads, _p(parts),
                                     _p(L), C.byref(ev), C.byref(ns), _p(gam), gp)
        return {"particles": parts, "likelihood": L, "evidence": ev.value, "nstage": ns.value,
                "gamma": gam[: ns.value].copy(), "status": status}


class OrcGsmc(C.Structure):
    _fields_ = [("qmean", C.c_void_p), ("qcov_chol", C.c_void_p), ("qcov_inv", C.c_void_p),
                ("log_qcov_det", C.c_double)]


def dc3d0(alpha, x, y, z, depth, dip, pot1, pot2, pot3, pot4):
    u = np.zeros(12)
    iret = C.c_int32()
    lib().orc_dc3d0(alpha, x, y, z, depth, dip, pot1, pot2, pot3, pot4, _p(u), C.byref(iret))
    return u, iret.value


def philox(ctr, key):
    c = np.ascontiguousarray(ctr, np.uint64)
    k = np.ascontiguousarray(key, np.uint64)
    o = np.zeros(4, np.uint64)
    lib().orc_philox4x64(_p(c), _p(k), _p(o))
    return o


def uniform(seed, stream, purpose, stage, i, j):
    return lib().orc_uniform(seed, stream, purpose, stage, i, j)


def normal(seed, stream, purpose, stage, i, d):
    return lib().orc_normal(seed, stream, purpose, stage, i, d)


def quad_uniform(seed, stream, purpose, stage):
    h, l = C.c_double(), C.c_double()
    lib().orc_quad_uniform(seed, stream, purpose, stage, C.byref(h), C.byref(l))
    return h.value, l.value


def resample(w, u_hi, u_lo):
    w = np.ascontiguousarray(w, np.float64)
    c = np.zeros(len(w), np.int32)
    lib().orc_resample(_p(w), len(w), u_hi, u_lo, _p(c))
    return c


def qsort_(arr, index):
    a = np.ascontiguousarray(arr, np.int32)
    n = C.c_int32(len(index))
    lib().orc_qsort_(_p(a), _p(index), C.byref(n))
