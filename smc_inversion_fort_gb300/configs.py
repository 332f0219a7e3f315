"""Settings (the reference's data/setting.dat fields plus the GB300 knobs),
the named workloads and their seeded synthetic observations.

The reference ships no data, so every workload is synthetic: stations,
line-of-sight vectors, a known fault with a Gaussian-shaped slip patch and
Gaussian noise, generated from a fixed seed.  The forward model used to make
the data is passed in (the GPU Green's build in production code, the oracle
in the CPU tests).
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np


@dataclasses.dataclass
class SmcSettings:
    layout: int = 2            # 0 trace, 1 trace with fixed bends, 2 buried rectangle
    basis: int = 1             # 0 nodal (reference), 1 patch-constant
    nplane: int = 1
    nxi: tuple = (8,)
    neta: tuple = (4,)
    xbend: tuple = ()
    xmin: float = -15.0
    xmax: float = 15.0
    zmin: float = -15.0
    nquad: int = 2
    rect_hyper: int = 0
    alpha: float = 2.0 / 3.0
    max_slip: float = 4.0
    nparticle_slip: int = 500
    ntau: int = 50
    tuning_factor: int = 5
    max_stages: int = 200
    cv_inner: float = 2.0
    cv_outer: float = 0.2
    sar_corr_len: float = 10.0
    max_outer_stages: int = 0
    inner_warps: int = 0          # GPU inner kernel: warps per geometry (0: by batch size)
    inner_engine: int = 0         # inner step engine: 0 warp MMA, 1 CUDA cores, 2 tcgen05, 3 global matrix, 4 auto
    patch_km: float = 0.0         # > 0: per-geometry meshes of this patch size (rectangle layout)

    def ndim_fault(self) -> int:
        if self.layout == 0:
            return 3 * self.nplane + 3
        if self.layout == 1:
            return 2 * self.nplane + 4
        return 10 if self.rect_hyper else 8

    def dims(self) -> dict:
        nn = sum((a + 1) * (b + 1) for a, b in zip(self.nxi, self.neta))
        npatch = sum(a * b for a, b in zip(self.nxi, self.neta))
        ndof = 0
        for k, (a, b) in enumerate(zip(self.nxi, self.neta)):
            d = (a + 1) * (b + 1) - (a + 1)
            if k == 0:
                d -= b
            if k == self.nplane - 1:
                d -= b
            ndof += d
        D = 2 * ndof if self.basis == 0 else 2 * npatch
        return {"nnode": nn, "npatch": npatch, "ndof": ndof, "D": D, "ndim_fault": self.ndim_fault()}


# Prior box of the buried-rectangle layout (x, y, top, length, width, strike,
# dip, log alpha^2 [, log sigma2_sar, log sigma2_gnss]).
RECT_RANGE = np.array([[-20.0, 20.0], [-20.0, 20.0], [0.0, 10.0], [10.0, 40.0], [5.0, 20.0],
                       [0.0, 360.0], [10.0, 90.0], [-10.0, 2.0]])
RECT_TRUE = np.array([2.0, -3.0, 2.0, 24.0, 12.0, 30.0, 45.0, -3.0])
# per-geometry meshes: length 10-60 km, width 5-30 km (c3); 4-12 km x 4-8 km (tiny-uneven)
C3_RANGE = RECT_RANGE.copy()
C3_RANGE[3] = [10.0, 60.0]
C3_RANGE[4] = [5.0, 30.0]
TINY_UNEVEN_RANGE = RECT_RANGE.copy()
TINY_UNEVEN_RANGE[3] = [4.0, 12.0]
TINY_UNEVEN_RANGE[4] = [4.0, 8.0]
TINY_UNEVEN_TRUE = np.array([2.0, -3.0, 2.0, 8.0, 6.0, 30.0, 45.0, -3.0])


@dataclasses.dataclass
class Workload:
    name: str
    settings: SmcSettings
    n_outer: int
    n_gnss: int
    n_sar: int
    npath: int
    area_km: float
    sigma_h: float          # cm
    sigma_v: float          # cm
    sigma_los: float        # cm
    near_fraction: float = 0.0
    n_theta_greens: int = 0


def preset(name: str) -> Workload:
    """Named workloads: c0..c4 of the benchmark plan and small parity cases."""
    if name == "c0":
        s = SmcSettings(layout=2, basis=1, nxi=(8,), neta=(4,), nquad=2, nparticle_slip=500)
        return Workload("c0", s, 500, 60, 0, 0, 60.0, 0.2, 0.5, 1.0)
    if name == "c0-nodal":   # reference layout twin of c0 (trace + nodal basis)
        s = SmcSettings(layout=0, basis=0, nxi=(8,), neta=(4,), nquad=2, nparticle_slip=500,
                        xmin=-12.0, xmax=12.0, zmin=-12.0)
        return Workload("c0-nodal", s, 500, 60, 0, 0, 60.0, 0.2, 0.5, 1.0)
    if name == "c1":
        s = SmcSettings(layout=2, basis=1, nxi=(16,), neta=(8,), nquad=5, nparticle_slip=2)
        return Workload("c1", s, 0, 400, 0, 0, 200.0, 0.2, 0.5, 1.0, near_fraction=0.1, n_theta_greens=8192)
    if name == "c2":
        s = SmcSettings(layout=2, basis=1, nxi=(16,), neta=(8,), nquad=2, nparticle_slip=2048, sar_corr_len=5.0)
        return Workload("c2", s, 4096, 400, 2000, 2, 100.0, 1.0, 1.0, 1.0)
    if name == "c3":
        # uneven patch counts: 2.5 km patches on a 10-60 km x 5-30 km rectangle
        # give 4x2 ... 24x12 patches (D = 16 ... 576) per geometry; data as c2
        s = SmcSettings(layout=2, basis=1, nxi=(24,), neta=(12,), nquad=2, nparticle_slip=2048, sar_corr_len=5.0,
                        patch_km=2.5, inner_engine=4)
        return Workload("c3", s, 4096, 400, 2000, 2, 100.0, 1.0, 1.0, 1.0)
    if name == "tiny-uneven":
        # per-geometry meshes small enough for the oracle: 2 km patches, 2x2 ... 6x4
        s = SmcSettings(layout=2, basis=1, nxi=(6,), neta=(4,), nquad=2, nparticle_slip=64, patch_km=2.0)
        return Workload("tiny-uneven", s, 16, 12, 0, 0, 60.0, 0.2, 0.5, 1.0)
    if name == "c4":
        s = SmcSettings(layout=2, basis=1, nxi=(32,), neta=(16,), nquad=2, nparticle_slip=4096, sar_corr_len=5.0)
        return Workload("c4", s, 16384, 400, 10000, 8, 100.0, 1.0, 1.0, 1.0)
    if name in ("d160", "d256"):   # parity cases above 128 slip dimensions (10x8 and 16x8 patches)
        nxi = 10 if name == "d160" else 16
        s = SmcSettings(layout=2, basis=1, nxi=(nxi,), neta=(8,), nquad=2, nparticle_slip=64, ntau=20)
        return Workload(name, s, 16, 30, 0, 0, 60.0, 0.2, 0.5, 1.0)
    if name in ("d512", "d544", "d1024", "d1056"):
        # global-matrix engine sizes: 16x16, 17x16, 32x16 (the c4 slip size) and
        # 33x16 patches; few inner particles and short trajectories so that the
        # oracle finishes in seconds
        nxi = {"d512": 16, "d544": 17, "d1024": 32, "d1056": 33}[name]
        s = SmcSettings(layout=2, basis=1, nxi=(nxi,), neta=(16,), nquad=2, nparticle_slip=64, ntau=10)
        return Workload(name, s, 16, 30, 0, 0, 60.0, 0.2, 0.5, 1.0)
    if name == "tiny":      # parity case small enough for the oracle
        s = SmcSettings(layout=2, basis=1, nxi=(4,), neta=(2,), nquad=2, nparticle_slip=64)
        return Workload("tiny", s, 16, 12, 0, 0, 60.0, 0.2, 0.5, 1.0)
    if name == "tiny-nodal":
        s = SmcSettings(layout=0, basis=0, nxi=(4,), neta=(3,), nquad=2, nparticle_slip=64,
                        xmin=-10.0, xmax=10.0, zmin=-10.0)
        return Workload("tiny-nodal", s, 16, 12, 0, 0, 60.0, 0.2, 0.5, 1.0)
    if name == "tiny-sar":
        s = SmcSettings(layout=0, basis=0, nxi=(4,), neta=(3,), nquad=2, nparticle_slip=64,
                        xmin=-10.0, xmax=10.0, zmin=-10.0)
        return Workload("tiny-sar", s, 16, 8, 30, 2, 60.0, 0.2, 0.5, 1.0)
    if name == "tiny-2plane":
        # the reference's bent trace (init.f90:152-167): two planes meeting
        # at a free bend point (x, y) in theta, nodal basis
        s = SmcSettings(layout=0, basis=0, nplane=2, nxi=(3, 3), neta=(3, 3), nquad=2, nparticle_slip=64,
                        xmin=-10.0, xmax=10.0, zmin=-10.0)
        return Workload("tiny-2plane", s, 16, 12, 0, 0, 60.0, 0.2, 0.5, 1.0)
    if name == "tiny-3plane-fix":
        # fix_xbend = .true. (init.f90:135-150): three planes, bends at fixed
        # x, their y in theta, uneven patch counts along strike
        s = SmcSettings(layout=1, basis=0, nplane=3, nxi=(2, 3, 2), neta=(3, 3, 3), xbend=(-3.0, 4.0), nquad=2,
                        nparticle_slip=64, xmin=-10.0, xmax=10.0, zmin=-10.0)
        return Workload("tiny-3plane-fix", s, 16, 12, 0, 0, 60.0, 0.2, 0.5, 1.0)
    if name == "tiny-2plane-sar":
        # two planes with InSAR paths (exponential covariance) and GNSS
        s = SmcSettings(layout=0, basis=0, nplane=2, nxi=(3, 3), neta=(3, 3), nquad=2, nparticle_slip=64,
                        xmin=-10.0, xmax=10.0, zmin=-10.0)
        return Workload("tiny-2plane-sar", s, 16, 8, 30, 2, 60.0, 0.2, 0.5, 1.0)
    raise KeyError(name)


def _trace_truth(s: SmcSettings):
    """Bend points of the synthetic trace: on the line from (xmin, -4) to
    (xmax, 5) with an alternating 1.5 km offset; dips 50, 58, 66, ..."""
    ymin, ymax = -4.0, 5.0
    n = s.nplane
    if s.layout == 1:
        xb = np.asarray(s.xbend[: n - 1], dtype=np.float64)
    else:
        xb = s.xmin + (s.xmax - s.xmin) * np.arange(1, n) / n
    yb = ymin + (ymax - ymin) * (xb - s.xmin) / (s.xmax - s.xmin) + 1.5 * (-1.0) ** np.arange(1, n)
    dips = 50.0 + 8.0 * (np.arange(n) % 3)
    return ymin, ymax, xb, yb, dips


def true_theta(w: Workload) -> np.ndarray:
    s = w.settings
    if w.name == "tiny-uneven":
        return TINY_UNEVEN_TRUE.copy()
    if s.layout == 2:
        t = RECT_TRUE.copy()
        if s.rect_hyper:
            t = np.concatenate([t, [0.0, 0.0]])
        return t
    # trace layouts (init.f90:121-196): [ymin, ymax, bends, dip_1..n,
    # log a2, log s2_sar, log s2_gnss]; bends are (x, y) pairs (layout 0) or
    # the y of each fixed x bend (layout 1)
    ymin, ymax, xb, yb, dips = _trace_truth(s)
    if s.layout == 0:
        bends = np.ravel(np.column_stack([xb, yb])) if s.nplane > 1 else np.zeros(0)
    else:
        bends = yb
    return np.concatenate([[ymin, ymax], bends, dips, [-3.0, 0.0, 0.0]])


def prior_range(w: Workload) -> np.ndarray:
    s = w.settings
    if w.name == "c3":
        return C3_RANGE.copy()
    if w.name == "tiny-uneven":
        return TINY_UNEVEN_RANGE.copy()
    if s.layout == 2:
        r = RECT_RANGE.copy()
        if s.rect_hyper:
            r = np.concatenate([r, [[-2.0, 2.0], [-2.0, 2.0]]])
        return r
    ymin, ymax, xb, yb, dips = _trace_truth(s)
    rows = [[-10.0, 2.0], [-2.0, 10.0]]
    for k in range(s.nplane - 1):
        if s.layout == 0:
            rows.append([xb[k] - 2.0, xb[k] + 2.0])
        rows.append([yb[k] - 3.0, yb[k] + 3.0])
    rows += [[20.0, 80.0]] * s.nplane
    rows += [[-10.0, 2.0], [0.0, 0.0], [0.0, 0.0]]
    return np.array(rows)


def make_stations(w: Workload, rng: np.random.Generator):
    """Observation arrays in read_observation2's layout (init.f90:24-80)."""
    half = w.area_km / 2.0
    if w.name.startswith("c0") or w.name.startswith("tiny"):
        n = int(round(math.sqrt(w.n_gnss)))
        m = int(math.ceil(w.n_gnss / n))
        gx, gy = np.meshgrid(np.linspace(-half, half, m), np.linspace(-half, half, n))
        g = np.stack([gx.ravel(), gy.ravel()], 1)[: w.n_gnss]
        step = w.area_km / max(m - 1, 1)
        g = g + rng.uniform(-0.3 * step, 0.3 * step, g.shape)
    else:
        g = rng.uniform(-half, half, (w.n_gnss, 2))
        k = int(round(w.near_fraction * w.n_gnss))
        if k:
            # stations within 1 km of the prior-mean fault trace (strike 0 through the origin)
            g[:k, 0] = rng.uniform(-1.0, 1.0, k)
            g[:k, 1] = rng.uniform(-20.0, 20.0, k)
    sar_pts = rng.uniform(-half, half, (w.n_sar, 2)) if w.n_sar else np.zeros((0, 2))
    nobs = w.n_sar + 3 * w.n_gnss
    pts = np.zeros((nobs, 2))
    e = np.zeros((nobs, 3))
    sig = np.zeros(nobs)
    pts[: w.n_sar] = sar_pts
    if w.n_sar:
        inc = np.radians(rng.uniform(30.0, 45.0, w.n_sar))
        az = np.radians(-10.0 + rng.uniform(-5.0, 5.0, w.n_sar))
        e[: w.n_sar, 0] = -np.sin(inc) * np.cos(az)
        e[: w.n_sar, 1] = np.sin(inc) * np.sin(az)
        e[: w.n_sar, 2] = np.cos(inc)
        sig[: w.n_sar] = w.sigma_los
    for k in range(w.n_gnss):
        r = w.n_sar + 3 * k
        pts[r: r + 3] = g[k]
        e[r, 0] = e[r + 1, 1] = e[r + 2, 2] = 1.0
        sig[r: r + 2] = w.sigma_h
        sig[r + 2] = w.sigma_v
    if w.npath:
        cuts = np.linspace(0, w.n_sar, w.npath + 1).round().astype(np.int32)
        idx = (cuts + 1).astype(np.int32)
    else:
        idx = np.array([1], np.int32)
    return {"obs_points": pts, "obs_unitvec": e, "obs_sigma": sig, "nsar_index": idx, "ngnss": w.n_gnss}


def true_slip(w: Workload) -> np.ndarray:
    """Gaussian-shaped slip, 1 m peak dip slip and 0.5 m strike slip, over
    the along-strike coordinate of the whole trace (all planes) and the
    down-dip coordinate; in the DOF order of discretize_fault
    (init.f90:198-293: per plane, node rows from the bottom edge up, no DOF
    on the bottom edge or on the outer ends of the end planes) for the nodal
    basis, patch order i + nxi*j per plane for the patch-constant basis."""
    s = w.settings
    tot = sum(s.nxi[:s.nplane])

    def bump(u, v):
        return np.exp(-((u - 0.5) ** 2 / (2 * 0.18 ** 2) + (v - 0.55) ** 2 / (2 * 0.25 ** 2)))

    vals = []
    off = 0
    for p in range(s.nplane):
        nxi, neta = s.nxi[p], s.neta[p]
        if s.basis == 1:
            for j in range(neta):
                for i in range(nxi):
                    vals.append(bump((off + i + 0.5) / tot, (j + 0.5) / neta))
        else:
            for j in range(neta + 1):
                for i in range(nxi + 1):
                    if j == 0 or (p == 0 and i == 0) or (p == s.nplane - 1 and i == nxi):
                        continue
                    vals.append(bump((off + i) / tot, j / neta))
        off += nxi
    vals = np.array(vals)
    sl = np.zeros(2 * len(vals))
    sl[0::2] = 0.5 * vals
    sl[1::2] = 1.0 * vals
    return sl


def synthesize(w: Workload, greens, seed: int = 2024):
    """Seeded observations for workload w; greens(theta) -> (D, nobs) G."""
    rng = np.random.default_rng(seed)
    obs = make_stations(w, rng)
    obs["dvec"] = np.zeros(len(obs["obs_sigma"]))
    G = greens(true_theta(w), obs)
    d = G.T @ true_slip(w)
    noise = rng.standard_normal(len(d)) * obs["obs_sigma"]
    obs["dvec"] = d + noise
    return obs


def random_thetas(w: Workload, n: int, seed: int = 7) -> np.ndarray:
    rng = np.random.default_rng(seed)
    r = prior_range(w)
    return r[:, 0] + rng.uniform(0.0, 1.0, (n, len(r))) * (r[:, 1] - r[:, 0])


def mesh_of(s: SmcSettings, theta) -> tuple:
    """Patch counts of a rectangle geometry under per-geometry meshes
    (patch_km > 0): round(length / patch_km) x round(width / patch_km),
    clamped to [2, nxi[0]] x [2, neta[0]]; the fixed mesh otherwise."""
    if s.patch_km <= 0:
        return s.nxi[0], s.neta[0]

    def count(v, mx):
        if not np.isfinite(v) or v <= 0:
            return 2
        return int(min(max(np.floor(v / s.patch_km + 0.5), 2), mx))
    return count(theta[3], s.nxi[0]), count(theta[4], s.neta[0])


def fixed_mesh(w: Workload, theta) -> Workload:
    """The workload with the fixed mesh of geometry theta (per-geometry meshes off)."""
    nx, ne = mesh_of(w.settings, theta)
    return dataclasses.replace(w, settings=dataclasses.replace(w.settings, nxi=(nx,), neta=(ne,), patch_km=0.0))
