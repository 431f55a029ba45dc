"""Resonance fits and the secular-frequency terrain over the native library (``include/mq_fit.h``).

A sweep's per-frequency counts (k transmitted of n) become a fitted Lorentzian or Gaussian on a
flat baseline, R = f0 / FWHM with a covariance and a bootstrap error, and R in m/z terms from the
local slope d f_sec / d(m/z) of the Mathieu secular frequency along the channel axis
(simulation/mqviz/src/fit.rs, terrain.rs, analysis.rs:10-18).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _native as N

LORENTZ, GAUSS = 0, 1
SHAPE_NAMES = {LORENTZ: "Lorentzian", GAUSS: "Gaussian"}
MIN_DELTA_CHI2 = 16.0   # fit.rs:257-259
F_RF = 500e3


@dataclass
class ResFit:
    """One fitted resonance (fit.rs ``ResFit``): p = [b, A, f0, w], w the FWHM."""
    shape: int
    p: np.ndarray
    e: np.ndarray
    cov: np.ndarray
    chi2: float
    chi2_flat: float
    dof: int
    scale: float
    n_pts: int
    r: float
    r_err: float
    r_boot: tuple | None
    f0_boot: float | None
    converged: bool
    _raw: N.mq_res_fit | None = None

    @classmethod
    def _from(cls, f: N.mq_res_fit) -> "ResFit":
        return cls(int(f.shape), np.array(f.p[:]), np.array(f.e[:]), np.array(f.cov[:]).reshape(4, 4), f.chi2,
                   f.chi2_flat, int(f.dof), f.scale, int(f.n_pts), f.r, f.r_err,
                   (f.r_boot_mean, f.r_boot_sd) if f.has_boot else None, f.f0_boot_sd if f.has_boot else None,
                   bool(f.converged), f)

    @property
    def shape_name(self) -> str:
        return SHAPE_NAMES[self.shape]

    def peak(self) -> float:
        return float(self.p[0] + self.p[1])

    def delta_chi2(self) -> float:
        return float(self.chi2_flat - self.chi2)

    def chi2_red(self) -> float:
        return self.chi2 / self.dof if self.dof > 0 else float("nan")

    def at(self, x: float) -> float:
        return model(self.shape, self.p, x)


def _d(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


def _u(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.uint64)


def model(shape: int, p, x: float) -> float:
    pp = _d(p)
    return float(N.lib().mq_fit_model(int(shape), pp.ctypes.data, float(x)))


def fit_shape_sigma(shape: int, xs, ys, sg) -> ResFit | None:
    """One shape with given sigma_i (fit.rs:185-191); None for fewer than 6 points or a singular fit."""
    x, y, s = _d(xs), _d(ys), _d(sg)
    if not (len(x) == len(y) == len(s)) or len(x) < 6:
        return None
    out = N.mq_res_fit()
    rc = N.lib().mq_fit_shape_sigma(int(shape), x.ctypes.data, y.ctypes.data, s.ctypes.data, len(x), C.byref(out))
    return ResFit._from(out) if rc == 0 else None


def fit_binomial_shape(shape: int, xs, ks, ns, boot: int = 0, seed: int = 0) -> ResFit | None:
    """One shape to k of n at each x, model-based variances, ``boot`` bootstrap replicas (fit.rs:211-246)."""
    x, k, n = _d(xs), _u(ks), _u(ns)
    if not (len(x) == len(k) == len(n)):
        raise ValueError("xs, ks and ns differ in length")
    out = N.mq_res_fit()
    rc = N.lib().mq_fit_binomial_shape(int(shape), x.ctypes.data, k.ctypes.data, n.ctypes.data, len(x), int(boot),
                                       int(seed) & (2 ** 64 - 1), C.byref(out))
    return ResFit._from(out) if rc == 0 else None


def fit_binomial_curve(xs, ks, ns, boot: int = 0, seed: int = 0) -> ResFit | None:
    """Both shapes, the lower chi2 wins (fit.rs:249-255)."""
    x, k, n = _d(xs), _u(ks), _u(ns)
    if not (len(x) == len(k) == len(n)):
        raise ValueError("xs, ks and ns differ in length")
    out = N.mq_res_fit()
    rc = N.lib().mq_fit_binomial_curve(x.ctypes.data, k.ctypes.data, n.ctypes.data, len(x), int(boot),
                                       int(seed) & (2 ** 64 - 1), C.byref(out))
    return ResFit._from(out) if rc == 0 else None


def is_significant(f: ResFit, xs) -> bool:
    """Beats the flat curve by MIN_DELTA_CHI2 and is well posed over the scanned range (fit.rs:257-265)."""
    x = _d(xs)
    raw = f._raw if f._raw is not None else _raw_of(f)
    return bool(N.lib().mq_fit_is_significant(C.byref(raw), x.ctypes.data, len(x)))


def _raw_of(f: ResFit) -> N.mq_res_fit:
    r = N.mq_res_fit()
    r.shape, r.converged = f.shape, int(f.converged)
    r.p[:], r.e[:], r.cov[:] = list(f.p), list(f.e), list(np.asarray(f.cov).ravel())
    r.chi2, r.chi2_flat, r.dof, r.scale, r.n_pts, r.r, r.r_err = f.chi2, f.chi2_flat, f.dof, f.scale, f.n_pts, f.r, f.r_err
    return r


def r_mz(mz: float, dfdmz: float, fwhm: float, fwhm_err: float) -> tuple:
    """(delta m/z, its error, R_mz, its error) from a frequency FWHM (fit.rs:268-272)."""
    out = (C.c_double * 4)()
    N.lib().mq_fit_r_mz(float(mz), float(dfdmz), float(fwhm), float(fwhm_err), out)
    return tuple(out)


class Rng:
    """The statistics generator of the reference (stats.rs:152-171): xorshift64 seeded seed*phi | 1."""

    def __init__(self, seed: int):
        self.state = C.c_uint64(N.lib().mq_rng_seed(int(seed) & (2 ** 64 - 1)))

    def u(self) -> float:
        return float(N.lib().mq_rng_uniform(C.byref(self.state)))

    def binomial(self, n, p) -> np.ndarray:
        """Binomial draws for arrays n, p, in order."""
        nn, pp = _u(np.atleast_1d(n)), _d(np.broadcast_to(p, np.shape(np.atleast_1d(n))))
        out = np.zeros(len(nn), np.uint64)
        N.lib().mq_rng_binomial_fill(C.byref(self.state), nn.ctypes.data, pp.ctypes.data, len(nn), out.ctypes.data)
        return out


# ------------------------------------------------------------------ terrain

def mathieu_beta(a: float, q: float) -> float:
    return float(N.lib().mq_mathieu_beta(float(a), float(q)))


def sec_freq_khz(g_rf: float, g_dc: float, qm: float, v_rf: float, f_rf: float = F_RF) -> float:
    return float(N.lib().mq_sec_freq_khz(float(g_rf), float(g_dc), float(qm), float(v_rf), float(f_rf)))


class TerrainTables:
    """Principal-axis RF and DC-basis gradients along the channel axis (world.rs:187-231)."""

    def __init__(self, fields, axis_mm: float | None = None):
        f = fields
        axis = f.geom.axis() if axis_mm is None else axis_mm
        self.cap = max(int(min(20.0, (f.nz - 2) * f.h * 1e3) / 0.1) + 4, 8)
        self.z_mm = np.zeros(self.cap)
        self.rf = np.zeros((self.cap, 2))
        self.dc = np.zeros((4, self.cap, 2))
        rf4 = np.ascontiguousarray(f.rf, np.float32)
        dcs = [np.ascontiguousarray(b, np.float32) for b in f.dc]
        ptrs = (C.c_void_p * 4)(*[b.ctypes.data for b in dcs])
        n = C.c_size_t(0)
        rc = N.lib().mq_terrain_tables(f.nx, f.ny, f.nz, f.h, axis * 1e-3, rf4.ctypes.data, ptrs, self.cap,
                                       self.z_mm.ctypes.data, self.rf.ctypes.data, self.dc.ctypes.data, C.byref(n))
        N.check(rc, "mq_terrain_tables")
        self.n = int(n.value)

    def compute(self, species, v_rf: float, dc, f_rf: float = F_RF) -> "Terrain":
        """Secular frequencies of each species along the axis (terrain.rs:40-55)."""
        m = _d([s.mass for s in species])
        z = _d([s.z for s in species])
        dd = _d(dc)
        fx = np.zeros((len(species), self.n))
        fy = np.zeros((len(species), self.n))
        rc = N.lib().mq_terrain_compute(self.n, self.cap, self.rf.ctypes.data, self.dc.ctypes.data, m.ctypes.data,
                                        z.ctypes.data, len(species), float(v_rf), dd.ctypes.data, float(f_rf),
                                        fx.ctypes.data, fy.ctypes.data)
        N.check(rc, "mq_terrain_compute")
        return Terrain(self.z_mm[: self.n].copy(), fx, fy)

    def dfdmz(self, sp, v_rf: float, dc, f_rf: float = F_RF) -> float:
        """d f_sec / d(m/z) [kHz per m/z] at the body plateau (analysis.rs:10-18)."""
        dd = _d(dc)
        return float(N.lib().mq_terrain_dfdmz(self.n, self.cap, self.z_mm.ctypes.data, self.rf.ctypes.data,
                                              self.dc.ctypes.data, float(sp.mass), float(sp.z), float(v_rf),
                                              dd.ctypes.data, float(f_rf)))


@dataclass
class Terrain:
    """Secular frequencies [kHz] per species along z (NaN where untrapped) (terrain.rs:32-38, 57-79)."""
    z_mm: np.ndarray
    fx: np.ndarray
    fy: np.ndarray

    def plateau(self, s: int) -> float:
        """Body-plateau frequency (first z >= 6 mm, x mode)."""
        k = int(np.argmax(self.z_mm >= 6.0)) if np.any(self.z_mm >= 6.0) else 0
        return float(self.fx[s][k])

    def nearest(self, f_khz: float) -> int:
        best, bd = 0, None
        for s in range(len(self.fx)):
            p = self.plateau(s)
            if np.isfinite(p) and (bd is None or abs(p - f_khz) < bd):
                best, bd = s, abs(p - f_khz)
        return best

    @staticmethod
    def crossings(z, f, f_khz: float) -> list:
        out = []
        for k in range(1, len(f)):
            a, b = f[k - 1] - f_khz, f[k] - f_khz
            if np.isfinite(a) and np.isfinite(b) and ((a <= 0.0) != (b <= 0.0)):
                t = a / (a - b)
                out.append(z[k - 1] + t * (z[k] - z[k - 1]))
        return out
