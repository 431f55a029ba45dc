"""Channel geometry and solved field bases (mirror of chsim ``Geom`` / ``Fields``).

Reference: ``simulation/chsim/src/channel.rs:16-231`` of filiprumenovski/multiq-workbench.
The solve, E field and DC combination run in ``libmqgb.so`` (C++).  Solved potentials are
cached on disk in the reference's own format so caches written by either project load in
the other: ``<cache_dir>/ch_<fnv1a64(format!("{:?}{:?}", geom, basis))>.bin`` holding the
raw little-endian f64 potential, index ``i + nx*(j + ny*k)`` (channel.rs:131-165).
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import os
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from . import _native as N

BASES = ("Rf", "Ac", "DcQ1", "DcPlate", "DcDown", "DcBox")   # chsim Basis, channel.rs:109


def _rust_f64(x: float) -> str:
    """Rust ``{:?}`` of an f64 (shortest round-trip; exponent form outside [1e-4, 1e16))."""
    if x != x:
        return "NaN"
    if x in (float("inf"), float("-inf")):
        return "inf" if x > 0 else "-inf"
    s = repr(float(x))
    if "e" in s:
        m, e = s.split("e")
        return f"{m}e{int(e)}"
    return s


@dataclass
class Geom:
    """Channel geometry in mm (channel.rs:18-44, defaults = their code)."""
    de: float = 6.35
    coef: float = 0.323
    q1_start: float = 3.0
    q1_len: float = 12.0
    alpha: float = 0.02
    gap: float = 1.0
    plate: float = 1.6
    hole_d: float = 7.0
    q2_len: float = 3.0
    stem_d: float = 4.6
    q2_flare_bug: bool = True
    grow: float = 0.0
    tilt_mode: int = 0
    ac_mode: int = 0
    mis: list = field(default_factory=lambda: [[0.0] * 4 for _ in range(4)])
    n_xy: int = 160
    h_mm: float = 0.1

    @classmethod
    def with_spacing(cls, h_mm: float, **kw) -> "Geom":
        """Default geometry at another spacing: n_xy = 16 mm / h (channel.rs:582)."""
        return cls(h_mm=h_mm, n_xy=int(round(16.0 / h_mm)), **kw)

    @classmethod
    def s14(cls, variant: str = "code", hole_d: float | None = None, **kw) -> "Geom":
        """S14 geometry variants (chsim s14_geom, channel.rs:605-619)."""
        base = dict(grow=0.4, q2_flare_bug=False)
        if variant == "inset":
            base.update(tilt_mode=1, ac_mode=1, alpha=0.525 / 12.0)
        elif variant == "paper":
            base.update(tilt_mode=1, ac_mode=1, alpha=0.01)
        elif variant == "asbuilt4":
            base.update(de=6.34, coef=(8.30 - 6.34) / 6.34, alpha=0.021, hole_d=5.75, ac_mode=1)
        elif variant == "asbuilt2":
            base.update(de=6.34, coef=(8.30 - 6.34) / 6.34, alpha=0.042, tilt_mode=1, hole_d=5.75, ac_mode=1)
        base.update(kw)
        g = cls(**base)
        if hole_d is not None:
            g.hole_d = hole_d
        return g

    def native(self) -> N.mq_geom:
        g = N.mq_geom()
        for f in ("de", "coef", "q1_start", "q1_len", "alpha", "gap", "plate", "hole_d", "q2_len", "stem_d", "grow", "h_mm"):
            setattr(g, f, float(getattr(self, f)))
        g.q2_flare_bug = 1 if self.q2_flare_bug else 0
        g.tilt_mode, g.ac_mode, g.n_xy = int(self.tilt_mode), int(self.ac_mode), int(self.n_xy)
        for i in range(4):
            for j in range(4):
                g.mis[4 * i + j] = float(self.mis[i][j])
        return g

    def dims(self) -> tuple[int, int, int]:
        d = (C.c_int32 * 3)()
        N.check(N.lib().mq_geom_dims(C.byref(self.native()), d), "mq_geom_dims")
        return int(d[0]), int(d[1]), int(d[2])

    def nz(self) -> int:
        return self.dims()[2]

    def layers(self) -> list[float]:
        out = (C.c_double * 8)()
        N.lib().mq_geom_layers(C.byref(self.native()), out)
        return list(out)

    def axis(self) -> float:
        """Channel axis coordinate in mm (x = y = axis)."""
        return float(N.lib().mq_geom_axis_mm(C.byref(self.native())))

    def z_len(self) -> float:
        return self.layers()[7]

    def r0(self) -> float:
        return (self.de + self.coef * self.de) / 2.0 ** 0.5 - self.de / 2.0

    def classify(self) -> np.ndarray:
        """Electrode code per node (0 free), shape (nz, ny, nx)."""
        nx, ny, nz = self.dims()
        out = np.zeros(nx * ny * nz, np.uint8)
        N.check(N.lib().mq_geom_classify(C.byref(self.native()), out.ctypes.data, out.size), "mq_geom_classify")
        return out.reshape(nz, ny, nx)

    def rust_debug(self) -> str:
        """``format!("{:?}", geom)`` of the reference struct (cache key)."""
        f = _rust_f64
        mis = "[" + ", ".join("[" + ", ".join(f(v) for v in row) + "]" for row in self.mis) + "]"
        return (f"Geom {{ de: {f(self.de)}, coef: {f(self.coef)}, q1_start: {f(self.q1_start)}, q1_len: {f(self.q1_len)}, "
                f"alpha: {f(self.alpha)}, gap: {f(self.gap)}, plate: {f(self.plate)}, hole_d: {f(self.hole_d)}, "
                f"q2_len: {f(self.q2_len)}, stem_d: {f(self.stem_d)}, q2_flare_bug: {'true' if self.q2_flare_bug else 'false'}, "
                f"grow: {f(self.grow)}, tilt_mode: {int(self.tilt_mode)}, ac_mode: {int(self.ac_mode)}, mis: {mis}, "
                f"n_xy: {int(self.n_xy)}, h_mm: {f(self.h_mm)} }}")


def fnv1a64(data: bytes) -> int:
    h = 1469598103934665603
    for b in data:
        h ^= b
        h = (h * 1099511628211) & 0xFFFFFFFFFFFFFFFF
    return h


def cache_dir() -> Path:
    """``$CHSIM_CACHE_DIR`` if set, else ``<repo>/_cache`` (channel.rs:138-141 uses ./cache)."""
    d = os.environ.get("CHSIM_CACHE_DIR")
    return Path(d) if d else Path(__file__).resolve().parent.parent / "_cache"


def cache_path(g: Geom, basis: int) -> Path:
    key = (g.rust_debug() + BASES[basis]).encode()
    return cache_dir() / f"ch_{fnv1a64(key):016x}.bin"


@dataclass
class SolveInfo:
    basis: str
    iterations: int
    residual: float
    seconds: float
    cached: bool


class Fields:
    """Per-volt basis fields of a geometry (chsim ``Fields``): float32 arrays of shape (n, 4)."""

    def __init__(self, geom: Geom, nx: int, ny: int, nz: int, h: float, rf, ac, dc, info=None, axis_phi=None,
                 rf_phi_near=None):
        self.geom, self.nx, self.ny, self.nz, self.h = geom, nx, ny, nz, h
        self.rf, self.ac, self.dc = rf, ac, list(dc)
        self.info: list[SolveInfo] = info or []
        # potentials kept from the solve: each basis on the axis column (i = j = nx / 2), and the RF
        # basis in a (2w + 1)^2 window around it (w >= 5 nodes and >= 0.5 mm) for the r0 fits
        self.axis_phi: dict = axis_phi or {}
        self.rf_phi_near = rf_phi_near

    @property
    def n(self) -> int:
        return self.nx * self.ny * self.nz

    @classmethod
    def build(cls, geom: Geom, tol: float = 1e-7, bases=None, threads: int = 0, cache: bool = True,
              device: int | None = None) -> "Fields":
        """Solve (or load from the cache) the bases.  ``bases`` = indices to solve (default all
        six); skipped DC bases are None and contribute nothing to ``dc_field``.  ``device``: solve
        on that CUDA device (bit-identical to the host solve) instead of the host."""
        nx, ny, nz = geom.dims()
        n = nx * ny * nz
        want = list(range(6)) if bases is None else sorted(set(int(b) for b in bases) | {0, 1})
        gn = geom.native()
        L = N.lib()
        out = {}
        info = []
        mask = None
        axis_phi, near = {}, None
        for b in want:
            e4 = np.zeros((n, 4), np.float32)
            phi = np.empty(n, np.float64)
            path = cache_path(geom, b)
            hit = False
            if cache and path.exists() and path.stat().st_size == n * 8:
                phi = np.fromfile(path, dtype="<f8")
                hit = True
                N.check(L.mq_efield_central(phi.ctypes.data, nx, ny, nz, geom.h_mm * 1e-3, e4.ctypes.data), "mq_efield_central")
                if b == 0:
                    if mask is None:
                        mask = (geom.classify().reshape(-1) != 0)
                    e4[:, 3] = mask.astype(np.float32)
                info.append(SolveInfo(BASES[b], 0, float("nan"), 0.0, True))
            else:
                st = N.mq_solve_stats()
                N.check(L.mq_channel_basis_ex(C.byref(gn), b, C.c_double(tol), int(threads),
                                              -1 if device is None else int(device), e4.ctypes.data, phi.ctypes.data,
                                              C.byref(st)), f"solve {BASES[b]}")
                info.append(SolveInfo(BASES[b], st.iterations, st.final_residual, st.seconds, False))
                if cache:
                    try:
                        path.parent.mkdir(parents=True, exist_ok=True)
                        tmp = path.with_suffix(".tmp")
                        phi.astype("<f8").tofile(tmp)
                        os.replace(tmp, path)
                    except OSError:
                        pass
            out[b] = e4
            p3 = phi.reshape(nz, ny, nx)
            a = nx // 2
            axis_phi[b] = p3[:, a, a].copy()
            if b == 0:
                w = near_window(geom.h_mm)
                near = p3[:, max(a - w, 0):a + w + 1, max(a - w, 0):a + w + 1].copy()
        dc = [out.get(b) for b in (2, 3, 4, 5)]
        return cls(geom, nx, ny, nz, geom.h_mm * 1e-3, out[0], out[1], dc, info, axis_phi, near)

    def dc_phi_axis(self, v) -> list:
        """On-axis static potential for DC voltages [q1, plate, down, box]: (z_mm, phi) per node
        (channel.rs:227-230)."""
        out = []
        for k in range(self.nz):
            p = 0.0
            for b in range(4):
                col = self.axis_phi.get(2 + b)
                if col is not None:
                    p += float(v[b]) * float(col[k])
            out.append((k * self.geom.h_mm, p))
        return out

    def dc_field(self, v) -> np.ndarray:
        """Combined static DC field for voltages [q1, plate, down, box] (channel.rs:219-226)."""
        res = np.zeros((self.n, 4), np.float32)
        ptrs = (C.c_void_p * 4)(*[(a.ctypes.data if a is not None else None) for a in self.dc])
        vv = (C.c_double * 4)(*[float(x) for x in v])
        N.check(N.lib().mq_dc_combine(self.n, ptrs, vv, res.ctypes.data), "mq_dc_combine")
        return res

    def grid_desc(self) -> N.mq_grid_desc:
        d = N.mq_grid_desc()
        d.nx, d.ny, d.nz, d.h = self.nx, self.ny, self.nz, self.h
        d.rf4, d.ac4 = self.rf.ctypes.data, self.ac.ctypes.data
        for k in range(4):
            d.dc4[k] = self.dc[k].ctypes.data if self.dc[k] is not None else None
        d.axis_mm = self.geom.axis()
        lay = self.geom.layers()
        for k in range(8):
            d.layers_mm[k] = lay[k]
        return d


def near_window(h_mm: float) -> int:
    """Half-width in nodes of the RF window kept around the axis: at least 5 nodes and 0.5 mm."""
    return max(5, int(round(0.5 / h_mm)))


def replace(g: Geom, **kw) -> Geom:
    return dataclasses.replace(g, **kw)
