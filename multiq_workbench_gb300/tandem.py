"""Nine-channel tandem transport (trapsim) on the GB300: a splitter cube feeding nine channel
ports and a combiner, every track advanced by the FP64 CUDA kernel behind ``mq_tandem_*``.

Python mirror of ``trapsim::Model`` (simulation/trapsim/src/lib.rs:55-336): ``TandemModel(tones,
n, seed, fine, mouth_start)`` builds the cube geometry and fields (``Geometry::as_built`` with the
3x3 port array, snapped to 1.04 / 0.52 mm), the calibrated channel world and the Fig. 5 ubiquitin
mixture, launches the tracks; ``advance(steps)`` and ``frame()`` behave as the reference's.
Each port may carry its own channel grid (``port_fields`` / ``port_grids``); by default the nine
ports share one, as in the reference.
"""
from __future__ import annotations

import ctypes as C
import hashlib
import os
from dataclasses import dataclass, field

import numpy as np

from . import _native as N
from .grid import Fields, Geom, cache_dir

DEFAULT_TONES = (39.0, 0.0, 47.0, 0.0, 0.0, 0.0, 53.0, 0.0, 59.25)   # kHz, lib.rs:13
F_RF = 500e3                                                       # world.rs:18
DT = 1.0 / F_RF / 50.0                                             # world.rs:20
Z_EXIT = 18.6e-3
Z_RETURN = 0.5e-3
DC_CAL = (18.0, 24.0, 15.0, 20.0)                                  # world.rs:33
GATE_BIAS_V = 4.0                                                  # lib.rs:196-199
# Fig. 5C control peak heights of ubiquitin 6+..10+ (presets.rs:25-27) and N2 CCS (presets.rs:20-23)
FIG5C_HEIGHT = ((6, 15.9), (7, 60.3), (8, 100.0), (9, 15.2), (10, 4.8))
REGIONS = ("split",) + tuple(f"port{i}" for i in range(9)) + ("combine", "lost", "back", "detected")
SPLIT, COMBINE, LOST, BACK, DETECTED = 0, 10, 11, 12, 13


def ubq_ccs(z: int) -> float:
    return {6: 1250.0, 7: 1262.0, 8: 1800.0, 9: 2090.0}.get(int(z), 2200.0)


@dataclass
class TandemSpecies:
    """Species of the track mixture (mqviz ``Sp``): mass [Da], charge, N2 CCS [A^2], abundance."""
    mass: float
    z: float
    ccs: float
    weight: float = 1.0

    @classmethod
    def ubq(cls, z: int, weight: float) -> "TandemSpecies":   # presets.rs:29-31
        return cls(8564.8 + z * 1.00728, float(z), ubq_ccs(z), weight)


@dataclass
class TandemPreset:
    """Drive and gas of a tandem run (mqviz ``Preset``; Fig. 5: presets.rs:51-55)."""
    species: list
    v_rf: float = 56.0
    v_ac: float = 0.20
    pressure_pa: float = 0.1
    temp_k: float = 300.0

    @classmethod
    def fig5(cls) -> "TandemPreset":
        return cls([TandemSpecies.ubq(z, h) for z, h in FIG5C_HEIGHT])


# ---------------------------------------------------------------------------------------- cube


@dataclass
class CubeGeometry:
    """trapsim ``Geometry`` in mm (geometry.rs:24-57)."""
    n: int = 10
    d: float = 6.34
    pitch: float = 8.30
    height: float = 6.34
    t_pcb: float = 1.5
    gap: float = (8.30 - 6.34) / 2.0
    stem_r: float = 2.0
    clear_r: float = 6.34 / 2.0
    l_ext: float = 6.0
    ap_r: float = 4.0
    rod_clear_extra: float = 0.5
    cap_gap: float = 2.0
    cap_r: float = 12.0
    entrance: tuple = (1, 1, (4, 4))
    exit: tuple = (2, 1, (4, 4))
    array: bool = False

    @classmethod
    def as_built(cls) -> "CubeGeometry":
        return cls.from_native(_as_built())

    @classmethod
    def code_dims(cls) -> "CubeGeometry":   # geometry.rs:58-64
        de = (83.0 - 3.0) / 10.0 / 1.323
        pitch = de * 1.323
        g = cls.as_built()
        g.d, g.pitch, g.height, g.gap, g.clear_r = de, pitch, de, (pitch - de) / 2.0, de / 2.0
        return g

    @classmethod
    def from_native(cls, c: N.mq_cube_geom) -> "CubeGeometry":
        return cls(n=c.n, d=c.d, pitch=c.pitch, height=c.height, t_pcb=c.t_pcb, gap=c.gap, stem_r=c.stem_r,
                   clear_r=c.clear_r, l_ext=c.l_ext, ap_r=c.ap_r, rod_clear_extra=c.rod_clear_extra, cap_gap=c.cap_gap,
                   cap_r=c.cap_r, entrance=(c.ent_axis, c.ent_side, (c.ent_cell[0], c.ent_cell[1])),
                   exit=(c.ext_axis, c.ext_side, (c.ext_cell[0], c.ext_cell[1])), array=bool(c.array))

    def native(self) -> N.mq_cube_geom:
        c = N.mq_cube_geom()
        c.n, c.array = int(self.n), 1 if self.array else 0
        for k in ("d", "pitch", "height", "t_pcb", "gap", "stem_r", "clear_r", "l_ext", "ap_r", "rod_clear_extra",
                  "cap_gap", "cap_r"):
            setattr(c, k, float(getattr(self, k)))
        c.ent_axis, c.ent_side = self.entrance[0], self.entrance[1]
        c.ent_cell[0], c.ent_cell[1] = self.entrance[2]
        c.ext_axis, c.ext_side = self.exit[0], self.exit[1]
        c.ext_cell[0], c.ext_cell[1] = self.exit[2]
        return c

    def snap(self, h_target: float) -> tuple["CubeGeometry", float]:
        out, h = N.mq_cube_geom(), C.c_double()
        N.check(N.lib().mq_cube_snap(C.byref(self.native()), float(h_target), C.byref(out), C.byref(h)), "mq_cube_snap")
        return CubeGeometry.from_native(out), h.value

    def c0(self) -> float:
        return self.t_pcb + self.gap + self.d / 2.0

    def lat(self, i: int) -> float:
        return self.c0() + self.pitch * i

    def r0(self) -> float:
        return self.pitch / 2.0 ** 0.5 - self.d / 2.0

    def size(self) -> float:
        return float(N.lib().mq_cube_size(C.byref(self.native())))

    def post_top_depth(self) -> float:
        return float(N.lib().mq_cube_post_top_depth(C.byref(self.native())))

    def classify(self, p, grow: float = 0.0) -> tuple[int, int]:
        pp = (C.c_double * 3)(*[float(v) for v in p])
        s = C.c_int32(0)
        i = N.lib().mq_cube_classify(C.byref(self.native()), pp, float(grow), C.byref(s))
        return int(i), int(s.value)

    def nearest_port(self, x: float, y: float) -> int:
        return int(N.lib().mq_cube_nearest_port(C.byref(self.native()), float(x), float(y)))

    def port_axis(self, index: int) -> tuple[float, float]:
        """Axis centre (mm) of exit port ``index``; ``index < 0``: the entrance."""
        xy = (C.c_double * 2)()
        N.check(N.lib().mq_cube_port_axis(C.byref(self.native()), int(index), xy), "mq_cube_port_axis")
        return float(xy[0]), float(xy[1])

    def key(self) -> str:
        return repr(sorted(self.__dict__.items()))


def _as_built() -> N.mq_cube_geom:
    c = N.mq_cube_geom()
    N.lib().mq_cube_as_built(C.byref(c))
    return c


class CubeFields:
    """trapsim ``Fields``: RF basis (w = electrode id) and the wall / entrance / exit DC bases,
    float32 (n, 4) each on the cube grid (fields.rs:28-75)."""

    def __init__(self, geom: CubeGeometry, h_mm: float, dims, lo_mm, rf, wall, ent, ext, stats=None):
        self.geom, self.h_mm = geom, h_mm
        self.dims, self.lo_mm = tuple(int(v) for v in dims), tuple(float(v) for v in lo_mm)
        self.rf, self.wall, self.ent, self.ext = rf, wall, ent, ext
        self.stats = stats or []

    @property
    def n(self) -> int:
        return self.dims[0] * self.dims[1] * self.dims[2]

    @classmethod
    def build(cls, geom: CubeGeometry, h_mm: float, grow: float = 0.4, tol: float = 1e-7, threads: int = 0,
              cache: bool = True, device: int | None = None) -> "CubeFields":
        g = geom.native()
        dims, lo = (C.c_int32 * 3)(), (C.c_double * 3)()
        L = N.lib()
        N.check(L.mq_cube_fields(C.byref(g), float(h_mm), float(grow), float(tol), int(threads), dims, lo,
                                 None, None, None, None, None), "mq_cube_fields")
        n = dims[0] * dims[1] * dims[2]
        key = hashlib.sha1(f"{geom.key()}|{h_mm!r}|{grow!r}|{tol!r}".encode()).hexdigest()[:16]
        path = cache_dir() / f"cube_{key}.npz"
        if cache and path.exists():
            z = np.load(path)
            if z["rf"].shape == (n, 4):
                return cls(geom, h_mm, dims, lo, z["rf"], z["wall"], z["ent"], z["ext"])
        arrs = [np.zeros((n, 4), np.float32) for _ in range(4)]
        st = (N.mq_solve_stats * 4)()
        N.check(L.mq_cube_fields_ex(C.byref(g), float(h_mm), float(grow), float(tol), int(threads),
                                    -1 if device is None else int(device), dims, lo, *[a.ctypes.data for a in arrs], st),
                "mq_cube_fields")
        if cache:
            try:
                path.parent.mkdir(parents=True, exist_ok=True)
                tmp = path.with_suffix(".tmp.npz")
                np.savez(tmp, rf=arrs[0], wall=arrs[1], ent=arrs[2], ext=arrs[3])
                os.replace(tmp, path)
            except OSError:
                pass
        return cls(geom, h_mm, dims, lo, *arrs, stats=[(s.iterations, s.final_residual) for s in st])

    def dc_combined(self, u0: float, uwall: float, q_in: float, q_out: float) -> np.ndarray:   # fields.rs:77-86
        out = np.zeros((self.n, 4), np.float32)
        N.check(N.lib().mq_cube_dc_combined(self.n, self.wall.ctypes.data, self.ent.ctypes.data, self.ext.ctypes.data,
                                            float(u0), float(uwall), float(q_in), float(q_out), out.ctypes.data),
                "mq_cube_dc_combined")
        return out


# ---------------------------------------------------------------------------------------- tracks


TRACK_FIELDS = (("x", np.float64), ("y", np.float64), ("z", np.float64), ("vx", np.float64), ("vy", np.float64),
                ("vz", np.float64), ("rng", np.uint64), ("sp", np.int32), ("region", np.int32), ("last", np.int32))


class Tracks:
    """Structure-of-arrays track states (region 0 split, 1..9 port, 10 combine, 11 lost, 12 back,
    13 detected; ``last`` = port of the last rejection or -1)."""

    def __init__(self, n: int, pinned: bool = False):
        self.n = int(n)
        self.pinned = bool(pinned)
        self._keep = []
        for k, dt in TRACK_FIELDS:
            if pinned:
                import torch   # page-locked host memory for the host<->device copies of an advance
                t = torch.zeros(self.n * np.dtype(dt).itemsize, dtype=torch.uint8, pin_memory=True)
                self._keep.append(t)
                setattr(self, k, np.frombuffer(t.numpy(), dtype=dt, count=self.n))
            else:
                setattr(self, k, np.zeros(self.n, dt))

    def __len__(self) -> int:
        return self.n

    def native(self) -> N.mq_tracks:
        t = N.mq_tracks()
        for k, _ in TRACK_FIELDS:
            setattr(t, k, getattr(self, k).ctypes.data)
        return t

    def copy(self, pinned: bool | None = None) -> "Tracks":
        t = Tracks(self.n, self.pinned if pinned is None else pinned)
        t.copy_from(self)
        return t

    def copy_from(self, other: "Tracks") -> None:
        """Overwrite these states with another set of the same size, in place."""
        if other.n != self.n:
            raise ValueError("track counts differ")
        for k, _ in TRACK_FIELDS:
            np.copyto(getattr(self, k), getattr(other, k))


@dataclass
class PortCounts:
    """trapsim ``Counts`` (lib.rs:29-39)."""
    entered: int = 0
    returned: int = 0
    forwarded: int = 0
    revisits: int = 0
    from_other: int = 0
    retry_from: list = field(default_factory=lambda: [0] * 9)
    reverse_entries: int = 0
    lost: int = 0
    by_charge: list = field(default_factory=lambda: [0] * 5)

    @classmethod
    def from_native(cls, c: N.mq_port_counts) -> "PortCounts":
        return cls(c.entered, c.returned, c.forwarded, c.revisits, c.from_other, list(c.retry_from),
                   c.reverse_entries, c.lost, list(c.by_charge))

    def as_array(self) -> np.ndarray:
        return np.array([self.entered, self.returned, self.forwarded, self.revisits, self.from_other,
                         *self.retry_from, self.reverse_entries, self.lost, *self.by_charge], np.uint32)


@dataclass
class Frame:
    """trapsim ``Frame`` (lib.rs:41-53): time, per-port counts, region census, in-flight points
    [x_mm, z_mm, species, id, y_mm] in the unfolded cube frame."""
    ms: float
    ports: list
    split: int
    channel: int
    combine: int
    lost: int
    back: int
    detected: int
    points: np.ndarray
    size_mm: float
    seam_mm: float


@dataclass
class TandemStats:
    """Executed track-steps by region kind, kernel time, launches and copies of one advance."""
    steps_cube: int
    steps_port: int
    steps_idle: int
    kernel_ms: float
    launches: int
    h2d_bytes: int
    d2h_bytes: int
    cell_fills_cube: int = 0   # mixed engine: cell-cache fills in the cube (8 x 32-byte records)
    cell_fills_port: int = 0   # mixed engine: cell-cache fills in the ports (8 x 48-byte records)

    @property
    def track_steps(self) -> int:
        return self.steps_cube + self.steps_port + self.steps_idle

    @classmethod
    def from_native(cls, s: N.mq_tandem_stats) -> "TandemStats":
        return cls(int(s.steps_cube), int(s.steps_port), int(s.steps_idle), float(s.kernel_ms), int(s.launches),
                   int(s.h2d_bytes), int(s.d2h_bytes), int(s.cell_fills_cube), int(s.cell_fills_port))


# ---------------------------------------------------------------------------------------- model


def _check_t(code: int, what: str, h) -> None:
    if code != N.MQ_OK:
        detail = ""
        if h is not None:
            detail = (N.lib().mq_tandem_last_error(h) or b"").decode()
        raise N.MqError(code, what, detail)


@dataclass
class PortGrid:
    """What one port reads: its channel grid's RF (w = conductor mask), AC, combined DC and gate
    plate basis, float32 (n, 4) each (the packed ``World`` of world.rs:141-160)."""
    nx: int
    ny: int
    nz: int
    h: float
    rf: np.ndarray
    ac: np.ndarray
    dc: np.ndarray
    gate: np.ndarray
    axis_mm: float
    q1_start_mm: float

    @classmethod
    def from_fields(cls, f: Fields, dc_cal=DC_CAL) -> "PortGrid":
        return cls(f.nx, f.ny, f.nz, f.h, f.rf, f.ac, f.dc_field(dc_cal), f.dc[1], f.geom.axis(), f.geom.q1_start)

    def replica(self) -> "PortGrid":
        """The same grid in arrays of its own (a port with a device-resident grid of its own)."""
        return PortGrid(self.nx, self.ny, self.nz, self.h, self.rf.copy(), self.ac.copy(), self.dc.copy(),
                        self.gate.copy(), self.axis_mm, self.q1_start_mm)


class TandemModel:
    """``trapsim::Model`` on the GB300 (lib.rs:106-336).

    ``channel``: channel basis fields (default: the calibrated S14 world, ``Geom.s14()``) shared
    by the nine ports unless ``port_fields`` (nine ``Fields``) or ``port_grids`` (nine
    ``PortGrid``) give ports grids of their own; arrays shared between ports are uploaded once.
    ``cube_h``: cube grid spacing target in mm (default 0.52 fine / 1.04 coarse).
    ``precision``: ``MQ_PREC_F64`` (the bit-exact FP64 twin) or ``MQ_PREC_MIXED`` (FP32 fields,
    compensated FP32 state, counter-based collisions: statistically equivalent, much faster)."""

    def __init__(self, tones=DEFAULT_TONES, n: int = 180, seed: int = 486, fine: bool = False,
                 mouth_start: bool = True, *, channel: Fields | None = None, port_fields=None,
                 port_grids=None, cube_h: float | None = None, preset: TandemPreset | None = None,
                 device: int = 0, dc_cal=DC_CAL, cube_tol: float = 1e-7, precision: int = N.MQ_PREC_F64):
        self.precision = int(precision)
        self.tones = tuple(float(t) for t in tones)
        assert len(self.tones) == 9
        self.preset = preset or TandemPreset.fig5()
        g = CubeGeometry.as_built()
        g.array = True
        self.geom, self.cube_h = g.snap(cube_h if cube_h is not None else (0.52 if fine else 1.04))
        self.cube = CubeFields.build(self.geom, self.cube_h, 0.4, cube_tol)
        self.dc = [self.cube.dc_combined(20.0, 20.1, 20.5, 18.0), self.cube.dc_combined(15.0, 15.1, 14.8, 15.0)]
        if port_grids is None:
            if port_fields is None:
                port_fields = [channel if channel is not None else Fields.build(Geom.s14())] * 9
            assert len(port_fields) == 9
            made = {}   # one PortGrid per distinct Fields: ports sharing a grid share its arrays
            for f in port_fields:
                if id(f) not in made:
                    made[id(f)] = PortGrid.from_fields(f, dc_cal)
            port_grids = [made[id(f)] for f in port_fields]
        assert len(port_grids) == 9
        self.port_grids = list(port_grids)
        self.desc = self._make_desc()
        self.seam, self.size, self.mouth = self.layout()
        self.axis = self.port_grids[0].axis_mm * 1e-3
        self.tracks = Tracks(n)
        t = self.tracks.native()
        N.check(N.lib().mq_tandem_inject(C.byref(self.desc), C.c_uint64(seed), 1 if mouth_start else 0, C.byref(t), n),
                "mq_tandem_inject")
        self.counts = (N.mq_port_counts * 9)()
        self.step = 0
        self.device_ms = 0.0
        self.device = int(device)
        self._h = None   # device state: fields uploaded on the first advance

    def _engine(self):
        if self._h is None:
            h = C.c_void_p()
            _check_t(N.lib().mq_tandem_create(C.byref(self.desc), self.device, C.byref(h)), "mq_tandem_create", None)
            self._h = h
        return self._h

    def _make_desc(self) -> N.mq_tandem_desc:
        d = N.mq_tandem_desc()
        d.cube = self.geom.native()
        for a in range(3):
            d.cube_dims[a] = self.cube.dims[a]
            d.cube_lo_mm[a] = self.cube.lo_mm[a]
        d.cube_h_mm = self.cube_h
        d.cube_rf4 = self.cube.rf.ctypes.data
        d.cube_dc4[0], d.cube_dc4[1] = self.dc[0].ctypes.data, self.dc[1].ctypes.data
        for i, g in enumerate(self.port_grids):
            p = d.port[i]
            p.dims[0], p.dims[1], p.dims[2] = g.nx, g.ny, g.nz
            p.h = g.h
            p.rf4, p.ac4, p.dc4, p.gate4 = g.rf.ctypes.data, g.ac.ctypes.data, g.dc.ctypes.data, g.gate.ctypes.data
            p.tone_khz = self.tones[i]
            p.v_ac = self.preset.v_ac
        d.ch_axis_mm, d.ch_q1_start_mm = self.port_grids[0].axis_mm, self.port_grids[0].q1_start_mm
        d.v_rf, d.f_rf, d.pressure_pa, d.temp_k, d.dt = (self.preset.v_rf, F_RF, self.preset.pressure_pa,
                                                         self.preset.temp_k, DT)
        d.gate_bias_v = GATE_BIAS_V
        d.precision = self.precision
        d.nspecies = len(self.preset.species)
        for k, s in enumerate(self.preset.species):
            d.species[k].mass, d.species[k].z, d.species[k].ccs, d.species[k].weight = s.mass, s.z, s.ccs, s.weight
        return d

    def layout(self) -> tuple[float, float, np.ndarray]:
        seam, size, m = C.c_double(), C.c_double(), (C.c_double * 18)()
        N.check(N.lib().mq_tandem_layout(C.byref(self.desc), C.byref(seam), C.byref(size), m), "mq_tandem_layout")
        return seam.value, size.value, np.array(m[:]).reshape(9, 2)

    def close(self) -> None:
        if getattr(self, "_h", None):
            N.lib().mq_tandem_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def advance(self, steps: int) -> "TandemStats":
        """Advance every track by ``steps`` global steps (lib.rs:176-276)."""
        h = self._engine()
        t = self.tracks.native()
        st = N.mq_tandem_stats()
        _check_t(N.lib().mq_tandem_advance(h, C.byref(t), self.tracks.n, C.c_uint64(self.step),
                                           C.c_uint64(int(steps)), self.counts, C.byref(st)), "mq_tandem_advance", h)
        self.step += int(steps)
        self.device_ms += st.kernel_ms
        self.last_stats = TandemStats.from_native(st)
        return self.last_stats

    def port_counts(self) -> list:
        return [PortCounts.from_native(c) for c in self.counts]

    def counts_array(self) -> np.ndarray:
        return np.array([PortCounts.from_native(c).as_array() for c in self.counts])

    def frame(self) -> Frame:   # lib.rs:277-336
        fc = N.mq_tandem_frame_counts()
        t = self.tracks.native()
        N.check(N.lib().mq_tandem_frame(C.byref(t), self.tracks.n, C.byref(fc)), "mq_tandem_frame")
        tr = self.tracks
        reg = tr.region
        live = reg <= COMBINE
        x, y, z = tr.x.copy(), tr.y.copy(), tr.z.copy()
        comb = reg == COMBINE
        z[comb] = 2.0 * self.seam + Z_EXIT - Z_RETURN - z[comb]
        port = (reg >= 1) & (reg <= 9)
        pi = reg[port] - 1
        x[port] = self.mouth[pi, 0] + x[port] - self.axis
        z[port] = self.seam + z[port] - Z_RETURN
        y[port] = self.mouth[pi, 1] + y[port] - self.axis
        ids = np.arange(tr.n, dtype=np.float64)
        pts = np.stack([x * 1000.0, z * 1000.0, tr.sp.astype(np.float64), ids, y * 1000.0], axis=1)[live]
        return Frame(ms=self.step * DT * 1000.0, ports=self.port_counts(), split=int(fc.split), channel=int(fc.channel),
                     combine=int(fc.combine), lost=int(fc.lost), back=int(fc.back), detected=int(fc.detected),
                     points=pts, size_mm=self.size * 1000.0, seam_mm=self.seam * 1000.0)
