"""ctypes binding of the tandem oracle (``oracle/mqtandem.c``).  TEST INFRASTRUCTURE ONLY:
used by tests/ and bench.py's CPU baseline for the reference results of the tandem transport.

The oracle's C structs have the same memory layout as the engine's ``mq_tandem_desc`` and
``mq_tracks``; a test copies the bytes of a description into the oracle's own struct, so
no oracle call routes through product code.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import build as _build

_lib = None
NC = 21   # counters per port


class Cube(C.Structure):
    _fields_ = [("n", C.c_int32), ("array", C.c_int32)] + [
        (k, C.c_double) for k in ("d", "pitch", "height", "t_pcb", "gap", "stem_r", "clear_r", "l_ext", "ap_r",
                                  "rod_clear_extra", "cap_gap", "cap_r")
    ] + [("ent_axis", C.c_int32), ("ent_side", C.c_int32), ("ent_cell", C.c_int32 * 2),
         ("ext_axis", C.c_int32), ("ext_side", C.c_int32), ("ext_cell", C.c_int32 * 2)]


class Port(C.Structure):
    _fields_ = [("dims", C.c_int32 * 3), ("pad", C.c_int32), ("h", C.c_double), ("rf4", C.c_void_p),
                ("ac4", C.c_void_p), ("dc4", C.c_void_p), ("gate4", C.c_void_p), ("tone_khz", C.c_double),
                ("v_ac", C.c_double)]


class Species(C.Structure):
    _fields_ = [("mass", C.c_double), ("z", C.c_double), ("ccs", C.c_double), ("weight", C.c_double)]


class Desc(C.Structure):
    _fields_ = [("cube", Cube), ("cube_dims", C.c_int32 * 3), ("pad0", C.c_int32), ("cube_lo_mm", C.c_double * 3),
                ("cube_h_mm", C.c_double), ("cube_rf4", C.c_void_p), ("cube_dc4", C.c_void_p * 2),
                ("port", Port * 9), ("ch_axis_mm", C.c_double), ("ch_q1_start_mm", C.c_double),
                ("v_rf", C.c_double), ("f_rf", C.c_double), ("pressure_pa", C.c_double), ("temp_k", C.c_double),
                ("dt", C.c_double), ("gate_bias_v", C.c_double), ("nspecies", C.c_int32), ("pad2", C.c_int32),
                ("species", Species * 8)]


class Tracks(C.Structure):
    _fields_ = [(k, C.c_void_p) for k in ("x", "y", "z", "vx", "vy", "vz", "rng", "sp", "region", "last")]


TRACK_FIELDS = (("x", np.float64), ("y", np.float64), ("z", np.float64), ("vx", np.float64), ("vy", np.float64),
                ("vz", np.float64), ("rng", np.uint64), ("sp", np.int32), ("region", np.int32), ("last", np.int32))


def lib():
    global _lib
    if _lib is None:
        L = C.CDLL(str(_build.build()))
        P = C.POINTER
        L.mqt_as_built.argtypes = [P(Cube)]
        L.mqt_as_built.restype = None
        L.mqt_size.argtypes = [P(Cube)]
        L.mqt_size.restype = C.c_double
        L.mqt_n_posts.argtypes = [P(Cube)]
        L.mqt_n_posts.restype = C.c_int
        L.mqt_classify.argtypes = [P(Cube), P(C.c_double), C.c_double, P(C.c_int32)]
        L.mqt_classify.restype = C.c_int
        L.mqt_nearest_port.argtypes = [P(Cube), C.c_double, C.c_double]
        L.mqt_nearest_port.restype = C.c_int
        L.mqt_port_axis.argtypes = [P(Cube), C.c_int, P(C.c_double)]
        L.mqt_port_axis.restype = None
        L.mqt_layout.argtypes = [P(Desc), P(C.c_double), P(C.c_double), P(C.c_double)]
        L.mqt_layout.restype = None
        L.mqt_inject.argtypes = [P(Desc), C.c_uint64, C.c_int, P(Tracks), C.c_size_t]
        L.mqt_inject.restype = C.c_int
        L.mqt_enter.argtypes = [P(Tracks), C.c_size_t, C.c_int, C.c_int, C.c_double, P(C.c_double), C.c_double,
                                P(C.c_uint32)]
        L.mqt_enter.restype = None
        L.mqt_leave.argtypes = [P(Tracks), C.c_size_t, C.c_int, C.c_double, P(C.c_double), C.c_double, P(C.c_uint32)]
        L.mqt_leave.restype = None
        L.mqt_advance.argtypes = [P(Desc), P(Tracks), C.c_size_t, C.c_uint64, C.c_uint64, P(C.c_uint32), C.c_int32,
                                  P(C.c_uint64)]
        L.mqt_advance.restype = C.c_int
        _lib = L
    return _lib


def cube_from(native) -> Cube:
    """Copy a layout-identical cube geometry struct (bytes) into the oracle's own struct."""
    c = Cube()
    assert C.sizeof(native) == C.sizeof(c)
    C.memmove(C.byref(c), C.byref(native), C.sizeof(c))
    return c


def desc_from(native) -> Desc:
    d = Desc()
    assert C.sizeof(native) == C.sizeof(d)
    C.memmove(C.byref(d), C.byref(native), C.sizeof(d))
    return d


def as_built() -> Cube:
    c = Cube()
    lib().mqt_as_built(C.byref(c))
    return c


def classify(cube: Cube, p, grow: float = 0.0) -> tuple[int, int]:
    pp = (C.c_double * 3)(*[float(v) for v in p])
    s = C.c_int32(0)
    i = lib().mqt_classify(C.byref(cube), pp, float(grow), C.byref(s))
    return int(i), int(s.value)


def port_axis(cube: Cube, index: int) -> tuple[float, float]:
    xy = (C.c_double * 2)()
    lib().mqt_port_axis(C.byref(cube), int(index), xy)
    return float(xy[0]), float(xy[1])


def layout(d: Desc) -> tuple[float, float, np.ndarray]:
    seam, size, m = C.c_double(), C.c_double(), (C.c_double * 18)()
    lib().mqt_layout(C.byref(d), C.byref(seam), C.byref(size), m)
    return seam.value, size.value, np.array(m[:]).reshape(9, 2)


class State:
    """Structure-of-arrays track states."""

    def __init__(self, n: int):
        for k, dt in TRACK_FIELDS:
            setattr(self, k, np.zeros(n, dt))
        self.n = n

    def native(self) -> Tracks:
        t = Tracks()
        for k, _ in TRACK_FIELDS:
            setattr(t, k, getattr(self, k).ctypes.data)
        return t

    def copy(self) -> "State":
        s = State(self.n)
        for k, _ in TRACK_FIELDS:
            setattr(s, k, getattr(self, k).copy())
        return s


def inject(d: Desc, seed: int, mouth_start: bool, n: int) -> State:
    s = State(n)
    t = s.native()
    if lib().mqt_inject(C.byref(d), C.c_uint64(seed), 1 if mouth_start else 0, C.byref(t), n) != 0:
        raise ValueError("mqt_inject refused the description")
    return s


def advance(d: Desc, s: State, step0: int, steps: int, counts: np.ndarray | None = None, threads: int = 0,
            nsteps: np.ndarray | None = None) -> np.ndarray:
    """Advance in place; returns the (9, 21) uint32 counters (accumulated into ``counts``);
    ``nsteps`` (3 uint64: cube, driven port, idle port track-steps) accumulates if given."""
    cnt = np.zeros((9, NC), np.uint32) if counts is None else counts
    t = s.native()
    ns = nsteps.ctypes.data_as(C.POINTER(C.c_uint64)) if nsteps is not None else None
    rc = lib().mqt_advance(C.byref(d), C.byref(t), s.n, C.c_uint64(step0), C.c_uint64(steps),
                           cnt.ctypes.data_as(C.POINTER(C.c_uint32)), int(threads), ns)
    if rc != 0:
        raise ValueError(f"mqt_advance failed ({rc})")
    return cnt
