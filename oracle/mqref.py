"""ctypes binding of the CPU oracle (``oracle/mqref.c``).  TEST INFRASTRUCTURE ONLY: used
by tests/, ``__graft_entry__.smoke()`` and bench.py's CPU baseline for the reference results.

The oracle takes the same inputs as the engine (a solved grid, jobs, physics, SoA ion
states) in its own C structs, so a parity test never routes through product code.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

from . import build as _build

_lib = None


class Grid(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32), ("h", C.c_double),
                ("rf4", C.c_void_p), ("ac4", C.c_void_p), ("dc4", C.c_void_p)]


class Batch(C.Structure):
    _fields_ = [("legacy_force", C.c_int32), ("legacy_collisions", C.c_int32), ("legacy_fields", C.c_int32),
                ("legacy_injection", C.c_int32), ("legacy_criteria", C.c_int32), ("launch", C.c_int32),
                ("rf_phase0", C.c_int32), ("pad0", C.c_int32), ("pressure_pa", C.c_double), ("temp_k", C.c_double),
                ("dt", C.c_double), ("t_max", C.c_double), ("r_inject_mm", C.c_double), ("sigma_mm", C.c_double),
                ("z_inject_mm", C.c_double), ("v_rf", C.c_double), ("f_rf", C.c_double), ("axis_mm", C.c_double),
                ("layers_mm", C.c_double * 8)]


class Job(C.Structure):
    _fields_ = [("mass", C.c_double), ("z", C.c_double), ("ccs_n2", C.c_double), ("v_ac", C.c_double),
                ("f_ac", C.c_double), ("n", C.c_uint64), ("seed", C.c_uint64)]


class Ions(C.Structure):
    _fields_ = [(k, C.c_void_p) for k in ("x", "y", "z", "vx", "vy", "vz", "ph_rf", "ph_ac", "rng", "steps", "ncoll",
                                          "leg", "status", "jid")]


class Outcome(C.Structure):
    _fields_ = [("n", C.c_uint64), ("crashed", C.c_uint64), ("returned", C.c_uint64), ("transmitted", C.c_uint64),
                ("left", C.c_uint64), ("timeout", C.c_uint64), ("mean_coll", C.c_double), ("mean_time", C.c_double)]


class Indep(C.Structure):
    _fields_ = [(k, C.c_double) for k in ("mass", "z", "ccs_n2", "v_rf", "f_rf", "v_ac", "f_ac", "pressure_pa", "dt",
                                          "t_max", "axis_mm", "z_exit", "z_return")] + \
               [("seed", C.c_uint64), ("rf_phase0", C.c_int32), ("pad", C.c_int32)]


class Counts(C.Structure):
    _fields_ = [(k, C.c_uint64) for k in ("n", "transmitted", "crashed", "returned", "timeout", "steps")]


FIELDS = (("x", np.float64), ("y", np.float64), ("z", np.float64), ("vx", np.float64), ("vy", np.float64),
          ("vz", np.float64), ("ph_rf", np.float64), ("ph_ac", np.float64), ("rng", np.uint64), ("steps", np.uint32),
          ("ncoll", np.uint32), ("leg", np.int32), ("status", np.int32), ("jid", np.uint32))


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(str(path))
        P = C.POINTER
        L.mqr_log.argtypes = [C.c_double]
        L.mqr_log.restype = C.c_double
        L.mqr_sincos2pi.argtypes = [C.c_double, P(C.c_double), P(C.c_double)]
        L.mqr_sincos2pi.restype = None
        L.mqr_splitmix.argtypes = [C.c_uint64]
        L.mqr_splitmix.restype = C.c_uint64
        L.mqr_max_steps.argtypes = [P(Batch)]
        L.mqr_max_steps.restype = C.c_uint32
        L.mqr_inject.argtypes = [P(Batch), P(Job), C.c_size_t, P(Ions), C.c_size_t]
        L.mqr_inject.restype = C.c_int
        L.mqr_run.argtypes = [P(Grid), P(Batch), P(Job), C.c_size_t, P(Ions), C.c_size_t, C.c_int32, P(C.c_uint64)]
        L.mqr_run.restype = C.c_int
        L.mqr_run_range.argtypes = [P(Grid), P(Batch), P(Job), C.c_size_t, P(Ions), C.c_size_t, C.c_size_t, C.c_uint32,
                                    C.c_int32, P(C.c_uint64)]
        L.mqr_run_range.restype = C.c_int
        L.mqr_summarize.argtypes = [P(Ions), C.c_size_t, P(Batch), C.c_size_t, P(Outcome)]
        L.mqr_summarize.restype = C.c_int
        L.mqr_run_independent.argtypes = [P(Grid), P(Indep), C.c_uint64, C.c_int32, P(Counts)]
        L.mqr_run_independent.restype = C.c_int
        _lib = L
    return _lib


def batch(ph, rf_v: float, rf_f: float, axis_mm: float, layers_mm) -> Batch:
    """Oracle batch constants from a Physics-like object (attribute access)."""
    b = Batch()
    b.legacy_force, b.legacy_collisions, b.legacy_fields = int(ph.legacy_force), int(ph.legacy_collisions), int(ph.legacy_fields)
    b.legacy_injection, b.legacy_criteria, b.launch = int(ph.legacy_injection), int(ph.legacy_criteria), int(ph.launch)
    b.rf_phase0 = int(ph.rf_phase0)
    b.pressure_pa, b.temp_k, b.dt, b.t_max = ph.pressure_pa, ph.temp_k, ph.dt, ph.t_max
    b.r_inject_mm, b.sigma_mm, b.z_inject_mm = ph.r_inject_mm, ph.sigma_mm, ph.z_inject_mm
    b.v_rf, b.f_rf, b.axis_mm = rf_v, rf_f, axis_mm
    for k in range(8):
        b.layers_mm[k] = layers_mm[k]
    return b


def jobs(js) -> C.Array:
    arr = (Job * len(js))()
    for k, j in enumerate(js):
        arr[k].mass, arr[k].z, arr[k].ccs_n2 = j.sp.mass, j.sp.z, j.sp.ccs_n2
        arr[k].v_ac, arr[k].f_ac, arr[k].n, arr[k].seed = j.drive.v_ac, j.drive.f_ac, int(j.n), int(j.seed) & (2 ** 64 - 1)
    return arr


class State:
    """Oracle-owned SoA ion states."""

    def __init__(self, n: int):
        self.n = n
        for name, dt in FIELDS:
            setattr(self, name, np.zeros(n, dt))

    def native(self) -> Ions:
        io = Ions()
        for name, _ in FIELDS:
            setattr(io, name, getattr(self, name).ctypes.data)
        return io

    def copy(self) -> "State":
        s = State(self.n)
        for name, _ in FIELDS:
            setattr(s, name, getattr(self, name).copy())
        return s

    @classmethod
    def from_arrays(cls, src) -> "State":
        s = cls(len(src.x))
        for name, dt in FIELDS:
            setattr(s, name, np.ascontiguousarray(getattr(src, name), dtype=dt).copy())
        return s


class Grid3:
    """Keeps the three float4 arrays alive for an oracle Grid."""

    def __init__(self, nx, ny, nz, h, rf4, ac4, dc4):
        self.arrs = [np.ascontiguousarray(a, np.float32) for a in (rf4, ac4, dc4)]
        self.g = Grid(nx, ny, nz, h, self.arrs[0].ctypes.data, self.arrs[1].ctypes.data, self.arrs[2].ctypes.data)


def inject(b: Batch, js, n: int) -> State:
    s = State(n)
    io = s.native()
    arr = jobs(js)
    if lib().mqr_inject(C.byref(b), arr, len(js), C.byref(io), n) != 0:
        raise RuntimeError("mqr_inject failed")
    return s


def run(g: Grid3, b: Batch, js, s: State, threads: int = 0, i0: int = 0, i1: int | None = None,
        max_more: int = 0xFFFFFFFF) -> int:
    io = s.native()
    arr = jobs(js)
    steps = C.c_uint64(0)
    i1 = s.n if i1 is None else i1
    if lib().mqr_run_range(C.byref(g.g), C.byref(b), arr, len(js), C.byref(io), i0, i1, max_more, int(threads),
                           C.byref(steps)) != 0:
        raise RuntimeError("mqr_run failed")
    return int(steps.value)


def summarize(s: State, b: Batch, njobs: int):
    out = (Outcome * njobs)()
    io = s.native()
    if lib().mqr_summarize(C.byref(io), s.n, C.byref(b), njobs, out) != 0:
        raise RuntimeError("mqr_summarize failed")
    return [dict(n=o.n, crashed=o.crashed, returned=o.returned, transmitted=o.transmitted, left=o.left,
                 timeout=o.timeout, mean_coll=o.mean_coll, mean_time=o.mean_time) for o in out]


def threads_default() -> int:
    return os.cpu_count() or 1


def run_independent(g: Grid3, sp, v_rf: float, f_rf: float, v_ac: float, f_ac: float, pressure_pa: float, dt: float,
                    t_max: float, axis_mm: float, z_exit: float, z_return: float, n: int, seed: int,
                    rf_phase0: bool = True, threads: int = 0) -> dict:
    """The independent per-ion form (simulation/mqviz/src/validate.rs:49-94) on a grid: counts of
    transmitted / crashed / returned / timed-out ions and the steps taken."""
    p = Indep(sp.mass, sp.z, sp.ccs_n2, v_rf, f_rf, v_ac, f_ac, pressure_pa, dt, t_max, axis_mm, z_exit, z_return,
              int(seed) & (2 ** 64 - 1), int(bool(rf_phase0)), 0)
    c = Counts()
    if lib().mqr_run_independent(C.byref(g.g), C.byref(p), int(n), int(threads), C.byref(c)) != 0:
        raise RuntimeError("mqr_run_independent failed")
    return dict(n=c.n, transmitted=c.transmitted, crashed=c.crashed, returned=c.returned, timeout=c.timeout,
                steps=c.steps)
