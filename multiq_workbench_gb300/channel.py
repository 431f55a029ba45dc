"""Batch engine API, mirroring chsim's (``simulation/chsim/src/channel.rs:233-506``).

``Engine(fields).run_batch(jobs, dc, ph) -> [Outcome]`` takes ion states x operating
settings and returns per-job outcome counts, like ``chsim::channel::Engine::run_batch``.
Every call goes through the C ABI of ``libmqgb.so`` (include/mq_engine.h) and runs on the
GPU; errors the reference turns into panics (no device, empty batch, RF not shared by the
batch) raise :class:`MqError` here.
"""
from __future__ import annotations

import ctypes as C
import os
from collections.abc import Sequence
from dataclasses import dataclass, field

import numpy as np

from . import _native as N
from .grid import Fields

MqError = N.MqError

PREC_F64 = 0
PREC_MIXED = 1
LAUNCH_DISC, LAUNCH_LEGACY, LAUNCH_GAUSSIAN = 0, 1, 2
# host-side fault injection (mq_engine_inject_fault): the engine's next stepping call fails once
FAULT_NONE, FAULT_LAUNCH_BUDGET, FAULT_ALLOC, FAULT_LAUNCH = 0, 1, 2, 3
STATUS = {0: "alive", 1: "crashed", 2: "returned", 3: "transmitted", 4: "left", 5: "timeout"}


@dataclass(frozen=True)
class Species:
    """Species (channel.rs:235-240): mass [Da], charge number, N2 CCS [A^2]."""
    mass: float
    z: float
    ccs_n2: float

    def mz(self) -> float:
        return self.mass / self.z


@dataclass(frozen=True)
class RfAc:
    """RF + AC drive of one job (channel.rs:245-247)."""
    v_rf: float
    f_rf: float
    v_ac: float
    f_ac: float


@dataclass(frozen=True)
class Job:
    """One scan point of a batch (channel.rs:250-252)."""
    sp: Species
    drive: RfAc
    n: int
    seed: int


@dataclass
class Physics:
    """Physics switches (channel.rs:254-273) plus the launch distribution."""
    legacy_force: bool = False
    legacy_collisions: bool = False
    legacy_fields: bool = False
    legacy_injection: bool = False
    legacy_criteria: bool = False
    pressure_pa: float = 0.1
    temp_k: float = 300.0
    dt: float = 4e-8
    t_max: float = 0.02
    r_inject_mm: float = 2.0
    launch: int = LAUNCH_DISC
    sigma_mm: float = 0.1
    z_inject_mm: float = 1.0
    rf_phase0: bool = True

    @classmethod
    def legacy(cls, pressure_pa: float) -> "Physics":
        return cls(True, True, True, True, True, pressure_pa, 300.0, 1e-7, 1.0, 0.0, LAUNCH_LEGACY)

    @classmethod
    def correct(cls, pressure_pa: float) -> "Physics":
        div = float(os.environ.get("CHSIM_DT_DIV", "50"))   # channel.rs:269
        return cls(False, False, False, False, False, pressure_pa, 300.0, 2e-6 / div, 0.02, 2.0, LAUNCH_DISC)

    def native(self) -> N.mq_physics:
        p = N.mq_physics()
        p.legacy_force, p.legacy_collisions, p.legacy_fields = int(self.legacy_force), int(self.legacy_collisions), int(self.legacy_fields)
        p.legacy_injection, p.legacy_criteria, p.launch = int(self.legacy_injection), int(self.legacy_criteria), int(self.launch)
        p.rf_phase0 = int(self.rf_phase0)
        p.pressure_pa, p.temp_k, p.dt, p.t_max = self.pressure_pa, self.temp_k, self.dt, self.t_max
        p.r_inject_mm, p.sigma_mm, p.z_inject_mm = self.r_inject_mm, self.sigma_mm, self.z_inject_mm
        return p

    def max_steps(self) -> int:
        import math
        return int(math.floor(self.t_max / self.dt + 0.5))


@dataclass
class Outcome:
    """Per-job counts (channel.rs:296-300)."""
    n: int = 0
    crashed: int = 0
    returned: int = 0
    transmitted: int = 0
    left: int = 0
    timeout: int = 0
    mean_coll: float = 0.0
    mean_time: float = 0.0

    def frac(self, k: int) -> float:
        return k / self.n if self.n else 0.0

    @classmethod
    def from_native(cls, o: N.mq_outcome) -> "Outcome":
        return cls(o.n, o.crashed, o.returned, o.transmitted, o.left, o.timeout, o.mean_coll, o.mean_time)


OUTCOME_DTYPE = np.dtype([("n", "<u8"), ("crashed", "<u8"), ("returned", "<u8"), ("transmitted", "<u8"), ("left", "<u8"),
                          ("timeout", "<u8"), ("mean_coll", "<f8"), ("mean_time", "<f8")])   # = mq_outcome


class Outcomes(Sequence):
    """Per-job outcomes (chsim's ``Vec<Outcome>``) held in one structured array filled by the
    engine: indexing and iteration give ``Outcome`` objects, and a column name gives all jobs'
    values at once (``outs.transmitted``), so no per-job object is built unless asked for."""

    __slots__ = ("arr",)

    def __init__(self, arr: np.ndarray):
        self.arr = arr

    @classmethod
    def empty(cls, njobs: int) -> "Outcomes":
        return cls(np.zeros(njobs, OUTCOME_DTYPE))

    def ptr(self):
        return self.arr.ctypes.data_as(C.POINTER(N.mq_outcome))

    def __len__(self) -> int:
        return len(self.arr)

    def __getitem__(self, i):
        if isinstance(i, slice):
            return [self[k] for k in range(*i.indices(len(self)))]
        r = self.arr[i]
        return Outcome(int(r["n"]), int(r["crashed"]), int(r["returned"]), int(r["transmitted"]), int(r["left"]),
                       int(r["timeout"]), float(r["mean_coll"]), float(r["mean_time"]))

    def __getattr__(self, name):
        if name in OUTCOME_DTYPE.names:
            return self.arr[name]
        raise AttributeError(name)

    def __eq__(self, other) -> bool:
        return list(self) == list(other)

    def __repr__(self) -> str:
        return f"Outcomes({len(self)} jobs)"


ION_FIELDS = (("x", np.float64), ("y", np.float64), ("z", np.float64), ("vx", np.float64), ("vy", np.float64),
              ("vz", np.float64), ("ph_rf", np.float64), ("ph_ac", np.float64), ("rng", np.uint64),
              ("steps", np.uint32), ("ncoll", np.uint32), ("leg", np.int32), ("status", np.int32), ("jid", np.uint32))


@dataclass
class IonStates:
    """Ion states, structure of arrays (the ABI's ``mq_ions``)."""
    x: np.ndarray
    y: np.ndarray
    z: np.ndarray
    vx: np.ndarray
    vy: np.ndarray
    vz: np.ndarray
    ph_rf: np.ndarray
    ph_ac: np.ndarray
    rng: np.ndarray
    steps: np.ndarray
    ncoll: np.ndarray
    leg: np.ndarray
    status: np.ndarray
    jid: np.ndarray
    _keep: list = field(default_factory=list, repr=False)

    @classmethod
    def empty(cls, n: int, pinned: bool = False) -> "IonStates":
        arrs = {}
        keep = []
        for name, dt in ION_FIELDS:
            if pinned:
                import torch   # page-locked host memory for the timed host<->device copies
                t = torch.empty(n * np.dtype(dt).itemsize, dtype=torch.uint8, pin_memory=True)
                keep.append(t)
                arrs[name] = np.frombuffer(t.numpy(), dtype=dt, count=n)
            else:
                arrs[name] = np.zeros(n, dt)
        return cls(**arrs, _keep=keep)

    def __len__(self) -> int:
        return len(self.x)

    def copy(self) -> "IonStates":
        return IonStates(**{name: getattr(self, name).copy() for name, _ in ION_FIELDS})

    def native(self) -> N.mq_ions:
        io = N.mq_ions()
        for name, dt in ION_FIELDS:
            a = getattr(self, name)
            assert a.dtype == dt and a.flags.c_contiguous, name
            setattr(io, name, a.ctypes.data)
        return io

    def pos(self) -> np.ndarray:
        return np.stack([self.x, self.y, self.z], 1)

    def vel(self) -> np.ndarray:
        return np.stack([self.vx, self.vy, self.vz], 1)


JOB_DTYPE = np.dtype([("mass", "<f8"), ("z", "<f8"), ("ccs_n2", "<f8"), ("v_rf", "<f8"), ("f_rf", "<f8"),
                      ("v_ac", "<f8"), ("f_ac", "<f8"), ("n", "<u8"), ("seed", "<u8")])
assert JOB_DTYPE.itemsize == C.sizeof(N.mq_job)


class JobTable:
    """A batch of jobs packed once into the ABI's ``mq_job`` layout (optionally in pinned host
    memory), so repeated calls pass a pointer instead of re-packing Python objects."""

    def __init__(self, arr: np.ndarray, keep=None):
        self.arr = arr
        self._keep = keep

    @classmethod
    def from_jobs(cls, jobs, pinned: bool = False) -> "JobTable":
        n = len(jobs)
        keep = None
        if pinned:
            import torch   # page-locked host memory for the per-call host-to-device copy
            keep = torch.empty(n * JOB_DTYPE.itemsize, dtype=torch.uint8, pin_memory=True)
            arr = np.frombuffer(keep.numpy(), dtype=JOB_DTYPE, count=n)
        else:
            arr = np.empty(n, JOB_DTYPE)
        arr[:] = [(j.sp.mass, j.sp.z, j.sp.ccs_n2, j.drive.v_rf, j.drive.f_rf, j.drive.v_ac, j.drive.f_ac, int(j.n),
                   int(j.seed) & 0xFFFFFFFFFFFFFFFF) for j in jobs]
        return cls(arr, keep)

    def __len__(self) -> int:
        return len(self.arr)

    def total_ions(self) -> int:
        return int(self.arr["n"].sum())

    def ptr(self):
        # data_as keeps a reference to the array, so a temporary table outlives the C call
        return self.arr.ctypes.data_as(C.POINTER(N.mq_job))

    def first(self):
        a = self.arr[0]
        return Job(Species(float(a["mass"]), float(a["z"]), float(a["ccs_n2"])),
                   RfAc(float(a["v_rf"]), float(a["f_rf"]), float(a["v_ac"]), float(a["f_ac"])), int(a["n"]), int(a["seed"]))


def jobs_native(jobs):
    """ABI pointer to a job array (packs a list; passes a JobTable through)."""
    if isinstance(jobs, JobTable):
        return jobs.ptr()
    return JobTable.from_jobs(jobs).ptr()


def _total(jobs) -> int:
    return jobs.total_ions() if isinstance(jobs, JobTable) else sum(int(j.n) for j in jobs)


@dataclass
class RunStats:
    ion_steps: int
    kernel_ms: float
    launches: int
    kernel_launches: int
    h2d_bytes: int
    d2h_bytes: int
    step_kernel_ms: float
    step_kernel_launches: int
    graph_replays: int = 0     # mixed engine: CUDA graph replays of its launch sequence
    cell_loads: int = 0        # mixed engine: cell-cache fills (8 corner node records each)
    ions_queued: int = 0       # mixed engine: ions taken from the work queue over the launches

    @classmethod
    def from_native(cls, s: N.mq_run_stats) -> "RunStats":
        return cls(s.ion_steps, s.kernel_ms, s.launches, s.kernel_launches, s.h2d_bytes, s.d2h_bytes, s.step_kernel_ms,
                   s.step_kernel_launches, s.graph_replays, s.cell_loads, s.ions_queued)


def device_count() -> int:
    return int(N.lib().mq_device_count())


class Engine:
    """GPU batch engine over one solved grid (chsim ``Engine``, channel.rs:309-340)."""

    def __init__(self, fields: Fields, precision: int = PREC_MIXED, device: int = 0):
        self.fields = fields
        self.precision = precision
        self._h = C.c_void_p()
        desc = fields.grid_desc()
        code = N.lib().mq_engine_create(C.byref(desc), int(precision), int(device), C.byref(self._h))
        N.check(code, "mq_engine_create")
        self.last_stats: RunStats | None = None

    def close(self) -> None:
        if self._h:
            N.lib().mq_engine_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def tuning(self) -> dict:
        t = N.mq_tuning()
        N.check(N.lib().mq_engine_get_tuning(self._h, C.byref(t)), "mq_engine_get_tuning", self._h)
        return dict(threads_per_block=t.threads_per_block, blocks_per_sm=t.blocks_per_sm, chunk=t.chunk,
                    use_graph=bool(t.use_graph), prefetch=bool(t.prefetch), wide_records=bool(t.wide_records),
                    sort_cells=bool(t.sort_cells))

    def set_tuning(self, blocks_per_sm: int | None = None, chunk: int | None = None, use_graph: bool | None = None,
                   prefetch: bool | None = None, wide_records: bool | None = None, sort_cells: bool | None = None) -> None:
        """Override the mixed engine's launch shape; ``wide_records`` picks 64-byte node records read
        with 256-bit loads (the default on grids below 1 GB of 48-byte records) over 48-byte ones;
        ``sort_cells`` puts every launch's live ions in the Morton order of their cells."""
        cur = self.tuning()
        t = N.mq_tuning(128, int(blocks_per_sm if blocks_per_sm is not None else cur["blocks_per_sm"]),
                        int(chunk if chunk is not None else cur["chunk"]),
                        int(use_graph if use_graph is not None else cur["use_graph"]),
                        int(prefetch if prefetch is not None else cur["prefetch"]),
                        int(wide_records if wide_records is not None else cur["wide_records"]),
                        int(sort_cells if sort_cells is not None else cur["sort_cells"]))
        N.check(N.lib().mq_engine_set_tuning(self._h, C.byref(t)), "mq_engine_set_tuning", self._h)

    def autotune(self, jobs, dc, ph: Physics, sample_per_job: int = 2048) -> tuple[dict, float]:
        """Time candidate launch shapes on a sample of the batch and keep the fastest."""
        t = N.mq_tuning()
        rate = C.c_double(0.0)
        v = (C.c_double * 4)(*[float(x) for x in dc])
        N.check(N.lib().mq_engine_autotune(self._h, jobs_native(jobs), len(jobs), v, C.byref(ph.native()),
                                           int(sample_per_job), C.byref(t), C.byref(rate)), "mq_engine_autotune", self._h)
        return self.tuning(), float(rate.value)

    def inject_fault(self, kind: int) -> None:
        """Make the next stepping call fail once, on the host (``FAULT_LAUNCH_BUDGET``: one 16-step
        launch, then the watchdog; ``FAULT_ALLOC``: out of device memory; ``FAULT_LAUNCH``: a failed
        kernel launch).  For tests of callers' error handling; nothing faults on the device."""
        N.check(N.lib().mq_engine_inject_fault(self._h, int(kind)), "mq_engine_inject_fault", self._h)

    def set_dc(self, dc) -> None:
        v = (C.c_double * 4)(*[float(x) for x in dc])
        N.check(N.lib().mq_engine_set_dc(self._h, v), "mq_engine_set_dc", self._h)

    def inject(self, jobs, ph: Physics, pinned: bool = False) -> IonStates:
        """Initial states of every job's ions in job order (chsim ``Engine::inject``)."""
        n = _total(jobs)
        ions = IonStates.empty(n, pinned)
        io = ions.native()
        js = jobs_native(jobs)
        N.check(N.lib().mq_inject(self._h, js, len(jobs), C.byref(ph.native()), C.byref(io), n), "mq_inject", self._h)
        return ions

    def run_ions(self, jobs, ph: Physics, ions: IonStates, max_more: int | None = None) -> RunStats:
        """Advance caller states in place (the core of ``run_batch_ions``)."""
        io = ions.native()
        st = N.mq_run_stats()
        mm = 0xFFFFFFFF if max_more is None else int(max_more)
        N.check(N.lib().mq_run_ions(self._h, jobs_native(jobs), len(jobs), C.byref(ph.native()), C.byref(io), len(ions), mm,
                                    C.byref(st)), "mq_run_ions", self._h)
        self.last_stats = RunStats.from_native(st)
        return self.last_stats

    def run_batch(self, jobs, dc, ph: Physics, ions_out: IonStates | None = None) -> Outcomes:
        """Run many scan points in one batch; one Outcome per job (channel.rs:437-440)."""
        out = Outcomes.empty(len(jobs))
        v = (C.c_double * 4)(*[float(x) for x in dc])
        st = N.mq_run_stats()
        io = C.byref(ions_out.native()) if ions_out is not None else None
        N.check(N.lib().mq_run_batch(self._h, jobs_native(jobs), len(jobs), v, C.byref(ph.native()), out.ptr(), io,
                                     C.byref(st)), "mq_run_batch", self._h)
        self.last_stats = RunStats.from_native(st)
        return out

    def run_batch_ions(self, jobs, dc, ph: Physics) -> tuple[IonStates, np.ndarray]:
        """Final per-ion states and the job id of each ion (channel.rs:458-475)."""
        n = _total(jobs)
        ions = IonStates.empty(n)
        self.run_batch(jobs, dc, ph, ions_out=ions)
        return ions, ions.jid.copy()


def inject(fields: Fields, jobs, ph: Physics, pinned: bool = False) -> IonStates:
    """Host injection for a grid without an engine (no device needed)."""
    n = _total(jobs)
    ions = IonStates.empty(n, pinned)
    io = ions.native()
    desc = fields.grid_desc()
    N.check(N.lib().mq_inject_grid(C.byref(desc), jobs_native(jobs), len(jobs), C.byref(ph.native()), C.byref(io), n),
            "mq_inject_grid")
    return ions


def summarize(ions: IonStates, njobs: int, dt: float) -> Outcomes:
    """Per-job outcome counts (channel.rs:496-506)."""
    out = Outcomes.empty(njobs)
    io = ions.native()
    N.check(N.lib().mq_summarize(C.byref(io), len(ions), float(dt), njobs, out.ptr()), "mq_summarize")
    return out
