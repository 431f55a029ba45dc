"""Benchmark: ion-steps/s of the batched mixed-precision engine on one GB300.

Workload (the batched sweep): 64 excitation frequencies (80-120 kHz, linear) x 8 excitation
amplitudes (0.1-1.0 V) x 32 m/z (470-532, step 2; z = +1, mass = m/z, N2 CCS = 2.95 m^(2/3))
x 256 ions = 4,194,304 ions in 16,384 jobs sharing one RF drive (100 V, 500 kHz), on the
channel geometry solved at 0.100 mm (160 x 160 x 242 nodes), DC [Q1 0, plate +5, down -5,
box 0] V, 1 mTorr N2 at 300 K, Gaussian launch sigma 0.1 mm at z = 1 mm with 300 K
Maxwell velocities, dt = 100 ns, at most 20,000 steps, legacy half-kick update rule.
Synthetic inputs (seeded); nothing is read from a dataset.

One bench step = one Engine.run_batch of that whole batch (device injection, the persistent
stepping kernel to completion, per-job counts).  ``value`` is device time (CUDA events on
the engine's stream); ``e2e`` is wall time of the public call with host-side jobs in and
outcomes out.  L2 is flushed (256 MB write) before every timed step.

``--impl reference`` times the reference's CPU algorithm (the FP64 C restatement under
oracle/) on the host cores for the same workload and metric, on a bounded sample.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "ion-steps/s, 1 GB300: batched mixed-precision vs plain FP64 at matched outcomes"
UNIT = "ion-steps/s"
# Bytes the stepping kernel must move, counted by the kernel itself: every cell-cache fill reads the
# 8 corner node records of a cell (64 or 48 B each), and every ion it takes from the queue reads its
# working state and job constants and writes them back (ION_STATE_BYTES).  The 384 B of corner
# values an ion-step interpolates (8 corners x 3 float4) come from registers between fills.
CORNERS = 8
ION_STATE_BYTES = 48 + 16 + 24 + 56 + 64   # double-floats, phase offsets, counters + key, job record; write-back


def stepping_bytes(stats, wide: bool, nearest: bool = False) -> float:
    """Algorithmic bytes of the stepping kernel(s) of one call, from the kernel's own counters: cell
    fills x 8 node records (1 record in the nearest-node field mode, which reads only the cell's
    lowest corner), plus the state traffic of every ion taken from the work queue."""
    rec = 64 if wide else 48
    return float(stats.cell_loads) * (1 if nearest else CORNERS) * rec + float(stats.ions_queued) * ION_STATE_BYTES


def cpu_model() -> str:
    """The host CPU's model name (/proc/cpuinfo, else lscpu), for the CPU baseline's line."""
    try:
        for line in Path("/proc/cpuinfo").read_text().splitlines():
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    return "unknown"


def workload(ions_per_job: int = 256, seed0: int = 0):
    import multiq_workbench_gb300 as mq
    fac = np.linspace(80e3, 120e3, 64)
    vac = np.linspace(0.1, 1.0, 8)
    mzs = [470.0 + 2 * k for k in range(32)]
    jobs = []
    for a in fac:
        for v in vac:
            for m in mzs:
                jobs.append(mq.Job(mq.Species(m, 1.0, 2.95 * m ** (2.0 / 3.0)), mq.RfAc(100.0, 500e3, float(v), float(a)),
                                   ions_per_job, seed0 + len(jobs)))
    ph = mq.Physics(legacy_force=True, pressure_pa=0.133322, temp_k=300.0, dt=1e-7, t_max=20000 * 1e-7,
                    launch=mq.LAUNCH_GAUSSIAN, sigma_mm=0.1, z_inject_mm=1.0)
    return jobs, ph, [0.0, 5.0, -5.0, 0.0]


def fields(device: int | None = None):
    """The 0.100 mm channel grid (RF, AC, plate and downstream DC bases); ``device`` solves it on
    the GPU (bit-identical to the host solve)."""
    import multiq_workbench_gb300 as mq
    return mq.Fields.build(mq.Geom(), bases=[0, 1, 3, 4], device=device)


GRID_METRIC = "ion-steps/s, 1 GB300: grid-resolution study, mixed precision vs plain FP64"
GRID_SPACINGS = (0.1, 0.05, 0.1 / 3.0)


def grid_workload(ions_per_job: int = 1000, njobs: int = 1024):
    """The grid study's launch: 1,000 ions of m/z 499 (z = +1, N2 CCS 185.6 A^2), 100 V / 500 kHz RF,
    0.5 V / 100 kHz excitation, replicated over 1,024 seeds; Gaussian sigma 0.1 mm at z = 1 mm,
    300 K, 1 mTorr, dt 100 ns, <= 20,000 steps, legacy half-kick (the corrected update loses
    every ion of this drive within a few RF periods)."""
    import multiq_workbench_gb300 as mq
    jobs = [mq.Job(mq.Species(499.0, 1.0, 185.6), mq.RfAc(100.0, 500e3, 0.5, 100e3), ions_per_job, seed)
            for seed in range(njobs)]
    ph = mq.Physics(legacy_force=True, pressure_pa=0.133322, temp_k=300.0, dt=1e-7, t_max=20000 * 1e-7,
                    launch=mq.LAUNCH_GAUSSIAN, sigma_mm=0.1, z_inject_mm=1.0)
    return jobs, ph, [0.0, 5.0, -5.0, 0.0]


def apply_tuning(eng, args) -> None:
    """Launch-shape overrides from the command line (--chunk, --sort-cells, --no-graph,
    --blocks-per-sm)."""
    kw = {}
    if args.chunk:
        kw["chunk"] = args.chunk
    if args.sort_cells:
        kw["sort_cells"] = True
    if args.blocks_per_sm:
        kw["blocks_per_sm"] = args.blocks_per_sm
    if args.no_graph:
        kw["use_graph"] = False
    if kw:
        eng.set_tuning(**kw)


def run_gridstudy(args, rank: int, world: int):
    """Config 3: the same launch on grids solved at 0.100, 0.050 and 0.0333 mm (on the GPU), the
    mixed engine timed on each, the FP64 kernel run on the same ions for counts and per-ion
    class agreement."""
    import torch
    import __graft_entry__ as ge
    import multiq_workbench_gb300 as mq
    ge.build()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    jobs, ph, dc = grid_workload(args.ions_per_job if args.ions_per_job != 256 else 1000)
    table = mq.JobTable.from_jobs(jobs, pinned=True)
    n = table.total_ions()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")
    peaks = measured_peaks()
    hbm = peaks.get("hbm_gbs") or 6800.0
    l2 = l2_read_gbs(local)
    grids = []
    clocks = Clocks(local)
    value = None
    cpu, fin_f = None, None
    spacings = [h for h in GRID_SPACINGS if not args.grid or abs(h - args.grid) < 1e-4]
    for h in spacings:
        t0 = time.perf_counter()
        f = mq.Fields.build(mq.Geom.with_spacing(h), bases=[0, 1, 3, 4], cache=False, device=local)
        t_solve = time.perf_counter() - t0
        with mq.Engine(f, mq.PREC_MIXED, device=local) as eng:
            apply_tuning(eng, args)
            tuned = eng.tuning()   # the default launch shape (a sampled autotune picks worse ones here)
            for _ in range(args.warmup):
                eng.run_batch(table, dc, ph)
            if h == spacings[-1]:
                clocks.start()
            ms, steps = [], 0
            walls = []
            launches = 0
            for _ in range(args.steps):
                flush_l2(flush)
                torch.cuda.synchronize()
                w0 = time.perf_counter()
                eng.run_batch(table, dc, ph)
                walls.append(time.perf_counter() - w0)
                ms.append(eng.last_stats.kernel_ms)
                steps = eng.last_stats.ion_steps
                launches += eng.last_stats.kernel_launches
            step_ms = eng.last_stats.step_kernel_ms
            moved = stepping_bytes(eng.last_stats, tuned["wide_records"])
            loads_per_step = eng.last_stats.cell_loads / max(steps, 1)
            ions_m = mq.IonStates.empty(n)
            om = eng.run_batch(table, dc, ph, ions_out=ions_m)
        rate = steps / (float(np.mean(ms)) * 1e-3)
        pulls, s64, agree = {}, None, None
        if not args.no_f64:
            with mq.Engine(f, mq.PREC_F64, device=local) as e64:
                ions_d = mq.IonStates.empty(n)
                o64 = e64.run_batch(table, dc, ph, ions_out=ions_d)
                s64 = e64.last_stats
            from multiq_workbench_gb300 import validate as V
            cmp = V.compare_classes(V.class_counts(om), V.class_counts(o64))
            pulls = {"chi2": cmp["chi2"], "dof": cmp["dof"], "p": cmp["p"],
                     "classes": {k: {"mixed": c["a"], "fp64": c["b"], "pull": c["pull"]} for k, c in cmp["classes"].items()}}
            agree = float(np.mean(ions_m.status == ions_d.status))
        nodes = f.nx * f.ny * f.nz
        grids.append({"h_mm": h, "dims": [f.nx, f.ny, f.nz], "nodes": nodes,
                      "node_records_gb": nodes * (64 if tuned["wide_records"] else 48) / 1e9, "solve_s": t_solve,
                      "tuning": tuned,
                      "mixed": {"value": rate, "unit": UNIT, "ms_per_step": float(np.mean(ms)), "gpu_launches": int(launches),
                                "e2e": steps / float(np.mean(walls)), "ion_steps": int(steps),
                                "cell_loads_per_ion_step": loads_per_step,
                                "achieved_gbs": moved / (step_ms * 1e-3) / 1e9,
                                "roofline_frac": moved / (step_ms * 1e-3) / 1e9 / hbm,
                                "roofline_l2_frac": (moved / (step_ms * 1e-3) / 1e9 / l2) if l2 else None},
                      "fp64_gpu": {"value": s64.ion_steps / (s64.kernel_ms * 1e-3), "unit": UNIT} if s64 else None,
                      "counts": pulls,
                      "mixed_counts": {k: int(sum(getattr(o, k) for o in om))
                                       for k in ("crashed", "returned", "transmitted", "left", "timeout")},
                      "class_agreement": agree})
        value = rate
        fin_f = f if h == spacings[-1] else None
        del f
    clk = clocks.stop()
    if fin_f is not None and not args.no_cpu and rank == 0:
        # the C oracle on the host cores, on the grid the line's value is quoted for (after the
        # clock sampling: the GPU idles meanwhile)
        r = cpu_rate(jobs, ph, dc, fin_f, 8, os.cpu_count() or 1, target_s=10.0)
        cpu = {"value": r["value"], "unit": UNIT, "cores": os.cpu_count() or 1, "cpu": cpu_model(), "kind": "port",
               "grid_mm": spacings[-1],
               "sample": f"{r['ions']} ions of {r['jobs']} evenly spaced jobs run to completion ({r['seconds']:.1f} s)"}
    del fin_f
    if rank != 0:
        return
    fin = grids[-1]
    line = {"metric": GRID_METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": fin["mixed"]["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
            "config": {"workload": f"grid study: {n:,} ions (1,000-ion m/z 499 launch x {len(jobs)} seeds), legacy "
                                   "half-kick, grids solved on the GPU at 0.100 / 0.050 / 0.0333 mm; value = the "
                                   "0.0333 mm grid", "l2_flush": "256 MB write before every timed step"},
            "e2e": {"value": fin["mixed"]["e2e"], "unit": UNIT, "h2d_bytes_per_step": int(table.arr.nbytes),
                    "d2h_bytes_per_step": int(len(jobs) * 64)},
            "gpu_launches": fin["mixed"]["gpu_launches"],
            "roofline": {"bound": "hbm", "achieved": fin["mixed"]["achieved_gbs"], "peak": hbm, "unit": "GB/s",
                         "frac": fin["mixed"]["roofline_frac"], "traffic": None,
                         "peak_source": "measured hbm_gbs" if peaks.get("hbm_gbs") else "fallback",
                         "kernel": "k_mixed",
                         "algorithmic_bytes": "cell fills counted by the kernel x 8 node records (48 B) + "
                                              f"{ION_STATE_BYTES} B per ion taken from the queue",
                         "cell_loads_per_ion_step": fin["mixed"]["cell_loads_per_ion_step"]},
            "roofline_l2": {"achieved": fin["mixed"]["achieved_gbs"], "peak": l2, "unit": "GB/s",
                            "frac": fin["mixed"]["roofline_l2_frac"],
                            "peak_source": "L2 read bandwidth measured in this run (mq_measure_l2_read_gbs)"},
            "cpu_baseline": cpu, "clocks": clk, "grids": grids}
    return line


LEGACY_METRIC = "ion-steps/s, 1 GB300: legacy Fig. 4 mass scan (legacy collisions), mixed precision vs plain FP64"


def legacy_workload(replicas: int = 16):
    """The reference's legacy Fig. 4 scan (chsim legacy-fig4): m/z 475..525 step 2 (26 values) of 5+
    ions (mass 5 m/z), 100 V / 500 kHz RF, 0.5 V / 100 kHz excitation, DC [0, +5, -5, 0] V, every
    legacy switch (half kick, stationary-gas collisions every mean free path, nearest-node fields,
    point-and-cone launch, legacy criteria), 1 mTorr; 1,000 ions per m/z, replicated over ``replicas``
    seed sets to fill the GPU (26,000 x replicas ions); at most 20,000 steps of 100 ns per ion, the
    step cap of every benchmark configuration (the preset's 1 s would let single ions run 10^7 steps)."""
    import multiq_workbench_gb300 as mq
    from multiq_workbench_gb300 import chsim as CH
    mzs = [475.0 + 2.0 * i for i in range(26)]
    jobs = [mq.Job(mq.Species(mz * 5.0, 5.0, 0.0), CH.FIG4_DRIVE, 1000, 1000 * r + int(mz))
            for r in range(replicas) for mz in mzs]
    ph = mq.Physics.legacy(1e-3 * 133.322)
    ph.t_max = 20000 * ph.dt
    return jobs, ph, list(CH.FIG4_DC)


def run_legacy(args, rank: int, world: int):
    """The legacy-collision path: the Fig. 4 scan x 16 seed sets (416,000 ions, <= 20,000 steps) on the 0.100 mm grid,
    the mixed engine timed (``k_mixed`` with legacy collisions), the FP64 kernel on one seed set
    (26,000 ions) for the speed ratio and the class counts, and the CPU oracle on a sample."""
    import torch
    import __graft_entry__ as ge
    import multiq_workbench_gb300 as mq
    from multiq_workbench_gb300 import validate as V
    ge.build()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    jobs, ph, dc = legacy_workload(args.replicas)
    if rank:
        jobs = [mq.Job(j.sp, j.drive, j.n, j.seed + rank_seed0(rank)) for j in jobs]
    f = mq.Fields.build(mq.Geom(), bases=[0, 1, 3, 4], cache=False, device=local)
    table = mq.JobTable.from_jobs(jobs, pinned=True)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")
    eng = mq.Engine(f, mq.PREC_MIXED, device=local)
    apply_tuning(eng, args)
    tuned = eng.tuning()
    for _ in range(args.warmup):
        eng.run_batch(table, dc, ph)
    clocks = Clocks(local)
    clocks.start()
    ms, step_ms, walls, steps, moved, loads, launches = [], [], [], 0, 0.0, 0, 0
    for _ in range(args.steps):
        flush_l2(flush)
        torch.cuda.synchronize()
        w0 = time.perf_counter()
        out = eng.run_batch(table, dc, ph)
        walls.append(time.perf_counter() - w0)
        st = eng.last_stats
        ms.append(st.kernel_ms)
        step_ms.append(st.step_kernel_ms)
        steps += st.ion_steps
        moved += stepping_bytes(st, tuned["wide_records"], ph.legacy_fields)
        loads += st.cell_loads
        launches += st.kernel_launches
        h2d, d2h = st.h2d_bytes, st.d2h_bytes
    clk = clocks.stop()
    (t_dev, t_wall), (steps_all,) = reduce_over_ranks([sum(ms) * 1e-3, sum(walls)], [steps], f"cuda:{local}")
    if rank != 0:
        eng.close()
        return
    sample = jobs[:26]
    om = eng.run_batch(sample, dc, ph)
    sm = eng.last_stats
    eng.close()
    extra = {}
    if not args.no_f64:
        with mq.Engine(f, mq.PREC_F64, device=local) as e64:
            o64 = e64.run_batch(sample, dc, ph)
            s64 = e64.last_stats
        cmp = V.compare_classes(V.class_counts(om), V.class_counts(o64))
        extra["fp64_gpu"] = {"value": s64.ion_steps / (s64.kernel_ms * 1e-3), "unit": UNIT,
                             "mixed_same_sample": sm.ion_steps / (sm.kernel_ms * 1e-3),
                             "speedup_mixed_over_fp64": (sm.ion_steps / sm.kernel_ms) / (s64.ion_steps / s64.kernel_ms),
                             "sample": "one seed set: 26 m/z x 1,000 ions",
                             "outcomes": {"chi2": cmp["chi2"], "dof": cmp["dof"], "p": cmp["p"],
                                          "classes": {k: {"mixed": c["a"], "fp64": c["b"], "pull": c["pull"]}
                                                      for k, c in cmp["classes"].items()}}}
    cpu = None
    if not args.no_cpu:
        r = cpu_rate(jobs, ph, dc, f, 26, os.cpu_count() or 1, target_s=12.0)
        cpu = {"value": r["value"], "unit": UNIT, "cores": os.cpu_count() or 1, "cpu": cpu_model(), "kind": "port",
               "sample": f"{r['ions']} ions of {r['jobs']} evenly spaced jobs run to completion ({r['seconds']:.1f} s)"}
    peaks = measured_peaks()
    hbm = peaks.get("hbm_gbs") or 6800.0
    l2 = l2_read_gbs(local)
    kern_s = sum(step_ms) * 1e-3
    achieved = moved / kern_s / 1e9
    line = {"metric": LEGACY_METRIC, "value": steps_all / t_dev, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t_dev / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
            "config": {"workload": f"legacy Fig. 4 scan: 26 m/z (475-525) x 1,000 ions x {args.replicas} seed sets "
                                   f"({table.total_ions():,} ions), Physics::legacy(1 mTorr), <=20000 steps, 0.100 mm grid",
                       "l2_flush": "256 MB write before every timed step", "tuning": tuned},
            "ion_steps_per_step": steps / args.steps,
            "e2e": {"value": steps_all / t_wall, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
            "gpu_launches": int(launches),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                         "traffic": None, "peak_source": "measured hbm_gbs" if peaks.get("hbm_gbs") else "fallback",
                         "kernel": "k_mixed (legacy collisions, nearest-node fields)",
                         "algorithmic_bytes": f"cell fills counted by the kernel x 1 node record ({64 if tuned['wide_records'] else 48} B) "
                                              f"+ {ION_STATE_BYTES} B per ion taken from the queue",
                         "cell_loads_per_ion_step": loads / max(steps, 1)},
            "roofline_l2": {"achieved": achieved, "peak": l2, "unit": "GB/s", "frac": achieved / l2 if l2 else None},
            "cpu_baseline": cpu, "clocks": clk,
            "outcomes": {k: int(getattr(out, k).sum()) for k in V.CLASSES}}
    line.update(extra)
    return line


class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int = 0):
        self.index = index
        self.rows = []
        self.proc = None
        self.t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        sm = [float(r[1]) for r in self.rows if len(r) >= 9 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) >= 9 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            if len(r) >= 9:
                for k, nm in enumerate(names):
                    if r[5 + k].lower().startswith("active"):
                        reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return json.loads(p.read_text())
        except ValueError:
            pass
    return {}


def cpu_rate(jobs, ph, dc, f, sample_jobs: int, threads: int, target_s: float | None = None) -> dict:
    """The FP64 CPU restatement of the reference integrator on a bounded sample of the batch:
    ``sample_jobs`` evenly spaced jobs, run to completion.  With ``target_s`` the sample is
    first sized so that the timed run takes about that long."""
    from oracle import mqref as R
    g = f.geom
    dcf = f.dc_field(dc)
    G = R.Grid3(f.nx, f.ny, f.nz, f.h, f.rf, f.ac, dcf)

    def one(k: int):
        step = max(1, len(jobs) // k)
        js = jobs[::step][:k]
        b = R.batch(ph, js[0].drive.v_rf, js[0].drive.f_rf, g.axis(), g.layers())
        n = sum(j.n for j in js)
        s = R.inject(b, js, n)
        t0 = time.perf_counter()
        steps = R.run(G, b, js, s, threads=threads)
        return steps, time.perf_counter() - t0, n, len(js)

    k = sample_jobs
    if target_s:
        steps, dt, _, _ = one(k)
        k = int(min(len(jobs), max(k, k * target_s / max(dt, 1e-3))))
    steps, dt, n, nj = one(k)
    return {"value": steps / dt, "steps": steps, "seconds": dt, "ions": n, "jobs": nj}


def reduce_over_ranks(times, counts, device) -> tuple[list, list]:
    """Whole-job figures of replicas: the slowest rank's times and the sum of every rank's
    counts (one all-reduce each; a no-op without an initialised process group)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return [float(t) for t in times], [float(c) for c in counts]
    tt = torch.tensor([float(t) for t in times], dtype=torch.float64, device=device)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    cc = torch.tensor([float(c) for c in counts], dtype=torch.float64, device=device)
    dist.all_reduce(cc, op=dist.ReduceOp.SUM)
    return tt.tolist(), cc.tolist()


def rank_seed0(rank: int) -> int:
    """First job seed of a rank's replica of the workload (disjoint seed ranges per rank)."""
    return rank * 1_000_003


def l2_read_gbs(device: int) -> float | None:
    """L2 read bandwidth measured in this run (32 MiB resident buffer, 200 sweeps, L1 bypassed),
    the denominator of the gather kernels' L2 roofline."""
    import ctypes as C
    from multiq_workbench_gb300 import _native as N
    best = None
    for _ in range(3):
        g = C.c_double(0.0)
        if N.lib().mq_measure_l2_read_gbs(int(device), 32 << 20, 200, C.byref(g)) == 0:
            best = g.value if best is None else max(best, g.value)
    return best


def flush_l2(buf):
    buf.fill_(1)


def run_reference(args, rank: int, world: int):
    if rank != 0:
        return
    jobs, ph, dc = workload()
    f = fields()
    threads = os.cpu_count() or 1
    vals = []
    # size one step to ~10 s of CPU work; warm-up steps run a small sample untimed
    probe = cpu_rate(jobs, ph, dc, f, 128, threads)
    sample = int(min(len(jobs), max(128, 128 * 10.0 / max(probe["seconds"], 1e-3))))
    for _ in range(max(0, args.warmup)):
        cpu_rate(jobs, ph, dc, f, 64, threads)
    r = None
    t_all = time.perf_counter()
    for _ in range(args.steps):
        r = cpu_rate(jobs, ph, dc, f, sample, threads)
        vals.append(r["value"])
    wall = time.perf_counter() - t_all
    v = float(np.median(vals))
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * wall / max(1, args.steps), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "batched sweep 64 f_ac x 8 V_ac x 32 m/z x 256 ions (4,194,304 ions), 0.100 mm grid, legacy half-kick",
                       "sample": f"{r['jobs']} of the 16384 jobs, evenly spaced, all their ions: {r['ions']} ions per step"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "cpu": cpu_model(), "kind": "port",
                             "sample": f"{r['ions']} ions of {r['jobs']} evenly spaced jobs, run to completion"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


TANDEM_METRIC = "track-steps/s, 1 GB300: nine-channel tandem transport, mixed precision vs plain FP64 at matched counts"
TANDEM_UNIT = "track-steps/s"
# algorithmic bytes per track-step: 8 corner nodes x float4 (16 B) x the fields the region reads
# (the mixed engine folds the gate bias of idle ports into their DC records)
TANDEM_BYTES = {"f64": {"cube": 8 * 16 * 2, "port": 8 * 16 * 3, "idle": 8 * 16 * 4},
                "mixed": {"cube": 8 * 16 * 2, "port": 8 * 16 * 3, "idle": 8 * 16 * 3}}


def tandem_setup(args, rank: int = 0, precision: int = 1, grids=None):
    """The tandem workload: Fig. 5 drives (tones 39 / 47 / 53 / 59.25 kHz on four ports, five
    idle ports gated +4 V), ubiquitin 6+..10+ mixture, tracks launched at the nine mouths, cube at
    0.51875 mm, the nine ports on the calibrated S14 channel grid at ``--port-h`` mm, each port
    holding its own device-resident copy of that grid unless ``--tandem-shared``."""
    import multiq_workbench_gb300 as mq
    h = float(args.port_h)
    if grids is None:
        ch = mq.Fields.build(mq.Geom.s14(h_mm=h, n_xy=int(round(16.0 / h))))
        pg = mq.PortGrid.from_fields(ch)
        grids = [pg] * 9 if args.tandem_shared else [pg] + [pg.replica() for _ in range(8)]
    m = mq.TandemModel(mq.DEFAULT_TONES, n=args.tracks, seed=486 + rank_seed0(rank), fine=True, mouth_start=True,
                       port_grids=grids, precision=precision)
    g0 = grids[0]
    wl = (f"tandem: {args.tracks:,} tracks at the nine mouths, Fig. 5 tones, ubiquitin 6+..10+, cube 0.51875 mm "
          f"{'x'.join(map(str, m.cube.dims))}, ports on S14 {h:g} mm {g0.nx}x{g0.ny}x{g0.nz} "
          f"({'one shared grid' if args.tandem_shared else 'nine device-resident copies'}), "
          f"{args.tandem_steps} global steps per bench step")
    return m, wl


def tandem_bytes(st, kind: str = "mixed") -> float:
    """Corner bytes the FP64 kernel gathers per track-step (it reads every corner every step)."""
    b = TANDEM_BYTES[kind]
    return b["cube"] * st.steps_cube + b["port"] * st.steps_port + b["idle"] * st.steps_idle


TRACK_STATE_BYTES = 68 + 56   # k_tm_step: a track's working state read and written once per launch


def tandem_moved(st, tracks: int) -> float:
    """Bytes the mixed tandem's step kernel must move, from its own counters: cell-cache fills (cube:
    8 x 32-byte records; port: 8 x 48-byte records) plus every track's state once per launch (the
    advance's launches are a load, a store, and a bucket + step pair per 256-step chunk)."""
    chunks = max((st.launches - 2) // 2, 0)
    return st.cell_fills_cube * 8 * 32 + st.cell_fills_port * 8 * 48 + float(tracks) * TRACK_STATE_BYTES * chunks


def tandem_cpu(m, pulse, steps: int, target_s: float, threads: int) -> dict:
    """The tandem oracle on the first k tracks of the pulse for the same global steps, k grown
    until the run takes about ``target_s``."""
    from oracle import mqtandem as O
    d = O.desc_from(m.desc)
    k = min(pulse.n, 2048)
    while True:
        s = O.State(k)
        for name, _ in O.TRACK_FIELDS:
            getattr(s, name)[:] = getattr(pulse, name)[:k]
        ns = np.zeros(3, np.uint64)
        t0 = time.perf_counter()
        O.advance(d, s, 0, steps, threads=threads, nsteps=ns)
        dt = time.perf_counter() - t0
        if dt >= 0.3 * target_s or k >= pulse.n:
            return {"value": float(ns.sum()) / dt, "track_steps": int(ns.sum()), "seconds": dt, "tracks": k}
        k = int(min(pulse.n, k * max(2.0, target_s / max(dt, 1e-3))))


def run_tandem(args, rank: int, world: int):
    import multiq_workbench_gb300 as mq
    threads = os.cpu_count() or 1
    if args.impl == "reference":
        if rank != 0:
            return
        m, wl = tandem_setup(args)
        pulse = m.tracks.copy()
        vals = []
        r = None
        for _ in range(max(0, args.warmup)):
            tandem_cpu(m, pulse, min(args.tandem_steps, 200), 1.0, threads)
        t_all = time.perf_counter()
        for _ in range(args.steps):
            r = tandem_cpu(m, pulse, args.tandem_steps, 10.0, threads)
            vals.append(r["value"])
        wall = time.perf_counter() - t_all
        v = float(np.median(vals))
        smp = f"first {r['tracks']} tracks of the pulse for {args.tandem_steps} steps ({r['seconds']:.1f} s)"
        print(json.dumps({"impl": "reference", "metric": TANDEM_METRIC, "value": v, "unit": TANDEM_UNIT, "n_gpus": world,
                          "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * wall / max(1, args.steps),
                          "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                          "data": "synthetic", "config": {"workload": wl, "sample": smp},
                          "cpu_baseline": {"value": v, "unit": TANDEM_UNIT, "cores": threads, "cpu": cpu_model(), "kind": "port",
                                           "sample": smp},
                          "e2e": {"value": v, "unit": TANDEM_UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}),
              flush=True)
        return
    import torch
    import __graft_entry__ as ge
    ge.build()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    m, wl = tandem_setup(args, rank, mq.PREC_MIXED)
    m.device = local
    pulse = m.tracks.copy()
    work = m.tracks.copy(pinned=True)   # the advance's host buffers: page-locked, filled from the pulse
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")

    def one(model=m):
        work.copy_from(pulse)
        model.tracks = work
        model.step = 0
        model.counts = type(model.counts)()
        t0 = time.perf_counter()
        st = model.advance(args.tandem_steps)
        return st, time.perf_counter() - t0

    for _ in range(args.warmup):
        one()
    clocks = Clocks(local)
    clocks.start()
    sts, walls = [], []
    torch.cuda.synchronize()
    for _ in range(args.steps):
        flush_l2(flush)
        torch.cuda.synchronize()
        st, w = one()
        sts.append(st)
        walls.append(w)
    torch.cuda.synchronize()
    clk = clocks.stop()
    ts = sum(s.track_steps for s in sts)
    t_dev = sum(s.kernel_ms for s in sts) * 1e-3
    t_wall = sum(walls)
    # replicas: every rank runs its own pulse; whole-job rate over the slowest rank
    (t_dev, t_wall), (ts_all,) = reduce_over_ranks([t_dev, t_wall], [ts], f"cuda:{local}")
    value = ts_all / t_dev
    e2e = ts_all / t_wall
    if rank != 0:
        m.close()
        return
    peaks = measured_peaks()
    hbm = peaks.get("hbm_gbs") or 6800.0
    l2 = l2_read_gbs(local)
    achieved = sum(tandem_moved(s, args.tracks) for s in sts) / (sum(s.kernel_ms for s in sts) * 1e-3) / 1e9
    fills = sum(s.cell_fills_cube + s.cell_fills_port for s in sts) / max(sum(s.track_steps for s in sts), 1)
    f = m.frame()
    cnt = m.counts_array()
    extra = {}
    if not args.no_f64:
        # the FP64 kernel (bit-exact with the oracle) on the same pulse: speed and matched counts
        m64, _ = tandem_setup(args, rank, mq.PREC_F64, grids=m.port_grids)
        m64.device = local
        s64, _ = one(m64)
        c64 = m64.counts_array()
        f64 = m64.frame()
        m64.close()

        def pull(a, b):
            return (a - b) / math.sqrt(max(a + b, 1))
        cmp = {}
        for name, a, b in (("entered", cnt[:, 0].sum(), c64[:, 0].sum()), ("returned", cnt[:, 1].sum(), c64[:, 1].sum()),
                           ("lost_in_ports", cnt[:, 15].sum(), c64[:, 15].sum()), ("split", f.split, f64.split),
                           ("channel", f.channel, f64.channel), ("lost", f.lost, f64.lost)):
            cmp[name] = {"mixed": int(a), "fp64": int(b), "pull": pull(float(a), float(b))}
        extra["fp64_gpu"] = {"value": s64.track_steps / (s64.kernel_ms * 1e-3), "unit": TANDEM_UNIT,
                             "speedup_mixed_over_fp64": (ts / t_dev) / (s64.track_steps / (s64.kernel_ms * 1e-3)),
                             "fp64_note": "GB300's FP64 rate is a small fraction of its FP32 rate, which the ratio reflects",
                             "roofline_achieved_gbs": tandem_bytes(s64, "f64") / (s64.kernel_ms * 1e-3) / 1e9,
                             "sample": "the same pulse and steps", "counts": cmp}
    cpu = None
    if not args.no_cpu:
        r = tandem_cpu(m, pulse, args.tandem_steps, 12.0, threads)
        cpu = {"value": r["value"], "unit": TANDEM_UNIT, "cores": threads, "cpu": cpu_model(), "kind": "port",
               "sample": f"first {r['tracks']} tracks of the pulse for {args.tandem_steps} steps ({r['seconds']:.1f} s)"}
    last = sts[-1]
    line = {"metric": TANDEM_METRIC, "value": value, "unit": TANDEM_UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t_dev / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
            "config": {"workload": wl, "tracks": args.tracks, "global_steps": args.tandem_steps,
                       "l2_flush": "256 MB write before every timed step"},
            "track_steps_per_step": ts / args.steps,
            "e2e": {"value": e2e, "unit": TANDEM_UNIT, "h2d_bytes_per_step": int(last.h2d_bytes),
                    "d2h_bytes_per_step": int(last.d2h_bytes)},
            "gpu_launches": int(sum(s.launches for s in sts)),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                         "traffic": None, "peak_source": "measured hbm_gbs" if peaks.get("hbm_gbs") else "fallback",
                         "kernel": "k_tm_step",
                         "algorithmic_bytes": "cell fills counted by the kernel x 8 records (cube 32 B, port 48 B) + "
                                              f"{TRACK_STATE_BYTES} B per track per 256-step launch",
                         "cell_fills_per_track_step": fills},
            "roofline_l2": {"achieved": achieved, "peak": l2, "unit": "GB/s", "frac": achieved / l2 if l2 else None,
                            "peak_source": "L2 read bandwidth measured in this run (mq_measure_l2_read_gbs)"},
            "cpu_baseline": cpu, "clocks": clk,
            "census": {"split": f.split, "channel": f.channel, "combine": f.combine, "lost": f.lost, "back": f.back,
                       "detected": f.detected},
            "ports": {"entered": cnt[:, 0].tolist(), "returned": cnt[:, 1].tolist(), "forwarded": cnt[:, 2].tolist(),
                      "revisits": int(cnt[:, 3].sum()), "from_other": int(cnt[:, 4].sum()),
                      "retry_matrix": cnt[:, 5:14].tolist(), "reverse_entries": int(cnt[:, 14].sum()),
                      "lost": cnt[:, 15].tolist(), "by_charge": cnt[:, 16:21].sum(0).tolist()}}
    line.update(extra)
    m.close()
    return line


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-f64", action="store_true", help="skip the FP64 comparison leg")
    ap.add_argument("--no-tune", action="store_true")
    ap.add_argument("--ions-per-job", type=int, default=256,
                    help="ions per job (256 = the benchmark workload; smaller = a profiling case)")
    ap.add_argument("--workload", default="sweep", choices=["sweep", "tandem", "gridstudy", "legacy"],
                    help="sweep: the batched channel sweep (default); tandem: the nine-channel tandem transport; "
                         "gridstudy: one launch on grids solved at 0.100 / 0.050 / 0.0333 mm; legacy: the Fig. 4 "
                         "mass scan with every legacy switch (legacy collisions)")
    ap.add_argument("--chunk", type=int, default=0, help="steps per launch of the mixed engine (0 = its tuning)")
    ap.add_argument("--sort-cells", action="store_true", help="Morton cell order of every launch's live list")
    ap.add_argument("--no-graph", action="store_true", help="issue a multi-launch sequence without a CUDA graph")
    ap.add_argument("--blocks-per-sm", type=int, default=0, help="resident blocks per SM of the mixed engine (0 = tuning)")
    ap.add_argument("--grid", type=float, default=0.0, help="gridstudy: only the grid of this spacing [mm]")
    ap.add_argument("--replicas", type=int, default=16, help="legacy: seed sets of the 26 x 1,000-ion scan")
    ap.add_argument("--sweep-only", action="store_true",
                    help="default workload: print the sweep's line without the other workloads' results")
    ap.add_argument("--tracks", type=int, default=1 << 20, help="tandem: tracks in the pulse")
    ap.add_argument("--tandem-steps", type=int, default=1000, help="tandem: global steps per bench step")
    ap.add_argument("--port-h", type=float, default=0.05, help="tandem: port grid spacing [mm]")
    ap.add_argument("--tandem-shared", action="store_true", help="tandem: the nine ports share one device grid")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if args.impl == "gb300" else "gloo")
    if args.workload == "gridstudy":
        if args.impl == "reference":
            if rank == 0:
                print(json.dumps({"impl": "reference", "metric": GRID_METRIC,
                                  "unavailable": "the grid study's reference arm is the sweep's CPU port; run "
                                                 "--impl reference without --workload for it"}), flush=True)
        else:
            line = run_gridstudy(args, rank, world)
            if line:
                print(json.dumps(line), flush=True)
        if dist:
            dist.barrier()
            dist.destroy_process_group()
        return
    if args.workload == "legacy":
        if args.impl == "reference":
            if rank == 0:
                print(json.dumps({"impl": "reference", "metric": LEGACY_METRIC,
                                  "unavailable": "the legacy scan's reference arm is the sweep's CPU port; run "
                                                 "--impl reference without --workload for it"}), flush=True)
        else:
            line = run_legacy(args, rank, world)
            if line:
                print(json.dumps(line), flush=True)
        if dist:
            dist.barrier()
            dist.destroy_process_group()
        return
    if args.workload == "tandem":
        line = run_tandem(args, rank, world)
        if line:
            print(json.dumps(line), flush=True)
        if dist:
            dist.barrier()
            dist.destroy_process_group()
        return
    if args.impl == "reference":
        run_reference(args, rank, world)
        if dist:
            dist.barrier()
            dist.destroy_process_group()
        return

    import torch
    import __graft_entry__ as ge
    import multiq_workbench_gb300 as mq

    ge.build()
    torch.cuda.set_device(local)
    jobs, ph, dc = workload(ions_per_job=args.ions_per_job, seed0=rank_seed0(rank))
    f = fields()
    eng = mq.Engine(f, mq.PREC_MIXED, device=local)
    tuned = None
    if not args.no_tune:
        tuned, _ = eng.autotune(jobs, dc, ph, sample_per_job=64)
    apply_tuning(eng, args)
    if tuned is not None:
        tuned = eng.tuning()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")

    table = mq.JobTable.from_jobs(jobs, pinned=True)   # the batch's host-side input, packed once
    for _ in range(args.warmup):
        eng.run_batch(table, dc, ph)
    torch.cuda.synchronize()
    clocks = Clocks(local)
    clocks.start()
    dev_ms, step_ms, steps_total, launches, walls = [], [], 0, 0, []
    h2d = d2h = 0
    moved, loads, replays, step_launches = 0.0, 0, 0, 0
    wide = eng.tuning()["wide_records"]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    for _ in range(args.steps):
        flush_l2(flush)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = eng.run_batch(table, dc, ph)
        walls.append(time.perf_counter() - t0)
        s = eng.last_stats
        dev_ms.append(s.kernel_ms)
        step_ms.append(s.step_kernel_ms)
        steps_total += s.ion_steps
        launches += s.kernel_launches
        h2d, d2h = s.h2d_bytes, s.d2h_bytes
        moved += stepping_bytes(s, wide)
        loads += s.cell_loads
        replays += s.graph_replays
        step_launches += s.step_kernel_launches
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clk = clocks.stop()
    t_dev = sum(dev_ms) * 1e-3
    t_wall = sum(walls)
    (t_dev, t_wall), (steps_all,) = reduce_over_ranks([t_dev, t_wall], [steps_total], f"cuda:{local}")
    value = steps_all / t_dev
    e2e_value = steps_all / t_wall
    counts = {k: int(getattr(out, k).sum()) for k in ("transmitted", "returned", "crashed", "left", "timeout")}

    extra = {}
    if rank == 0 and not args.no_f64:
        # FP64 kernel vs mixed engine on the same 1/16 sample (16 ions of every job): speed and outcomes
        sj = [mq.Job(j.sp, j.drive, 16, j.seed) for j in jobs]
        with mq.Engine(f, mq.PREC_F64, device=local) as e64:
            o64 = e64.run_batch(sj, dc, ph)
            s64 = e64.last_stats
        om = eng.run_batch(sj, dc, ph)
        sm = eng.last_stats
        from multiq_workbench_gb300 import validate as V
        cmp = V.compare_classes(V.class_counts(om), V.class_counts(o64))
        extra["fp64_gpu"] = {"value": s64.ion_steps / (s64.kernel_ms * 1e-3), "unit": UNIT,
                             "mixed_same_sample": sm.ion_steps / (sm.kernel_ms * 1e-3),
                             "speedup_mixed_over_fp64": (sm.ion_steps / sm.kernel_ms) / (s64.ion_steps / s64.kernel_ms),
                             "fp64_note": "GB300's FP64 rate is a small fraction of its FP32 rate, which the ratio reflects",
                             "sample": f"{sum(j.n for j in sj)} ions (16 of each job)",
                             "outcomes": {"chi2": cmp["chi2"], "dof": cmp["dof"], "p": cmp["p"],
                                          "classes": {k: {"mixed": c["a"], "fp64": c["b"], "pull": c["pull"]}
                                                      for k, c in cmp["classes"].items()}}}
    cpu = None
    if rank == 0 and not args.no_cpu:
        r = cpu_rate(jobs, ph, dc, f, 128, os.cpu_count() or 1, target_s=12.0)
        cpu = {"value": r["value"], "unit": UNIT, "cores": os.cpu_count() or 1, "cpu": cpu_model(), "kind": "port",
               "sample": f"{r['ions']} ions of {r['jobs']} evenly spaced jobs run to completion ({r['seconds']:.1f} s)"}

    peaks = measured_peaks()
    hbm = peaks.get("hbm_gbs")
    peak_src = "measured" if hbm else "fallback"
    l2 = l2_read_gbs(local) if rank == 0 else None
    hbm = hbm or 6800.0
    kern_s = sum(step_ms) * 1e-3
    achieved = moved / kern_s / 1e9
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": 1e3 * t_dev / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
                "config": {"workload": f"batched sweep 64 f_ac x 8 V_ac x 32 m/z x {args.ions_per_job} ions "
                                       f"({len(jobs) * args.ions_per_job:,} ions), "
                                       "0.100 mm channel grid 160x160x242, legacy half-kick, <=20000 steps",
                           "jobs": len(jobs), "ions": sum(j.n for j in jobs), "l2_flush": "256 MB write before every timed step",
                           "tuning": {**(tuned or eng.tuning()), "use_graph": replays > 0,
                                      "graph_replays_per_step": replays / args.steps,
                                      "step_launches_per_step": step_launches / args.steps}},
                "ion_steps_per_step": steps_total / args.steps,
                "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
                "gpu_launches": int(launches),
                "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                             "traffic": None, "peak_source": f"{peak_src} hbm_gbs",
                             "kernel": "k_mixed",
                             "algorithmic_bytes": f"cell fills counted by the kernel x 8 node records ({64 if wide else 48} B) "
                                                  f"+ {ION_STATE_BYTES} B per ion taken from the queue",
                             "algorithmic_bytes_per_ion_step": moved / max(steps_total, 1),
                             "cell_loads_per_ion_step": loads / max(steps_total, 1)},
                "roofline_l2": {"achieved": achieved, "peak": l2, "unit": "GB/s",
                                "frac": achieved / l2 if l2 else None,
                                "peak_source": "L2 read bandwidth measured in this run (mq_measure_l2_read_gbs: "
                                               "32 MiB resident, 200 sweeps, best of 3)"},
                "cpu_baseline": cpu, "clocks": clk, "outcomes": counts}
        line.update(extra)
    eng.close()
    if rank == 0 and world == 1 and not args.sweep_only:
        line["workloads"] = other_workloads(args)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


def other_workloads(args) -> dict:
    """The other measured workloads, run after the headline sweep in the default invocation so that
    every configuration has a measured line: the grid study (config 3), the tandem (config 4) and the
    legacy Fig. 4 scan (legacy collisions), each with 2 timed steps after 3 warm-up steps.  A
    workload that fails is recorded with its error instead of a line."""
    import copy
    import gc
    out = {}
    for name, fn in (("gridstudy", run_gridstudy), ("tandem", run_tandem), ("legacy", run_legacy)):
        a = copy.copy(args)
        a.steps, a.warmup, a.workload = 2, 3, name
        a.ions_per_job = 256
        try:
            out[name] = fn(a, 0, 1)
        except Exception as e:   # keep the headline line whatever happens here
            out[name] = {"error": f"{type(e).__name__}: {e}"}
        gc.collect()
    return out


if __name__ == "__main__":
    main()
