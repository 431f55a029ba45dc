"""Scan drivers over ``Engine.run_batch``: the persistent result cache and the adaptive two-stage
frequency scan of chsim (simulation/chsim/src/scan.rs:1-78).

The cache is the reference's own format, so either project reads the other's file: one line per
job, ``<key>\\t<n>,<crashed>,<returned>,<transmitted>,<left>,<timeout>,<mean_coll>,<mean_time>``,
where the key is ``format!("{:?}|{:?}|{:?}|{}|{}|{:?}|{:?}", geom, species, drive, n, seed, dc,
physics)`` of the reference structs (scan.rs:9-11) and the values are Rust ``Display`` output.
Physics options the reference does not have (the Gaussian launch, a random RF phase) are appended
to the key, so such entries never collide with the reference's.
"""
from __future__ import annotations

import math
import sys
from pathlib import Path

import numpy as np

from .channel import Job, Outcome, Physics, RfAc, Species
from .grid import Geom, _rust_f64, cache_dir

LAUNCH_DISC, LAUNCH_LEGACY = 0, 1


def _b(x) -> str:
    return "true" if x else "false"


def rust_display_f64(x: float) -> str:
    """Rust ``{}`` of an f64: shortest round-trip digits, never an exponent, no trailing ``.0``."""
    x = float(x)
    if x != x:
        return "NaN"
    if math.isinf(x):
        return "inf" if x > 0 else "-inf"
    return np.format_float_positional(x, unique=True, trim="-")


def species_debug(sp: Species) -> str:
    return f"Species {{ mass: {_rust_f64(sp.mass)}, z: {_rust_f64(sp.z)}, ccs_n2: {_rust_f64(sp.ccs_n2)} }}"


def rfac_debug(d: RfAc) -> str:
    return (f"RfAc {{ v_rf: {_rust_f64(d.v_rf)}, f_rf: {_rust_f64(d.f_rf)}, v_ac: {_rust_f64(d.v_ac)}, "
            f"f_ac: {_rust_f64(d.f_ac)} }}")


def physics_debug(ph: Physics) -> str:
    """``{:?}`` of chsim's ``Physics`` (channel.rs:254-259); options beyond it are appended."""
    s = (f"Physics {{ legacy_force: {_b(ph.legacy_force)}, legacy_collisions: {_b(ph.legacy_collisions)}, "
         f"legacy_fields: {_b(ph.legacy_fields)}, legacy_injection: {_b(ph.legacy_injection)}, "
         f"legacy_criteria: {_b(ph.legacy_criteria)}, pressure_pa: {_rust_f64(ph.pressure_pa)}, "
         f"temp_k: {_rust_f64(ph.temp_k)}, dt: {_rust_f64(ph.dt)}, t_max: {_rust_f64(ph.t_max)}, "
         f"r_inject_mm: {_rust_f64(ph.r_inject_mm)} }}")
    # the engine launches legacy-style when either switch asks for it; the reference has only the switch
    launch = LAUNCH_LEGACY if (ph.legacy_injection or int(ph.launch) == LAUNCH_LEGACY) else int(ph.launch)
    native = LAUNCH_LEGACY if ph.legacy_injection else LAUNCH_DISC
    extra = []
    if launch != native:
        extra.append(f"launch: {launch}, sigma_mm: {_rust_f64(ph.sigma_mm)}")
    if not ph.rf_phase0:
        extra.append("rf_phase0: false")
    if _rust_f64(ph.z_inject_mm) != "1.0":
        extra.append(f"z_inject_mm: {_rust_f64(ph.z_inject_mm)}")
    return s + (" + {" + ", ".join(extra) + "}" if extra else "")


def result_key(geom: Geom, job: Job, dc, ph: Physics) -> str:
    """The cache key of scan.rs:9-11."""
    dcs = "[" + ", ".join(_rust_f64(float(v)) for v in dc) + "]"
    return (f"{geom.rust_debug()}|{species_debug(job.sp)}|{rfac_debug(job.drive)}|{int(job.n)}|{int(job.seed)}|"
            f"{dcs}|{physics_debug(ph)}")


def results_path() -> Path:
    """``<cache dir>/results.tsv`` (the reference keeps ``cache/results.tsv``)."""
    return cache_dir() / "results.tsv"


def outcome_line(key: str, o: Outcome) -> str:
    return (f"{key}\t{o.n},{o.crashed},{o.returned},{o.transmitted},{o.left},{o.timeout},"
            f"{rust_display_f64(o.mean_coll)},{rust_display_f64(o.mean_time)}\n")


def load_results(path: Path | None = None) -> dict:
    """The cache as {key: Outcome}; lines that do not parse as 8 numbers are skipped (scan.rs:13-28)."""
    path = Path(path) if path is not None else results_path()
    out = {}
    try:
        text = path.read_text()
    except OSError:
        return out
    for line in text.splitlines():
        parts = line.split("\t")
        if len(parts) < 2:
            continue
        vals = []
        for x in parts[1].split(","):
            try:
                vals.append(float(x))
            except ValueError:
                pass
        if len(vals) == 8:
            out[parts[0]] = Outcome(int(vals[0]), int(vals[1]), int(vals[2]), int(vals[3]), int(vals[4]), int(vals[5]),
                                    vals[6], vals[7])
    return out


def cached_batch(engine, geom: Geom, jobs, dc, ph: Physics, path: Path | None = None, log: bool = True) -> list:
    """``run_batch`` that never reruns a job already in the cache (scan.rs:30-48): the misses run as
    one batch and are appended to the file."""
    path = Path(path) if path is not None else results_path()
    cache = load_results(path)
    keys = [result_key(geom, j, dc, ph) for j in jobs]
    miss = [i for i, k in enumerate(keys) if k not in cache]
    if miss:
        out = engine.run_batch([jobs[i] for i in miss], dc, ph)
        path.parent.mkdir(parents=True, exist_ok=True)
        with open(path, "a") as fh:
            for i, o in zip(miss, out):
                fh.write(outcome_line(keys[i], o))
                cache[keys[i]] = o
    if log:
        print(f"  [cache: {len(jobs) - len(miss)} hits, {len(miss)} computed]", file=sys.stderr)
    return [cache[k] for k in keys]


def _round4(g: float) -> float:   # (g * 1e4).round() / 1e4, Rust round = half away from zero
    x = g * 1e4
    r = math.floor(abs(x) + 0.5)
    return math.copysign(r, x) / 1e4


def adaptive_scan(engine, geom: Geom, sp: Species, rf: RfAc, dc, ph: Physics, f_lo: float, f_hi: float, f_step: float,
                  n_lo: int, n_hi: int, base: float, seed0: int, path: Path | None = None, log: bool = True) -> list:
    """Two-stage excitation-frequency scan (scan.rs:50-78): ``n_lo`` ions per point at ``f_step``
    [kHz], then ``n_hi`` ions at ``f_step / 4`` around the points whose transmission is within 35% of
    the maximum and more than 4 sigma above ``base``.  Returns (f_kHz, transmitted fraction, crashed
    fraction, n) sorted by frequency."""
    fs = []
    i = 0
    while True:
        f = f_lo + f_step * i
        if f > f_hi + 1e-9:
            break
        fs.append(f)
        i += 1
    j1 = [Job(sp, RfAc(rf.v_rf, rf.f_rf, rf.v_ac, f * 1e3), n_lo, seed0 + k) for k, f in enumerate(fs)]
    o1 = cached_batch(engine, geom, j1, dc, ph, path, log)
    t1 = [o.transmitted / o.n if o.n else 0.0 for o in o1]
    tmax = max([0.0] + t1)
    fine = []
    for k, f in enumerate(fs):
        sig = math.sqrt(max(t1[k], 1.0 / n_lo) / n_lo)
        if t1[k] >= 0.35 * tmax and t1[k] - base > 4.0 * sig:
            g = f - f_step
            while g <= f + f_step + 1e-9:
                fine.append(_round4(g))
                g += f_step / 4.0
    fine = sorted(fine)
    fine = [g for k, g in enumerate(fine) if k == 0 or g != fine[k - 1]]
    j2 = [Job(sp, RfAc(rf.v_rf, rf.f_rf, rf.v_ac, g * 1e3), n_hi, seed0 + 100_000 + k) for k, g in enumerate(fine)]
    o2 = cached_batch(engine, geom, j2, dc, ph, path, log) if j2 else []
    pts = [(f, o.transmitted / o.n, o.crashed / o.n, n_lo) for f, o in zip(fs, o1)
           if not any(abs(g - f) < 1e-6 for g in fine)]
    pts += [(g, o.transmitted / o.n, o.crashed / o.n, n_hi) for g, o in zip(fine, o2)]
    pts.sort(key=lambda p: p[0])
    if log:
        cost_full = len(fs) * 4.0 * n_hi
        cost = len(fs) * n_lo + len(fine) * n_hi
        print(f"  [adaptive scan: {len(fs)} coarse x {n_lo} + {len(fine)} fine x {n_hi} ions = "
              f"{100.0 * cost / cost_full:.0f}% of a uniform fine scan]", file=sys.stderr)
    return pts
