"""Excitation-frequency sweeps of a species mixture and their resonance fits: counts per frequency
point and species, a Lorentzian / Gaussian fit per species, R = f0 / FWHM and R in m/z terms
(simulation/mqviz/src/engine.rs:420-431,751-808 ``start_sweep`` / ``sweep_cli``,
analysis.rs:20-58 ``fit_sweep``, presets.rs).

The reference sweeps with tagged cohorts inside its live single-stream engine: ions are injected
one at a time, ``ions_per_point`` of them carry the tag of the current frequency point, and the
tone steps to the next point after each cohort.  Each tagged ion's single-pass outcome depends only
on its own species and tone, so here every (point, species) cohort is one job of ONE batch on the
device engine: all points run concurrently instead of one after another.  A cohort's species mix
is the mixture's weights apportioned exactly (largest remainder) rather than drawn ion by ion.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from .channel import Job, Physics, RfAc, Species, LAUNCH_DISC
from . import fit as F

DC_CAL = (18.0, 24.0, 15.0, 20.0)   # world.rs:33, [Q1, gate, down, box] V
FIG5C_HEIGHT = ((6, 15.9), (7, 60.3), (8, 100.0), (9, 15.2), (10, 4.8))


def ubq_ccs(z: int) -> float:
    return {6: 1250.0, 7: 1262.0, 8: 1800.0, 9: 2090.0}.get(int(z), 2200.0)


def ccs_guess(m: float) -> float:
    """Compact-ion N2 CCS, 2.95 M^(2/3) [A^2] (presets.rs:33-34)."""
    return 2.95 * m ** (2.0 / 3.0)


@dataclass
class SweepSpecies:
    """One species of a mixture (mqviz ``Sp``): label, mass [Da], charge, N2 CCS [A^2], abundance."""
    label: str
    mass: float
    z: float
    ccs: float
    weight: float = 1.0

    def mz(self) -> float:
        return self.mass / self.z

    def species(self) -> Species:
        return Species(self.mass, self.z, self.ccs)

    @classmethod
    def ubq(cls, z: int, weight: float) -> "SweepSpecies":   # presets.rs:29-31
        return cls(f"{z}+", 8564.8 + z * 1.00728, float(z), ubq_ccs(z), weight)

    @classmethod
    def custom(cls, mz: float, z: float, ccs: float = 0.0) -> "SweepSpecies":   # presets.rs:36-39
        mass = mz * z
        return cls(f"{int(z)}+ m/z {mz:.1f}", mass, z, ccs if ccs > 0.0 else ccs_guess(mass), 1.0)


@dataclass
class SweepPreset:
    """Instrument settings and mixture of a preset (presets.rs:41-61)."""
    name: str
    species: list
    v_rf: float
    v_ac: float
    f_ac_khz: float
    gate_v: float
    pressure_pa: float
    sweep: tuple   # (lo, hi, step) kHz

    @classmethod
    def s14(cls) -> "SweepPreset":
        return cls("S14 · Bak BH3 2+", [SweepSpecies("2+ 863.5", 2.0 * 863.473, 2.0, 425.0, 0.95),
                                        SweepSpecies("2+ Na 874.5", 2.0 * 874.466, 2.0, 430.0, 0.05)],
                   70.0, 0.35, 84.25, 24.0, 0.1, (70.0, 100.0, 1.0))

    @classmethod
    def fig5(cls) -> "SweepPreset":
        return cls("Fig. 5 · ubiquitin 6+…10+", [SweepSpecies.ubq(z, h) for z, h in FIG5C_HEIGHT],
                   56.0, 0.20, 59.25, 24.0, 0.1, (35.0, 65.0, 1.0))

    @classmethod
    def custom(cls, mz: float = 863.5, z: float = 2.0, ccs: float = 0.0) -> "SweepPreset":
        return cls("Custom m/z", [SweepSpecies.custom(mz, z, ccs)], 70.0, 0.35, 84.0, 24.0, 0.1, (70.0, 100.0, 1.0))

    def dc(self) -> list:
        d = list(DC_CAL)
        d[1] = self.gate_v
        return d


@dataclass
class SweepCfg:
    """Frequency grid and statistics of a sweep (engine.rs ``SweepCfg``)."""
    f_lo_khz: float
    f_hi_khz: float
    step_khz: float
    ions_per_point: int = 2000
    sweeps: int = 1

    def freqs(self) -> list:
        """lo + i step for i = 0..=round((hi - lo) / step), at most 101 points (engine.rs:421-423)."""
        n = int(math.floor(abs((self.f_hi_khz - self.f_lo_khz) / self.step_khz) + 0.5))
        if (self.f_hi_khz - self.f_lo_khz) / self.step_khz < 0:
            n = 0
        return [self.f_lo_khz + i * self.step_khz for i in range(min(n, 100) + 1)]


def sweep_physics(pressure_pa: float) -> Physics:
    """Single-pass physics of the mqviz world (world.rs:18-27): dt = T_RF / 50, t_max 3 ms, disc
    launch r <= 2 mm at z = 1 mm, exit at 18.6 mm, return below 0.5 mm, RF phase at birth random."""
    return Physics(pressure_pa=pressure_pa, dt=4e-8, t_max=3e-3, launch=LAUNCH_DISC, r_inject_mm=2.0, rf_phase0=False)


def apportion(total: int, weights) -> list:
    """Integer split of ``total`` proportional to ``weights`` (largest remainder, ties to the first)."""
    w = np.asarray(weights, dtype=np.float64)
    if total <= 0 or len(w) == 0 or not np.all(w >= 0) or w.sum() <= 0:
        return [0] * len(w)
    q = total * w / w.sum()
    base = np.floor(q).astype(np.int64)
    rem = q - base
    order = sorted(range(len(w)), key=lambda i: (-rem[i], i))
    for i in order[: total - int(base.sum())]:
        base[i] += 1
    return [int(x) for x in base]


@dataclass
class SweepView:
    """Outcome counts per point and species: counts[point, species] = (T, C, R, timeout), C counting
    crashes on electrodes and leaving the box alike (world.rs:309-314)."""
    f: list
    counts: np.ndarray
    labels: list = field(default_factory=list)

    def frac(self, point: int, s: int) -> tuple:
        """(k transmitted, n) of one cohort (engine.rs:434-438)."""
        c = self.counts[point, s]
        return int(c[0]), int(c.sum())

    def ks_ns(self, s: int):
        return [int(self.counts[i, s, 0]) for i in range(len(self.f))], [int(self.counts[i, s].sum()) for i in range(len(self.f))]


def sweep_jobs(species, cfg: SweepCfg, v_rf: float, v_ac: float, seed: int, f_rf: float = 500e3) -> list:
    """One job per (point, species): n from the weights, seed = seed + point * nspecies + species."""
    ns = apportion(int(cfg.ions_per_point) * int(cfg.sweeps), [s.weight for s in species])
    jobs = []
    for i, f in enumerate(cfg.freqs()):
        for s, sp in enumerate(species):
            jobs.append(Job(sp.species(), RfAc(v_rf, f_rf, v_ac, f * 1e3), ns[s], int(seed) + i * len(species) + s))
    return jobs


def run_sweep(engine, species, cfg: SweepCfg, v_rf: float, v_ac: float, dc, ph: Physics, seed: int = 0) -> SweepView:
    """All cohorts of the sweep as one ``run_batch`` (jobs with n = 0 are not sent)."""
    fs = cfg.freqs()
    jobs = sweep_jobs(species, cfg, v_rf, v_ac, seed)
    live = [k for k, j in enumerate(jobs) if j.n > 0]
    counts = np.zeros((len(fs), len(species), 4), np.int64)
    if live:
        out = engine.run_batch([jobs[k] for k in live], dc, ph)
        for k, o in zip(live, out):
            i, s = divmod(k, len(species))
            counts[i, s] = (o.transmitted, o.crashed + o.left, o.returned, o.timeout)
    return SweepView(fs, counts, [s.label for s in species])


@dataclass
class SweepFit:
    """A species' fitted resonance (analysis.rs:20-35): values as (value, error)."""
    label: str
    mz: float
    fit: F.ResFit
    dfdmz: float
    fwhm: tuple
    fwhm_mz: tuple
    r_f: tuple
    r_mz: tuple
    peak: tuple
    min_ions: int


def fit_sweep(sv: SweepView, species, tables: F.TerrainTables | None, v_rf: float, dc, boot: int = 200,
              seed: int = 0, dfdmz=None) -> list:
    """Fit every species' single-pass transmission curve (analysis.rs:37-58): species with no
    transmitted ion or a maximum below 0.5 % are skipped, fits that are not significant too.  The
    slope d f / d(m/z) comes from the terrain tables, or from ``dfdmz[s]`` when given."""
    out = []
    for s, sp in enumerate(species):
        ks, ns = sv.ks_ns(s)
        if max(ks, default=0) == 0:
            out.append(None)
            continue
        ymax = max([k / n for k, n in zip(ks, ns) if n > 0], default=0.0)
        if ymax < 0.005:
            out.append(None)
            continue
        f = F.fit_binomial_curve(sv.f, ks, ns, boot, int(seed) ^ s)
        if f is None or not F.is_significant(f, sv.f):
            out.append(None)
            continue
        slope = float(dfdmz[s]) if dfdmz is not None else tables.dfdmz(sp, v_rf, dc)
        _, _, rmz, rmz_e = F.r_mz(sp.mz(), slope, f.p[3], f.e[3])
        den = max(abs(slope), 1e-12)
        peak_e = math.sqrt(max(f.e[0] ** 2 + f.e[1] ** 2 + 2.0 * f.cov[0][1], 0.0))
        out.append(SweepFit(sp.label, sp.mz(), f, slope, (f.p[3], f.e[3]), (f.p[3] / den, f.e[3] / den), (f.r, f.r_err),
                            (rmz, rmz_e), (f.peak(), peak_e), min([n for n in ns if n > 0], default=0)))
    return out


def sweep_csv(sv: SweepView) -> str:
    """Per-point table: f_khz, then T, C, R, timeout and n for each species."""
    head = ["f_khz"] + [f"{lab}:{k}" for lab in sv.labels for k in ("T", "C", "R", "timeout", "n")]
    lines = [",".join(head)]
    for i, f in enumerate(sv.f):
        row = [f"{f:g}"]
        for s in range(len(sv.labels)):
            c = sv.counts[i, s]
            row += [str(int(x)) for x in c] + [str(int(c.sum()))]
        lines.append(",".join(row))
    return "\n".join(lines) + "\n"
