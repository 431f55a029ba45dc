"""Validation at the S14 calibrated point (simulation/mqviz/src/validate.rs:1-184): the device engines
against each other and against chsim's own GPU counts, which the reference embeds
(``REF_CHSIM_GPU``), with its binomial pulls and its acceptance mark (|pull| <= 2 "ok").

``python -m multiq_workbench_gb300.validate [--n N] [--device D]`` solves the calibrated channel
on the GPU, runs the FP64 and the mixed engine at the point with a random RF phase at injection
and with phase 0 (chsim's convention), and prints the reference's tables.
"""
from __future__ import annotations

import argparse
import math
import time
from dataclasses import dataclass

from .channel import Engine, Job, Physics, RfAc, Species, PREC_F64, PREC_MIXED
from .grid import Fields, Geom

# validate.rs:8-11, world.rs:25,33
CAL_VRF, CAL_VAC, CAL_FAC_KHZ, CAL_P = 70.0, 0.35, 84.25, 0.1
T_MAX = 3.0e-3
DC_CAL = (18.0, 24.0, 15.0, 20.0)
BAK_2PLUS = Species(2.0 * 863.473, 2.0, 425.0)   # presets.rs:46
# chsim's GPU engine at the point, n = 100,000, seed 4242: (n, transmitted, crashed + left, returned,
# timeout) (validate.rs:110-112)
REF_CHSIM_GPU = (100_000, 19_669, 3_412, 75_797, 1_122)


@dataclass
class Counts:
    """Outcome counts of one run (validate.rs:13-21)."""
    n: int
    trans: int
    crash: int
    ret: int
    timeout: int
    steps: int = 0

    def frac(self, k: int) -> float:
        return k / max(self.n, 1)

    def se(self, k: int) -> float:
        """Binomial standard error of a count out of n."""
        p = self.frac(k)
        return math.sqrt(p * (1.0 - p) / max(self.n, 1))

    def t_over_tc(self) -> float:
        return self.trans / max(self.trans + self.crash, 1)

    def se_eff(self) -> float:
        """Standard error of T / (T + C) (binomial on the T + C subset)."""
        m = max(self.trans + self.crash, 1)
        p = self.t_over_tc()
        return math.sqrt(p * (1.0 - p) / m)

    @classmethod
    def from_outcomes(cls, outs, steps: int = 0) -> "Counts":
        return cls(int(sum(o.n for o in outs)), int(sum(o.transmitted for o in outs)),
                   int(sum(o.crashed + o.left for o in outs)), int(sum(o.returned for o in outs)),
                   int(sum(o.timeout for o in outs)), int(steps))


def embedded_metal() -> Counts:
    n, t, c, r, to = REF_CHSIM_GPU
    return Counts(n, t, c, r, to)


@dataclass
class Row:
    name: str
    live: float
    live_se: float
    refv: float
    ref_se: float

    def pull(self) -> float:
        return (self.live - self.refv) / max(math.sqrt(self.live_se ** 2 + self.ref_se ** 2), 1e-12)


def rows(live: Counts, r: Counts) -> list:
    """The four compared quantities (validate.rs:119-126)."""
    return [Row("transmitted", live.frac(live.trans), live.se(live.trans), r.frac(r.trans), r.se(r.trans)),
            Row("crashed", live.frac(live.crash), live.se(live.crash), r.frac(r.crash), r.se(r.crash)),
            Row("returned", live.frac(live.ret), live.se(live.ret), r.frac(r.ret), r.se(r.ret)),
            Row("T/(T+C)", live.t_over_tc(), live.se_eff(), r.t_over_tc(), r.se_eff())]


def table(title: str, a_name: str, b_name: str, a: Counts, b: Counts) -> str:
    """The reference's comparison table (validate.rs:128-135) as text."""
    out = [f"  {title}", f"    {'outcome':<12} {a_name:>18} {b_name:>18} {'pull':>8}"]
    for row in rows(a, b):
        ok = "ok" if abs(row.pull()) <= 2.0 else "DIFF"
        out.append(f"    {row.name:<12} {row.live:>9.4f} ± {row.live_se:.4f} {row.refv:>9.4f} ± {row.ref_se:.4f} "
                   f"{row.pull():>7.2f}σ {ok}")
    return "\n".join(out)


def _gamma_q(a: float, x: float) -> float:
    """Regularised upper incomplete gamma Q(a, x): the power series of P below x = a + 1 and the
    Lentz continued fraction of Q above (Press et al., Numerical Recipes, 3rd ed., section 6.2)."""
    if x <= 0.0:
        return 1.0
    lg = math.lgamma(a)
    if x < a + 1.0:
        term = total = 1.0 / a
        ap = a
        for _ in range(10_000):
            ap += 1.0
            term *= x / ap
            total += term
            if abs(term) < abs(total) * 1e-15:
                break
        return max(0.0, 1.0 - total * math.exp(-x + a * math.log(x) - lg))
    tiny = 1e-300
    b = x + 1.0 - a
    c = 1.0 / tiny
    d = 1.0 / b
    h = d
    for i in range(1, 10_000):
        an = -i * (i - a)
        b += 2.0
        d = an * d + b
        d = tiny if abs(d) < tiny else d
        c = b + an / c
        c = tiny if abs(c) < tiny else c
        d = 1.0 / d
        delta = d * c
        h *= delta
        if abs(delta - 1.0) < 1e-15:
            break
    return math.exp(-x + a * math.log(x) - lg) * h


def chi2_sf(x: float, dof: int) -> float:
    """P(X >= x) for X chi-square distributed with ``dof`` degrees of freedom (1 when dof = 0)."""
    return 1.0 if dof <= 0 else _gamma_q(0.5 * dof, 0.5 * x)


def compare_classes(a: dict, b: dict) -> dict:
    """Outcome-class counts of two engines run on the same ions with independent random streams
    (``a`` and ``b``: class name -> count, each summing to the same n): the chi-square test of
    homogeneity of the 2 x K table of classes with a non-zero total (K - 1 degrees of freedom),
    its p-value, and per class the pooled binomial pull of the two fractions, (a / na - b / nb) /
    sqrt(p (1 - p) (1 / na + 1 / nb)) with p the pooled fraction."""
    keys = [k for k in a if a[k] + b[k] > 0]
    na, nb = sum(a.values()), sum(b.values())
    tot = na + nb
    stat = 0.0
    pulls = {}
    for k in keys:
        col = a[k] + b[k]
        for obs, rowsum in ((a[k], na), (b[k], nb)):
            e = rowsum * col / tot
            stat += (obs - e) ** 2 / e
        p = col / tot
        se = math.sqrt(p * (1 - p) * (1.0 / na + 1.0 / nb)) if 0 < p < 1 else 0.0
        pulls[k] = {"a": int(a[k]), "b": int(b[k]), "pull": (a[k] / na - b[k] / nb) / se if se > 0 else 0.0}
    dof = max(len(keys) - 1, 0)
    return {"chi2": stat, "dof": dof, "p": chi2_sf(stat, dof), "n": [int(na), int(nb)], "classes": pulls}


def compare_jobs(a_jobs: list, b_jobs: list) -> dict:
    """Per-job homogeneity over many jobs: the sum of each job's 2 x K chi-square and of its degrees
    of freedom (the jobs are independent), with the p-value of the sum."""
    stat, dof = 0.0, 0
    for a, b in zip(a_jobs, b_jobs):
        r = compare_classes(a, b)
        stat += r["chi2"]
        dof += r["dof"]
    return {"chi2": stat, "dof": dof, "p": chi2_sf(stat, dof), "jobs": len(a_jobs)}


def compare_paired(a_status, b_status) -> dict:
    """Per-ion final classes of two engines run from the same launch draws (``a_status``,
    ``b_status``: status arrays of equal length): the fraction of ions in the same class and
    Bowker's test of symmetry of the class-transition table, sum over class pairs i < j of
    (n_ij - n_ji)^2 / (n_ij + n_ji), one degree of freedom per pair seen.  With independent random
    streams and no bias between the engines, an ion moves from class i to j as often as from j to i."""
    import numpy as np
    a = np.asarray(a_status).astype(np.int64)
    b = np.asarray(b_status).astype(np.int64)
    k = int(max(a.max(initial=0), b.max(initial=0))) + 1
    t = np.zeros((k, k), np.int64)
    np.add.at(t, (a, b), 1)
    stat, dof = 0.0, 0
    for i in range(k):
        for j in range(i + 1, k):
            m = t[i, j] + t[j, i]
            if m:
                stat += (t[i, j] - t[j, i]) ** 2 / m
                dof += 1
    return {"agree": float((a == b).mean()) if len(a) else 1.0, "bowker": stat, "dof": dof, "p": chi2_sf(stat, dof),
            "table": t.tolist()}


CLASSES = ("crashed", "returned", "transmitted", "left", "timeout")


def class_counts(outs, jobs=None) -> dict:
    """Outcome-class totals of a batch's ``Outcomes`` (all jobs, or the job indices in ``jobs``)."""
    idx = range(len(outs)) if jobs is None else jobs
    return {k: int(sum(getattr(outs[j], k) for j in idx)) for k in CLASSES}


def s14_fields(device: int | None = 0) -> Fields:
    """The calibrated S14 channel ("code" variant, hole 7.0 mm; validate.rs:98)."""
    return Fields.build(Geom.s14("code", hole_d=7.0), device=device)


def point_physics(rf_phase0: bool = True) -> Physics:
    ph = Physics.correct(CAL_P)
    ph.t_max = T_MAX
    ph.rf_phase0 = bool(rf_phase0)
    return ph


def run_engine(engine: Engine, n: int, seed: int, rf_phase0: bool = True) -> Counts:
    """n ions of the Bak BH3 2+ species at the calibrated point through ``run_batch``
    (``run_chsim_gpu``, validate.rs:96-108)."""
    job = Job(BAK_2PLUS, RfAc(CAL_VRF, 500e3, CAL_VAC, CAL_FAC_KHZ * 1e3), int(n), int(seed))
    out = engine.run_batch([job], list(DC_CAL), point_physics(rf_phase0))
    return Counts.from_outcomes(out, engine.last_stats.ion_steps)


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--n", type=int, default=100_000)
    ap.add_argument("--device", type=int, default=0)
    a = ap.parse_args(argv)
    t0 = time.time()
    f = s14_fields(a.device)
    print(f"fields ready in {time.time() - t0:.1f} s")
    print(f"S14 calibrated point: Bak BH3 2+ (m/z {BAK_2PLUS.mass / BAK_2PLUS.z:.1f}, CCS {BAK_2PLUS.ccs_n2} A^2), "
          f"RF {CAL_VRF} V @ 500 kHz, AC ±{CAL_VAC} V @ {CAL_FAC_KHZ} kHz, DC {list(DC_CAL)}, {CAL_P} Pa")
    res = {}
    for name, prec in (("FP64", PREC_F64), ("mixed", PREC_MIXED)):
        with Engine(f, prec, device=a.device) as e:
            t = time.time()
            res[name] = run_engine(e, a.n, 4242, True)
            dt = time.time() - t
            res[name + " random RF"] = run_engine(e, a.n, 12345, False)
        print(f"  {name} engine, n = {a.n}: {dt:.2f} s, {res[name].steps / dt / 1e9:.2f} G ion-steps/s")
    metal = embedded_metal()
    print(table(f"FP64 vs mixed engine, RF phase 0, n = {a.n}", "FP64", "mixed", res["FP64"], res["mixed"]))
    print(table(f"FP64 engine vs chsim GPU (embedded, n = {metal.n})", "FP64 (RF0)", "chsim GPU", res["FP64"], metal))
    print(table(f"mixed engine vs chsim GPU (embedded, n = {metal.n})", "mixed (RF0)", "chsim GPU", res["mixed"], metal))
    print(table("random RF phase vs phase 0 (the RF-phase convention), mixed engine", "random", "RF0",
                res["mixed random RF"], res["mixed"]))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
