"""Regenerate the golden fixtures in this directory.

  pins.json          the reference's published results for this path, read from the reference
                     checkout (docs/mass-scan.csv, docs/grid-counts.csv, the embedded chsim GPU
                     counts in simulation/mqviz/src/validate.rs), next to the CPU oracle's
                     results for the same settings on grids solved by this project.
  oracle_coarse.npz  per-ion final states of the oracle on the 0.4 mm grid for three physics
                     variants (seeded), used to check that the oracle and the FP64 kernel
                     reproduce them bit for bit on any host.

Run from the repository root:  python tests/golden/make_golden.py [--reference PATH]
(the reference checkout is only needed for pins.json; it is read as data).
"""
from __future__ import annotations

import argparse
import csv
import json
import re
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

import multiq_workbench_gb300 as mq  # noqa: E402
from oracle import mqref as R  # noqa: E402


def oracle_counts(f, jobs, ph, dc):
    g = f.geom
    G = R.Grid3(f.nx, f.ny, f.nz, f.h, f.rf, f.ac, f.dc_field(dc))
    b = R.batch(ph, jobs[0].drive.v_rf, jobs[0].drive.f_rf, g.axis(), g.layers())
    s = R.inject(b, jobs, sum(j.n for j in jobs))
    steps = R.run(G, b, jobs, s)
    return R.summarize(s, b, len(jobs)), steps


def read_reference(ref: Path) -> dict:
    out = {}
    with open(ref / "docs" / "mass-scan.csv") as fh:
        rows = list(csv.DictReader(fh))
    out["mass_scan"] = {"source": "docs/mass-scan.csv",
                        "mz": [int(r["mz"]) for r in rows], "ions_per_mass": int(rows[0]["ions_per_mass"]),
                        "rust_legacy": [int(r["rust_legacy"]) for r in rows],
                        "java_original": [int(r["java_original"]) for r in rows],
                        "rust_full_kick": [int(r["rust_full_kick"]) for r in rows]}
    with open(ref / "docs" / "grid-counts.csv") as fh:
        rows = list(csv.DictReader(fh))
    g01 = [r for r in rows if r["grid"].startswith("fresh") and abs(float(r["spacing_mm"]) - 0.1) < 1e-9][0]
    out["grid_study_0p1"] = {"source": "docs/grid-counts.csv (fresh1, 0.1 mm)", "n": 1000,
                             "returned": int(g01["return"]), "electrode": int(g01["electrode"]), "box": int(g01["box"]),
                             "transmit": int(g01["transmit"]), "timeout": int(g01["timeout"])}
    src = (ref / "simulation" / "mqviz" / "src" / "validate.rs").read_text()
    m = re.search(r"REF_CHSIM_GPU[^=]*=\s*Some\(\(([^)]*)\)\)", src)
    vals = [int(x.strip().replace("_", "")) for x in m.group(1).split(",")]
    out["s14_chsim_gpu"] = {"source": "simulation/mqviz/src/validate.rs REF_CHSIM_GPU", "n": vals[0], "transmitted": vals[1],
                            "crashed_or_left": vals[2], "returned": vals[3], "timeout": vals[4]}
    return out


def pins(ref: Path) -> dict:
    res = read_reference(ref)
    t0 = time.time()
    g = mq.Geom()
    f = mq.Fields.build(g, bases=[0, 1, 3, 4])
    drive = mq.RfAc(100.0, 500e3, 0.5, 100e3)
    dc = [0.0, 5.0, -5.0, 0.0]
    mzs = res["mass_scan"]["mz"]
    n = res["mass_scan"]["ions_per_mass"]
    # legacy Fig. 4 scan (chsim legacy-fig4: 5+ ions of mass 5 m/z, Physics::legacy, seed 1000 + m/z)
    jobs = [mq.Job(mq.Species(mz * 5.0, 5.0, 0.0), drive, n, 1000 + mz) for mz in mzs]
    leg, _ = oracle_counts(f, jobs, mq.Physics.legacy(1e-3 * 133.322), dc)
    ph_fk = mq.Physics.legacy(1e-3 * 133.322)
    ph_fk.legacy_force = False
    fk, _ = oracle_counts(f, jobs, ph_fk, dc)
    res["mass_scan"]["oracle_legacy"] = [o["transmitted"] for o in leg]
    res["mass_scan"]["oracle_full_kick"] = [o["transmitted"] for o in fk]
    # grid study: corrected physics, legacy point + cone launch, 5+ ions m/z 499, dt 100 ns
    ph_gs = mq.Physics(pressure_pa=1e-3 * 133.322, dt=1e-7, t_max=0.02, legacy_injection=True, launch=mq.LAUNCH_LEGACY)
    gs, _ = oracle_counts(f, [mq.Job(mq.Species(2495.0, 5.0, 2.95 * 2495.0 ** (2 / 3)), drive, 1000, 1499)], ph_gs, dc)
    res["grid_study_0p1"]["oracle"] = {k: gs[0][k] for k in ("returned", "crashed", "left", "transmitted", "timeout")}
    res["grid_study_0p1"]["oracle_settings"] = ("Physics::correct switches, dt 1e-7 s, legacy point+cone launch, "
                                                "mass 2495 Da z 5, N2 CCS 2.95 m^(2/3), DC [0,5,-5,0], seed 1499")
    # S14 calibrated point (validate.rs:97-112): chsim Physics::correct(0.1), t_max 3 ms, seed 4242
    gs14 = mq.Geom.s14("code", hole_d=7.0)
    f14 = mq.Fields.build(gs14)
    ph14 = mq.Physics.correct(0.1)
    ph14.t_max = 3e-3
    n14 = res["s14_chsim_gpu"]["n"]
    o14, _ = oracle_counts(f14, [mq.Job(mq.Species(2 * 863.473, 2.0, 425.0), mq.RfAc(70.0, 500e3, 0.35, 84.25e3), n14, 4242)],
                           ph14, [18.0, 24.0, 15.0, 20.0])
    o = o14[0]
    res["s14_chsim_gpu"]["oracle"] = {"n": o["n"], "transmitted": o["transmitted"], "crashed_or_left": o["crashed"] + o["left"],
                                      "returned": o["returned"], "timeout": o["timeout"]}
    res["generated_seconds"] = time.time() - t0
    return res


def coarse_fixture() -> dict:
    g = mq.Geom.with_spacing(0.4)
    f = mq.Fields.build(g, cache=False)
    drive = [mq.RfAc(100.0, 500e3, 0.5, 100e3 + 1e3 * k) for k in range(3)]
    out = {}
    variants = {
        "half_kick_gauss": (mq.Physics(legacy_force=True, pressure_pa=0.133322, dt=1e-7, t_max=3000e-7, launch=mq.LAUNCH_GAUSSIAN,
                                       sigma_mm=0.1), False, [0.0, 5.0, -5.0, 0.0]),
        "legacy_all": (mq.Physics(True, True, True, True, True, 0.133322, 300.0, 1e-7, 3000e-7, 0.0, mq.LAUNCH_LEGACY), True,
                       [0.0, 5.0, -5.0, 0.0]),
        "s14_like": (mq.Physics(pressure_pa=0.1, dt=4e-8, t_max=4000 * 4e-8, launch=mq.LAUNCH_DISC), False, [18.0, 24.0, 15.0, 20.0]),
    }
    for name, (ph, legsp, dc) in variants.items():
        jobs = []
        for k, mz in enumerate((493.0, 499.0, 505.0)):
            sp = mq.Species(mz * 5, 5.0, 0.0) if legsp else mq.Species(mz, 1.0, 2.95 * mz ** (2 / 3))
            jobs.append(mq.Job(sp, drive[k], 64, 1000 + k))
        G = R.Grid3(f.nx, f.ny, f.nz, f.h, f.rf, f.ac, f.dc_field(dc))
        b = R.batch(ph, 100.0, 500e3, g.axis(), g.layers())
        s = R.inject(b, jobs, 192)
        R.run(G, b, jobs, s)
        for k, _ in R.FIELDS:
            out[f"{name}.{k}"] = getattr(s, k)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default="/root/reference")
    ap.add_argument("--skip-pins", action="store_true")
    a = ap.parse_args()
    np.savez_compressed(HERE / "oracle_coarse.npz", **coarse_fixture())
    print("wrote oracle_coarse.npz")
    if not a.skip_pins:
        res = pins(Path(a.reference))
        (HERE / "pins.json").write_text(json.dumps(res, indent=1))
        print("wrote pins.json")


if __name__ == "__main__":
    main()
