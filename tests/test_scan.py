"""Scan drivers on the CPU: the result cache's key and line format match the reference's Rust
Debug / Display output (simulation/chsim/src/scan.rs:9-48), the cache round-trips, and the
adaptive scan picks its refinement points as scan.rs:50-78 does (driven by a stand-in engine)."""
import math


import multiq_workbench_gb300 as mq
from multiq_workbench_gb300 import scan as S


def test_rust_formatting():
    assert S.species_debug(mq.Species(499.0, 1.0, 185.6)) == "Species { mass: 499.0, z: 1.0, ccs_n2: 185.6 }"
    assert S.rfac_debug(mq.RfAc(100.0, 500e3, 0.5, 100e3)) == \
        "RfAc { v_rf: 100.0, f_rf: 500000.0, v_ac: 0.5, f_ac: 100000.0 }"
    assert S.physics_debug(mq.Physics.legacy(1e-3 * 133.322)) == (
        "Physics { legacy_force: true, legacy_collisions: true, legacy_fields: true, legacy_injection: true, "
        "legacy_criteria: true, pressure_pa: 0.133322, temp_k: 300.0, dt: 1e-7, t_max: 1.0, r_inject_mm: 0.0 }")
    assert S.physics_debug(mq.Physics.correct(0.1)) == (
        "Physics { legacy_force: false, legacy_collisions: false, legacy_fields: false, legacy_injection: false, "
        "legacy_criteria: false, pressure_pa: 0.1, temp_k: 300.0, dt: 4e-8, t_max: 0.02, r_inject_mm: 2.0 }")
    g = mq.Physics.correct(0.1)
    g.launch = mq.LAUNCH_GAUSSIAN
    assert S.physics_debug(g).endswith(" + {launch: 2, sigma_mm: 0.1}")
    for x, want in ((3.0, "3"), (0.1, "0.1"), (1.25e-5, "0.0000125"), (123.5, "123.5"), (0.0, "0"), (2e20, "200000000000000000000")):
        assert S.rust_display_f64(x) == want, x
    key = S.result_key(mq.Geom(), mq.Job(mq.Species(2495.0, 5.0, 0.0), mq.RfAc(100.0, 500e3, 0.5, 100e3), 1000, 1499),
                       [0.0, 5.0, -5.0, 0.0], mq.Physics.legacy(0.133322))
    assert key.startswith("Geom { de: 6.35, coef: 0.323, ")
    assert "|Species { mass: 2495.0, z: 5.0, ccs_n2: 0.0 }|RfAc { v_rf: 100.0, f_rf: 500000.0, v_ac: 0.5, f_ac: 100000.0 }|1000|1499|[0.0, 5.0, -5.0, 0.0]|Physics { " in key


class FakeEngine:
    """Stands in for Engine.run_batch: transmission follows a resonance in f_ac."""

    def __init__(self, f0=84.0, width=1.0, peak=0.6):
        self.calls = []
        self.f0, self.width, self.peak = f0, width, peak

    def run_batch(self, jobs, dc, ph):
        self.calls.append(list(jobs))
        out = []
        for j in jobs:
            f = j.drive.f_ac / 1e3
            t = int(round(j.n * self.peak * math.exp(-0.5 * ((f - self.f0) / self.width) ** 2)))
            out.append(mq.Outcome(j.n, j.n - t, 0, t, 0, 0, 1.5, 2.5e-5))
        return out


def test_cache_round_trip_and_hits(tmp_path):
    eng = FakeEngine()
    path = tmp_path / "results.tsv"
    geom = mq.Geom()
    ph = mq.Physics.legacy(0.133322)
    jobs = [mq.Job(mq.Species(499.0, 1.0, 185.6), mq.RfAc(100.0, 500e3, 0.5, f * 1e3), 100, k)
            for k, f in enumerate((80.0, 84.0, 88.0))]
    a = S.cached_batch(eng, geom, jobs, [0, 5, -5, 0], ph, path, log=False)
    b = S.cached_batch(eng, geom, jobs, [0, 5, -5, 0], ph, path, log=False)
    assert len(eng.calls) == 1 and a == b
    line = path.read_text().splitlines()[0]
    key, vals = line.split("\t")
    assert vals.endswith(",1.5,0.000025")
    assert len(S.load_results(path)) == 3
    # a line the reference wrote loads too, and a malformed one is skipped
    with open(path, "a") as fh:
        fh.write("some key\t10,1,2,3,4,0,0.5,0.001\nbroken\t1,2\n")
    got = S.load_results(path)
    assert got["some key"] == mq.Outcome(10, 1, 2, 3, 4, 0, 0.5, 0.001) and "broken" not in got


def test_adaptive_scan_refines_the_peak(tmp_path):
    eng = FakeEngine(f0=84.0, width=1.6)
    pts = S.adaptive_scan(eng, mq.Geom(), mq.Species(499.0, 1.0, 185.6), mq.RfAc(100.0, 500e3, 0.5, 0.0),
                          [0, 5, -5, 0], mq.Physics.legacy(0.133322), 70.0, 100.0, 2.0, 200, 2000, 0.0, 7,
                          tmp_path / "r.tsv", log=False)
    coarse, fine = eng.calls
    assert [j.drive.f_ac for j in coarse] == [(70.0 + 2.0 * i) * 1e3 for i in range(16)]
    assert [j.seed for j in coarse] == list(range(7, 23))
    ff = sorted({j.drive.f_ac / 1e3 for j in fine})
    # coarse points 82, 84, 86 are above 35% of the maximum: fine grid 80..88 in 0.5 kHz steps
    assert ff == [80.0 + 0.5 * k for k in range(17)]
    assert [j.seed for j in fine] == [7 + 100_000 + k for k in range(17)] and all(j.n == 2000 for j in fine)
    fs = [p[0] for p in pts]
    assert fs == sorted(fs) and len(pts) == 16 - 5 + 17
    assert all(p[3] == (2000 if 80.0 <= p[0] <= 88.0 else 200) for p in pts)


def test_adaptive_scan_flat_spectrum_needs_no_second_stage(tmp_path):
    eng = FakeEngine(peak=0.0)
    pts = S.adaptive_scan(eng, mq.Geom(), mq.Species(499.0, 1.0, 185.6), mq.RfAc(100.0, 500e3, 0.5, 0.0),
                          [0, 5, -5, 0], mq.Physics.legacy(0.133322), 70.0, 80.0, 2.0, 200, 2000, 0.0, 0,
                          tmp_path / "r.tsv", log=False)
    assert len(eng.calls) == 1 and len(pts) == 6
