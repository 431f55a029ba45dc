"""Parity on the five benchmark configurations as they are stated, on the GPU.

Each configuration is run by the plain FP64 kernel and by the mixed-precision engine:

* the FP64 kernel must equal the CPU oracle bit for bit on every ion it is compared on (all 14
  state fields);
* the mixed engine draws its own random numbers (Philox, not the FP64 path's xorshift), so its
  ions differ one by one while the distributions must not: its outcome-class counts are held to
  the FP64 kernel's at the 95% level by one chi-square test of homogeneity per configuration and
  update rule over the outcome classes (crashed, returned, transmitted, left, timeout; classes
  empty in both are dropped), p >= 0.05.  Both engines start from the same launch draws, so the
  classes are also compared ion by ion: Bowker's test of symmetry of the class-transition table
  (an ion moves from class i to j as often as from j to i), p >= 0.05.  Those two joint tests per
  configuration are the multiplicity rule: classes are not tested one by one.  Per-class pooled
  binomial pulls and the per-ion agreement are printed beside them.

Configurations (channel geometry solved on the GPU, 100 V / 500 kHz RF, 0.5 V / 100 kHz
excitation, DC [0, +5, -5, 0] V, 1 mTorr N2 at 300 K, z = +1 with N2 CCS 2.95 m^(2/3) A^2,
Gaussian launch sigma 0.1 mm at z = 1 mm with 300 K Maxwell velocities, dt 100 ns, <= 20,000 steps):

0. single channel: 1,000 ions of m = 499 Da, seed 0, 0.100 mm grid, corrected and half-kick rules;
1. mass scan: m/z 475..523 step 2 (25 jobs) x 1,000 ions, job k seed k, both rules (also the
   per-job chi-squares summed over the 25 jobs, the scan's shape);
3. grid study: the config-0 launch on grids solved at 0.100 / 0.050 / 0.0333 mm (half-kick rule):
   FP64 = oracle on 192 ions, mixed vs FP64 on 16 seeds x 1,000 ions;
4. tandem: 1,048,576 tracks at the nine mouths, nine 0.050 mm port grids, 1,000 global steps:
   per-port entered / returned / forwarded / lost counts of the two engines (one Poisson chi-square
   over the 36 counters) and the per-track final region (one multinomial chi-square).

Config 2 (the 4.2 M-ion sweep) is covered in test_gpu_fullsize.py and by the bench.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELDS = ("x", "y", "z", "vx", "vy", "vz", "ph_rf", "ph_ac", "rng", "steps", "ncoll", "leg", "status", "jid")
P_MIN = 0.05
DC = [0.0, 5.0, -5.0, 0.0]


def _mq():
    import multiq_workbench_gb300 as mq
    return mq


def _physics(half_kick: bool):
    mq = _mq()
    return mq.Physics(legacy_force=half_kick, pressure_pa=0.133322, temp_k=300.0, dt=1e-7, t_max=20000 * 1e-7,
                      launch=mq.LAUNCH_GAUSSIAN, sigma_mm=0.1, z_inject_mm=1.0)


def _job(mz: float, n: int, seed: int):
    mq = _mq()
    return mq.Job(mq.Species(mz, 1.0, 2.95 * mz ** (2.0 / 3.0)), mq.RfAc(100.0, 500e3, 0.5, 100e3), n, seed)


def _oracle(f, jobs, ph):
    from oracle import mqref as R
    g = f.geom
    G = R.Grid3(f.nx, f.ny, f.nz, f.h, f.rf, f.ac, f.dc_field(DC))
    b = R.batch(ph, jobs[0].drive.v_rf, jobs[0].drive.f_rf, g.axis(), g.layers())
    s = R.inject(b, jobs, sum(j.n for j in jobs))
    R.run(G, b, jobs, s)
    return s


def _bitequal(a, b, what):
    for k in FIELDS:
        x, y = np.asarray(getattr(a, k)), np.asarray(getattr(b, k))
        same = x.view(np.uint8).reshape(len(x), -1) == y.view(np.uint8).reshape(len(y), -1)
        bad = np.nonzero(~same.all(1))[0]
        assert len(bad) == 0, f"{what}: {k} differs in {len(bad)} ions (first {bad[:5]})"


def _gate(name, om, o64, st_m=None, st_64=None):
    """One chi-square over the outcome classes and, given both engines' per-ion statuses, Bowker's
    symmetry test of the class transitions (each p >= 0.05); prints both with the per-class pulls
    and the per-ion class agreement."""
    from multiq_workbench_gb300 import validate as V
    r = V.compare_classes(V.class_counts(om), V.class_counts(o64))
    pulls = ", ".join(f"{k} {c['a']}/{c['b']} ({c['pull']:+.2f})" for k, c in r["classes"].items())
    paired = ""
    if st_m is not None:
        q = V.compare_paired(st_64, st_m)
        paired = f"; per ion: {q['agree'] * 100:.1f}% same class, Bowker {q['bowker']:.2f} dof {q['dof']} p {q['p']:.3f}"
    print(f"\nPARITY {name}: chi2 {r['chi2']:.2f} dof {r['dof']} p {r['p']:.3f}; mixed/FP64: {pulls}{paired}")
    assert r["p"] >= P_MIN, (name, r)
    if st_m is not None:
        assert q["p"] >= P_MIN, (name, q)
    return r


@pytest.fixture(scope="module")
def grid_0p1(built):
    return _mq().Fields.build(_mq().Geom(), bases=[0, 1, 3, 4], cache=False, device=0)


@pytest.mark.parametrize("half_kick", [False, True], ids=["corrected", "half_kick"])
def test_config0_single_channel(grid_0p1, half_kick):
    """1,000 ions of m = 499 Da, seed 0: FP64 = oracle bit for bit on every ion; mixed vs FP64 at 95%."""
    mq = _mq()
    ph = _physics(half_kick)
    jobs = [_job(499.0, 1000, 0)]
    with mq.Engine(grid_0p1, mq.PREC_F64) as e:
        ions = mq.IonStates.empty(1000)
        o64 = e.run_batch(jobs, DC, ph, ions_out=ions)
    _bitequal(ions, _oracle(grid_0p1, jobs, ph), "config 0 FP64 vs oracle")
    assert (ions.status != 0).all()
    with mq.Engine(grid_0p1, mq.PREC_MIXED) as e:
        im = mq.IonStates.empty(1000)
        om = e.run_batch(jobs, DC, ph, ions_out=im)
    assert int(om.n.sum()) == 1000
    _gate(f"config 0 {'half-kick' if half_kick else 'corrected'}", om, o64, im.status, ions.status)


@pytest.mark.parametrize("half_kick", [False, True], ids=["corrected", "half_kick"])
def test_config1_mass_scan(grid_0p1, half_kick):
    """m/z 475..523 step 2 x 1,000 ions, job k seed k: FP64 = oracle bit for bit on all 25,000 ions;
    mixed vs FP64 at 95% on the class totals (the gate) and, reported, the per-job chi-squares summed
    over the 25 jobs."""
    mq = _mq()
    from multiq_workbench_gb300 import validate as V
    ph = _physics(half_kick)
    jobs = [_job(475.0 + 2 * k, 1000, k) for k in range(25)]
    n = 25_000
    with mq.Engine(grid_0p1, mq.PREC_F64) as e:
        ions = mq.IonStates.empty(n)
        o64 = e.run_batch(jobs, DC, ph, ions_out=ions)
    _bitequal(ions, _oracle(grid_0p1, jobs, ph), "config 1 FP64 vs oracle")
    with mq.Engine(grid_0p1, mq.PREC_MIXED) as e:
        im = mq.IonStates.empty(n)
        om = e.run_batch(jobs, DC, ph, ions_out=im)
    assert list(om.n) == [1000] * 25
    _gate(f"config 1 {'half-kick' if half_kick else 'corrected'}", om, o64, im.status, ions.status)
    pj = V.compare_jobs([V.class_counts(om, [j]) for j in range(25)], [V.class_counts(o64, [j]) for j in range(25)])
    print(f"PARITY config 1 per-job: chi2 {pj['chi2']:.1f} dof {pj['dof']} p {pj['p']:.3f}; transmitted per m/z "
          f"mixed {[int(x) for x in om.transmitted]} FP64 {[int(x) for x in o64.transmitted]}")


def test_config1_fig4_legacy_physics(grid_0p1):
    """The reference's own legacy mass scan (chsim legacy-fig4: m/z 475..525 step 2 of 5+ ions, 1,000
    each, every legacy switch: half kick, stationary-gas collisions, nearest-node fields, point-and-cone
    launch, legacy criteria): FP64 = oracle bit for bit on every ion; mixed vs FP64 at 95%."""
    mq = _mq()
    from multiq_workbench_gb300 import chsim as CH
    ph = mq.Physics.legacy(1e-3 * 133.322)
    jobs = CH.fig4_jobs(1000)
    n = sum(j.n for j in jobs)
    with mq.Engine(grid_0p1, mq.PREC_F64) as e:
        ions = mq.IonStates.empty(n)
        o64 = e.run_batch(jobs, CH.FIG4_DC, ph, ions_out=ions)
    from oracle import mqref as R
    g = grid_0p1.geom
    G = R.Grid3(grid_0p1.nx, grid_0p1.ny, grid_0p1.nz, grid_0p1.h, grid_0p1.rf, grid_0p1.ac, grid_0p1.dc_field(CH.FIG4_DC))
    b = R.batch(ph, jobs[0].drive.v_rf, jobs[0].drive.f_rf, g.axis(), g.layers())
    s = R.inject(b, jobs, n)
    R.run(G, b, jobs, s)
    _bitequal(ions, s, "Fig. 4 legacy scan FP64 vs oracle")
    with mq.Engine(grid_0p1, mq.PREC_MIXED) as e:
        im = mq.IonStates.empty(n)
        om = e.run_batch(jobs, CH.FIG4_DC, ph, ions_out=im)
    _gate("config 1 Fig. 4 legacy physics", om, o64, im.status, ions.status)


@pytest.mark.parametrize("h_mm", [0.1, 0.05, 0.1 / 3.0], ids=["0.100mm", "0.050mm", "0.0333mm"])
def test_config3_grid_study(built, h_mm):
    """The config-0 launch (half-kick rule) on a grid solved on the GPU at 0.100 / 0.050 / 0.0333 mm
    (6.2 M / 49.6 M / 167.3 M nodes): the FP64 kernel equals the oracle bit for bit on 2 x 96 ions
    run to completion, and the mixed engine's class counts on 16 seeds x 1,000 ions match the FP64
    kernel's at 95%."""
    mq = _mq()
    ph = _physics(True)
    f = mq.Fields.build(mq.Geom.with_spacing(h_mm), bases=[0, 1, 3, 4], cache=False, device=0)
    sample = [_job(499.0, 96, s) for s in (11, 12)]
    with mq.Engine(f, mq.PREC_F64) as e:
        ions, _ = e.run_batch_ions(sample, DC, ph)
        jobs = [_job(499.0, 1000, 100 + s) for s in range(16)]
        i64 = mq.IonStates.empty(16_000)
        o64 = e.run_batch(jobs, DC, ph, ions_out=i64)
    _bitequal(ions, _oracle(f, sample, ph), f"config 3 at {h_mm:.4f} mm: FP64 vs oracle")
    with mq.Engine(f, mq.PREC_MIXED) as e:
        im = mq.IonStates.empty(16_000)
        om = e.run_batch(jobs, DC, ph, ions_out=im)
    assert int(om.n.sum()) == 16_000
    _gate(f"config 3 at {h_mm:.4f} mm", om, o64, im.status, i64.status)
    del f


def test_config4_tandem_full_pulse(built):
    """1,048,576 tracks at the nine mouths, ports on nine device copies of the 0.050 mm S14 grid,
    1,000 global steps from the same pulse in both engines.  Gates at 95%: the per-track final
    region (split, nine ports, combiner, lost, back, detected: one multinomial chi-square over the
    tracks, and Bowker's symmetry test of the per-track region transitions), and the per-port
    entered / returned / forwarded / lost counters (one chi-square over the 36 counters, each
    difference scaled by its Poisson variance a + b)."""
    mq = _mq()
    from multiq_workbench_gb300 import validate as V
    h = 0.05
    ch = mq.Fields.build(mq.Geom.s14(h_mm=h, n_xy=int(round(16.0 / h))), cache=False, device=0)
    pg = mq.PortGrid.from_fields(ch)
    grids = [pg] + [pg.replica() for _ in range(8)]
    n = 1 << 20
    res = {}
    for prec in (mq.PREC_F64, mq.PREC_MIXED):
        m = mq.TandemModel(mq.DEFAULT_TONES, n=n, seed=486, fine=True, mouth_start=True, port_grids=grids,
                           precision=prec, device=0)
        m.advance(1000)
        res[prec] = (m.counts_array().astype(np.int64), np.bincount(m.tracks.region, minlength=14), m.tracks.region.copy())
        m.close()
    (c64, r64, g64), (cm, rm, gm) = res[mq.PREC_F64], res[mq.PREC_MIXED]
    q = V.compare_paired(g64, gm)
    assert r64.sum() == n and rm.sum() == n
    reg = V.compare_classes({str(k): int(rm[k]) for k in range(14)}, {str(k): int(r64[k]) for k in range(14)})
    cols = {"entered": 0, "returned": 1, "forwarded": 2, "lost": 15}
    stat, dof, worst = 0.0, 0, (0.0, "")
    for name, c in cols.items():
        for p in range(9):
            a, b = int(cm[p, c]), int(c64[p, c])
            if a + b == 0:
                continue
            z = (a - b) / math.sqrt(a + b)
            stat += z * z
            dof += 1
            if abs(z) > abs(worst[0]):
                worst = (z, f"port {p + 1} {name} {a}/{b}")
    p_ports = V.chi2_sf(stat, dof)
    print(f"\nPARITY config 4 regions: chi2 {reg['chi2']:.2f} dof {reg['dof']} p {reg['p']:.3f}; mixed/FP64 "
          f"{[(k, c['a'], c['b']) for k, c in reg['classes'].items()]}; per track: {q['agree'] * 100:.1f}% same region, "
          f"Bowker {q['bowker']:.2f} dof {q['dof']} p {q['p']:.3f}")
    print(f"PARITY config 4 ports: chi2 {stat:.2f} dof {dof} p {p_ports:.3f}; largest pull {worst[0]:+.2f} ({worst[1]}); "
          f"totals mixed {cm[:, list(cols.values())].sum(0).tolist()} FP64 {c64[:, list(cols.values())].sum(0).tolist()}")
    assert reg["p"] >= P_MIN, reg
    assert q["p"] >= P_MIN, q
    assert p_ports >= P_MIN, (stat, dof, worst)
