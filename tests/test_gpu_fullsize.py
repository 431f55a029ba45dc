"""Parity at the full sizes of the measured workloads, through properties that do not depend on size
(the oracle is too slow to replay these batches ion by ion):

* the batched sweep (64 f_ac x 8 V_ac x 32 m/z x 256 ions = 4,194,304 ions on the 0.100 mm
  grid): every ion finishes and is counted once; a rerun gives the same bits; every ion of
  sampled jobs has the state it gets when its job runs alone; the mixed engine's outcome counts
  match the FP64 kernel's (which is bit-exact with the oracle) within binomial limits;
* the tandem (1,048,576 tracks, nine 0.050 mm port grids): the region census conserves tracks
  at every frame, the port counters balance, and a rerun gives the same bits;
* the grid study's 0.050 mm grid (49.6 M nodes): the FP64 kernel equals the oracle bit for bit on
  a sample of its launch (the oracle replays a few hundred ions there in under a second), and the
  mixed engine's outcome totals match the FP64 kernel's on 16,000 ions.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sweep_jobs(mq, ions_per_job=256):
    fac = np.linspace(80e3, 120e3, 64)
    vac = np.linspace(0.1, 1.0, 8)
    mzs = [470.0 + 2 * k for k in range(32)]
    jobs = []
    for a in fac:
        for v in vac:
            for m in mzs:
                jobs.append(mq.Job(mq.Species(m, 1.0, 2.95 * m ** (2.0 / 3.0)), mq.RfAc(100.0, 500e3, float(v), float(a)),
                                   ions_per_job, len(jobs)))
    ph = mq.Physics(legacy_force=True, pressure_pa=0.133322, temp_k=300.0, dt=1e-7, t_max=20000 * 1e-7,
                    launch=mq.LAUNCH_GAUSSIAN, sigma_mm=0.1, z_inject_mm=1.0)
    return jobs, ph, [0.0, 5.0, -5.0, 0.0]


@pytest.fixture(scope="module")
def grid_0p1(built):
    import multiq_workbench_gb300 as mq
    return mq.Fields.build(mq.Geom(), bases=[0, 1, 3, 4], cache=False, device=0)


def test_full_sweep_properties(grid_0p1):
    import multiq_workbench_gb300 as mq
    from multiq_workbench_gb300 import check
    jobs, ph, dc = _sweep_jobs(mq)
    n = sum(j.n for j in jobs)
    assert n == 4_194_304
    with mq.Engine(grid_0p1, mq.PREC_MIXED) as e:
        a = mq.IonStates.empty(n)
        oa = e.run_batch(jobs, dc, ph, ions_out=a)
        b = mq.IonStates.empty(n)
        ob = e.run_batch(jobs, dc, ph, ions_out=b)
        # every ion finishes, once, in its own job
        assert np.all(a.status != 0) and np.all(oa.n == 256)
        assert int(oa.crashed.sum() + oa.returned.sum() + oa.transmitted.sum() + oa.left.sum() + oa.timeout.sum()) == n
        assert np.array_equal(a.jid, np.repeat(np.arange(len(jobs), dtype=np.uint32), 256))
        # a rerun of the whole batch gives the same bits
        assert oa == ob and check.compare(a, b)["differ"] == 0
        # sampled jobs run alone give their ions the batch's states
        for k in (0, 1, 4097, 8191, 12000, 16383):
            alone, _ = e.run_batch_ions([jobs[k]], dc, ph)
            part = mq.IonStates.empty(256)
            for name, _ in mq.channel.ION_FIELDS:
                getattr(part, name)[:] = getattr(a, name)[k * 256:(k + 1) * 256]
            part.jid[:] = 0
            assert check.compare(alone, part)["differ"] == 0, k
        # mixed vs FP64 on 16 ions of every job
        sj = [mq.Job(j.sp, j.drive, 16, j.seed) for j in jobs]
        om = e.run_batch(sj, dc, ph)
    with mq.Engine(grid_0p1, mq.PREC_F64) as e64:
        o64 = e64.run_batch(sj, dc, ph)
    m = int(o64.n.sum())
    for k in ("transmitted", "returned", "crashed", "timeout"):
        x, y = int(getattr(om, k).sum()), int(getattr(o64, k).sum())
        p = (x + y + 1) / (2 * m + 2)
        pull = (x - y) / math.sqrt(2 * m * p * (1 - p))
        assert abs(pull) < 4.0, (k, x, y, pull)


def test_full_tandem_properties(built):
    import multiq_workbench_gb300 as mq
    h = 0.05
    ch = mq.Fields.build(mq.Geom.s14(h_mm=h, n_xy=int(round(16.0 / h))), cache=False, device=0)
    pg = mq.PortGrid.from_fields(ch)
    grids = [pg] + [pg.replica() for _ in range(8)]
    n = 1 << 20
    runs = []
    for _ in range(2):
        m = mq.TandemModel(mq.DEFAULT_TONES, n=n, seed=486, fine=True, mouth_start=True, port_grids=grids,
                           precision=1, device=0)
        fr = []
        for _ in range(3):
            m.advance(100)
            f = m.frame()
            fr.append(f)
            assert f.split + f.channel + f.combine + f.lost + f.back + f.detected == n
        cnt = m.counts_array()
        # trapsim's routing identities (lib.rs:494-501): every entry into a port (forward or
        # reverse) ends as a return, a forward or a loss, or is still inside a port
        entered, returned, forwarded, lost_p, reverse = cnt[:, 0], cnt[:, 1], cnt[:, 2], cnt[:, 15], cnt[:, 14]
        assert int((entered + reverse).sum()) == int((returned + forwarded + lost_p).sum()) + f.channel
        assert cnt[:, 3].sum() == cnt[:, 5:14].sum() and cnt[:, 16:21].sum() == forwarded.sum()
        assert (entered > 0).all()
        runs.append((m.tracks.copy(), cnt.copy()))
        m.close()
    (ta, ca), (tb, cb) = runs
    assert np.array_equal(ca, cb)
    from multiq_workbench_gb300.tandem import TRACK_FIELDS
    for k, _ in TRACK_FIELDS:
        assert np.array_equal(getattr(ta, k).view(np.uint8), getattr(tb, k).view(np.uint8)), k


def test_default_shape_follows_the_grid_size(built):
    """Fewer resident blocks per SM on grids far larger than L2 (node records of 0.30 / 2.4 /
    8.0 GB at 0.100 / 0.050 / 0.0333 mm give 3 / 2 / 1), and each shape runs the grid-study
    launch to completion."""
    import multiq_workbench_gb300 as mq
    ph = mq.Physics(legacy_force=True, pressure_pa=0.133322, temp_k=300.0, dt=1e-7, t_max=2000 * 1e-7,
                    launch=mq.LAUNCH_GAUSSIAN, sigma_mm=0.1)
    jobs = [mq.Job(mq.Species(499.0, 1.0, 2.95 * 499.0 ** (2 / 3)), mq.RfAc(100.0, 500e3, 0.5, 100e3), 1000, s)
            for s in range(8)]
    for h, want in ((0.05, 2), (0.1 / 3.0, 1)):
        f = mq.Fields.build(mq.Geom.with_spacing(h), bases=[0, 1, 3, 4], cache=False, device=0)
        with mq.Engine(f, mq.PREC_MIXED) as e:
            assert e.tuning()["blocks_per_sm"] == want, h
            assert not e.tuning()["wide_records"], h   # 48-byte records beyond 1 GB
            out = e.run_batch(jobs, [0.0, 5.0, -5.0, 0.0], ph)
            assert int(out.n.sum()) == 8000
        del f


@pytest.fixture(scope="module")
def grid_0p05(built):
    import multiq_workbench_gb300 as mq
    return mq.Fields.build(mq.Geom.with_spacing(0.05), bases=[0, 1, 3, 4], cache=False, device=0)


def test_f64_bitexact_vs_oracle_on_the_0p05_grid(grid_0p05):
    """Bit-exact FP64 parity at a large grid: on the 0.050 mm channel grid of the grid study
    (320 x 320 x 484 = 49.6 M nodes, solved on the GPU) the FP64 kernel's final states of 2 jobs x
    96 ions of the grid-study launch, run to completion, equal the oracle's in all 14 fields."""
    import multiq_workbench_gb300 as mq
    from oracle import mqref as R
    f = grid_0p05
    dc = [0.0, 5.0, -5.0, 0.0]
    ph = mq.Physics(legacy_force=True, pressure_pa=0.133322, temp_k=300.0, dt=1e-7, t_max=20000 * 1e-7,
                    launch=mq.LAUNCH_GAUSSIAN, sigma_mm=0.1)
    drive = mq.RfAc(100.0, 500e3, 0.5, 100e3)
    jobs = [mq.Job(mq.Species(499.0, 1.0, 2.95 * 499.0 ** (2.0 / 3.0)), drive, 96, s) for s in (11, 12)]
    with mq.Engine(f, mq.PREC_F64) as e:
        ions, _ = e.run_batch_ions(jobs, dc, ph)
    g = f.geom
    G = R.Grid3(f.nx, f.ny, f.nz, f.h, f.rf, f.ac, f.dc_field(dc))
    b = R.batch(ph, drive.v_rf, drive.f_rf, g.axis(), g.layers())
    s = R.inject(b, jobs, len(ions))
    R.run(G, b, jobs, s)
    assert int((s.status != 0).sum()) == len(ions)
    for name, _ in R.FIELDS:
        a, c = np.asarray(getattr(ions, name)), np.asarray(getattr(s, name))
        assert np.array_equal(a.view(np.uint8), c.view(np.uint8)), name


def test_mixed_counts_vs_fp64_on_the_0p05_grid(grid_0p05):
    """The mixed engine on the same 0.050 mm grid (48-byte records, 2 blocks per SM): 16 seeds x
    1,000 ions of the grid-study launch give outcome totals within 5 pooled binomial sigma of the
    FP64 kernel's, and every ion is counted once."""
    import multiq_workbench_gb300 as mq
    dc = [0.0, 5.0, -5.0, 0.0]
    ph = mq.Physics(legacy_force=True, pressure_pa=0.133322, temp_k=300.0, dt=1e-7, t_max=20000 * 1e-7,
                    launch=mq.LAUNCH_GAUSSIAN, sigma_mm=0.1)
    drive = mq.RfAc(100.0, 500e3, 0.5, 100e3)
    jobs = [mq.Job(mq.Species(499.0, 1.0, 2.95 * 499.0 ** (2.0 / 3.0)), drive, 1000, 100 + s) for s in range(16)]
    with mq.Engine(grid_0p05, mq.PREC_F64) as e:
        o64 = e.run_batch(jobs, dc, ph)
    with mq.Engine(grid_0p05, mq.PREC_MIXED) as e:
        t = e.tuning()
        assert t["blocks_per_sm"] == 2 and not t["wide_records"]
        om = e.run_batch(jobs, dc, ph)
    n = 16 * 1000
    assert int(om.n.sum()) == n and int(o64.n.sum()) == n
    for k in ("transmitted", "returned", "crashed", "timeout"):
        a, b = int(getattr(om, k).sum()), int(getattr(o64, k).sum())
        p = (a + b + 1) / (2 * n + 2)
        assert abs(a - b) <= 5 * math.sqrt(2 * n * p * (1 - p)) + 2, (k, a, b)
