"""Parity at the full sizes of the measured workloads, through properties that do not depend on size
(the oracle is too slow to replay these batches ion by ion):

* the batched sweep (64 f_ac x 8 V_ac x 32 m/z x 256 ions = 4,194,304 ions on the 0.100 mm
  grid): every ion finishes and is counted once; a rerun gives the same bits; every ion of
  sampled jobs has the state it gets when its job runs alone; on 16 ions of every job the mixed
  engine's outcome-class counts match the FP64 kernel's (which is bit-exact with the oracle) at the
  95% level (one chi-square over the classes, p >= 0.05), and so do the whole batch's totals over
  four seed sets;
* the tandem (1,048,576 tracks, nine 0.050 mm port grids): the region census conserves tracks
  at every frame, the port counters balance, and a rerun gives the same bits;
* the default launch shapes of the finer grids.

The grid study's grids (FP64 = oracle, mixed vs FP64) are in test_gpu_configs.py.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sweep_jobs(mq, ions_per_job=256, seed0=0):
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
    from multiq_workbench_gb300 import validate as V
    r = V.compare_classes(V.class_counts(om), V.class_counts(o64))
    print(f"\nPARITY config 2 (16 ions of each of the 16,384 jobs): chi2 {r['chi2']:.2f} dof {r['dof']} p {r['p']:.3f}; "
          + ", ".join(f"{k} {c['a']}/{c['b']} ({c['pull']:+.2f})" for k, c in r["classes"].items()))
    assert r["p"] >= 0.05, r


def test_full_sweep_counts_at_four_seed_sets(grid_0p1):
    """The whole batch (4,194,304 ions) on both kernels at four seed sets (job seeds offset by 0, 1e6,
    2e6, 3e6): the mixed engine's outcome-class totals over the four sets match the FP64 kernel's at
    the 95% level (one chi-square over the classes of the pooled 16.8 M ions; each set's own p is
    printed, and with four sets a single one below 0.05 is expected one time in five)."""
    import multiq_workbench_gb300 as mq
    from multiq_workbench_gb300 import validate as V
    tot_m, tot_64, per_set = None, None, []
    for seed0 in (0, 1_000_000, 2_000_000, 3_000_000):
        jobs, ph, dc = _sweep_jobs(mq, seed0=seed0)
        table = mq.JobTable.from_jobs(jobs)
        with mq.Engine(grid_0p1, mq.PREC_MIXED) as e:
            cm = V.class_counts(e.run_batch(table, dc, ph))
        with mq.Engine(grid_0p1, mq.PREC_F64) as e64:
            c64 = V.class_counts(e64.run_batch(table, dc, ph))
        per_set.append(V.compare_classes(cm, c64)["p"])
        tot_m = cm if tot_m is None else {k: tot_m[k] + cm[k] for k in cm}
        tot_64 = c64 if tot_64 is None else {k: tot_64[k] + c64[k] for k in c64}
    r = V.compare_classes(tot_m, tot_64)
    print(f"\nPARITY config 2, whole batch at four seed sets: chi2 {r['chi2']:.2f} dof {r['dof']} p {r['p']:.3f} "
          f"(per set {' / '.join(f'{q:.2f}' for q in per_set)}); "
          + ", ".join(f"{k} {c['a']}/{c['b']} ({c['pull']:+.2f})" for k, c in r["classes"].items()))
    assert r["p"] >= 0.05, r


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
    8.0 GB at 0.100 / 0.050 / 0.0333 mm give 3 / 1 / 1), and each shape runs the grid-study
    launch to completion."""
    import multiq_workbench_gb300 as mq
    ph = mq.Physics(legacy_force=True, pressure_pa=0.133322, temp_k=300.0, dt=1e-7, t_max=2000 * 1e-7,
                    launch=mq.LAUNCH_GAUSSIAN, sigma_mm=0.1)
    jobs = [mq.Job(mq.Species(499.0, 1.0, 2.95 * 499.0 ** (2 / 3)), mq.RfAc(100.0, 500e3, 0.5, 100e3), 1000, s)
            for s in range(8)]
    for h, want in ((0.05, 1), (0.1 / 3.0, 1)):
        f = mq.Fields.build(mq.Geom.with_spacing(h), bases=[0, 1, 3, 4], cache=False, device=0)
        with mq.Engine(f, mq.PREC_MIXED) as e:
            assert e.tuning()["blocks_per_sm"] == want, h
            assert not e.tuning()["wide_records"], h   # 48-byte records beyond 1 GB
            out = e.run_batch(jobs, [0.0, 5.0, -5.0, 0.0], ph)
            assert int(out.n.sum()) == 8000
        del f
