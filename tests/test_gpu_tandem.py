"""Tandem transport on the GPU: the FP64 kernel against the oracle, bit for bit (track states
and every per-port counter), across resumed advances, both launch modes, per-port grids of
different spacing, and the host's refusals."""
import numpy as np
import pytest

import multiq_workbench_gb300 as mq
from oracle import mqtandem as O

pytestmark = pytest.mark.gpu


def _same_tracks(a, b):
    for k, _ in O.TRACK_FIELDS:
        x, y = getattr(a, k), getattr(b, k)
        if not np.array_equal(x.view(np.uint8), y.view(np.uint8)):
            diff = np.flatnonzero(x != y)
            raise AssertionError(f"{k}: {diff.size} tracks differ, first {diff[:5]}: {x[diff[:5]]} vs {y[diff[:5]]}")


def _run_both(m, chunks, seed, mouth):
    d = O.desc_from(m.desc)
    ref = O.inject(d, seed, mouth, m.tracks.n)
    cnt = np.zeros((9, O.NC), np.uint32)
    s0 = 0
    for k in chunks:
        m.advance(k)
        O.advance(d, ref, s0, k, counts=cnt)
        s0 += k
    return ref, cnt


@pytest.mark.parametrize("mouth", [True, False])
def test_tandem_gpu_matches_oracle_bitwise(tandem_small, mouth):
    m = tandem_small(n=301, seed=486, mouth_start=mouth)
    ref, cnt = _run_both(m, [5000, 7001, 12999], 486, mouth)
    _same_tracks(m.tracks, ref)
    assert np.array_equal(m.counts_array(), cnt)
    assert m.counts_array()[:, 0].sum() > 0   # ports were entered
    m.close()


def test_tandem_gpu_per_port_grids(tandem_small, s14_coarse):
    """Ragged batching by field id: ports on grids of different spacing and shape."""
    other = mq.Fields.build(mq.Geom.s14(h_mm=0.5, n_xy=32))
    ports = [s14_coarse if i % 2 == 0 else other for i in range(9)]
    m = tandem_small(n=200, seed=99, port_fields=ports)
    ref, cnt = _run_both(m, [9000, 9000], 99, True)
    _same_tracks(m.tracks, ref)
    assert np.array_equal(m.counts_array(), cnt)
    m.close()


def test_tandem_gpu_long_run_conservation(tandem_small):
    n = 2048
    m = tandem_small(n=n, seed=2024)
    ref, cnt = _run_both(m, [40000, 40000], 2024, True)
    _same_tracks(m.tracks, ref)
    got = m.counts_array()
    assert np.array_equal(got, cnt)
    f = m.frame()
    assert f.split + f.channel + f.combine + f.detected + f.lost + f.back == n
    assert (got[:, 0] + got[:, 14]).sum() == (got[:, 1] + got[:, 2] + got[:, 15]).sum() + f.channel
    assert got[:, 4].sum() > 0 and got[:, 2].sum() > 0   # from_other and forwarded happen
    m.close()


def test_tandem_gpu_refuses_bad_tracks(tandem_small):
    m = tandem_small(n=8)
    m.tracks.sp[3] = 6
    with pytest.raises(mq.MqError) as e:
        m.advance(10)
    assert e.value.code == -1
    m.tracks.sp[3] = 0
    m.tracks.region[5] = 14
    with pytest.raises(mq.MqError):
        m.advance(10)
    m.tracks.region[5] = 0
    m.advance(10)   # the model is still usable
    m.close()


def test_tandem_gpu_replica_grids_match_shared(tandem_small):
    """Nine device-resident copies of one grid give exactly the shared-grid result."""
    a = tandem_small(n=150, seed=5)
    pg = a.port_grids[0]
    b = tandem_small(n=150, seed=5, port_grids=[pg] + [pg.replica() for _ in range(8)])
    for m in (a, b):
        m.advance(6000)
    _same_tracks(a.tracks, b.tracks)
    assert np.array_equal(a.counts_array(), b.counts_array())
    st = b.last_stats
    assert st.track_steps == st.steps_cube + st.steps_port + st.steps_idle > 0
    a.close()
    b.close()


def test_tandem_gpu_step_counts_match_oracle(tandem_small):
    m = tandem_small(n=500, seed=8)
    d = O.desc_from(m.desc)
    ref = O.inject(d, 8, True, 500)
    ns = np.zeros(3, np.uint64)
    O.advance(d, ref, 0, 7000, nsteps=ns)
    st = m.advance(7000)
    assert (st.steps_cube, st.steps_port, st.steps_idle) == tuple(int(v) for v in ns)
    assert st.launches >= 1 and st.kernel_ms > 0
    m.close()


def test_port_track_advances_like_the_fp64_channel_engine(tandem_small, s14_coarse):
    """The GPU tandem's port region against the GPU FP64 channel engine over one 128-step block
    (lib.rs:458-482): position within 1e-12 m, velocity within 1e-7 m/s, equal RNG state."""
    from multiq_workbench_gb300 import tandem as T
    m = tandem_small(n=1, seed=42)
    f = s14_coarse
    ph = mq.Physics.correct(m.preset.pressure_pa)
    ph.dt, ph.t_max = T.DT, 3e-3
    sp = m.preset.species[0]
    job = mq.Job(mq.Species(sp.mass, sp.z, sp.ccs), mq.RfAc(m.preset.v_rf, T.F_RF, m.preset.v_ac, m.tones[0] * 1e3), 1, 42)
    with mq.Engine(f, mq.PREC_F64) as eng:
        eng.set_dc(list(T.DC_CAL))
        ions = eng.inject([job], ph)
        ions.ph_ac[0] = 0.0
        ions.ph_rf[0] = 0.0
        tr = m.tracks
        tr.x[0], tr.y[0], tr.z[0] = ions.x[0], ions.y[0], ions.z[0]
        tr.vx[0], tr.vy[0], tr.vz[0] = ions.vx[0], ions.vy[0], ions.vz[0]
        tr.rng[0], tr.sp[0], tr.region[0], tr.last[0] = ions.rng[0], 0, 1, -1
        eng.run_ions([job], ph, ions, max_more=128)
    m.advance(128)
    assert ions.status[0] == 0 and ions.steps[0] == 128 and tr.region[0] == 1
    for a in ("x", "y", "z"):
        assert abs(getattr(ions, a)[0] - getattr(tr, a)[0]) < 1e-12
    for a in ("vx", "vy", "vz"):
        assert abs(getattr(ions, a)[0] - getattr(tr, a)[0]) < 1e-7
    assert int(ions.rng[0]) == int(tr.rng[0])
    m.close()


# ------------------------------------------------------------------ the mixed-precision tandem engine


def _region_counts(m):
    return np.bincount(m.tracks.region, minlength=14)


def test_tandem_mixed_deterministic(tandem_small):
    a = tandem_small(n=3000, seed=21, precision=mq.PREC_MIXED)
    b = tandem_small(n=3000, seed=21, precision=mq.PREC_MIXED)
    for m in (a, b):
        m.advance(7000)
    _same_tracks(a.tracks, b.tracks)
    assert np.array_equal(a.counts_array(), b.counts_array())
    assert a.counts_array()[:, 0].sum() > 0
    a.close()
    b.close()


def test_tandem_mixed_collision_free_tracks_fp64(tandem_small):
    """Without gas the mixed engine follows the FP64 kernel: after 400 steps ≥ 99% of the tracks
    are in the same region and ≥ 99% of those at the same place to 1e-6 m with the same velocity
    to 1e-4 relative (a track that crosses a routing threshold one step apart drifts further)."""
    fig5 = mq.TandemPreset.fig5()
    vac = mq.TandemPreset(species=fig5.species, pressure_pa=0.0)
    a = tandem_small(n=2000, seed=77, preset=vac)
    b = tandem_small(n=2000, seed=77, preset=vac, precision=mq.PREC_MIXED)
    for m in (a, b):
        m.advance(400)
    same = a.tracks.region == b.tracks.region
    assert same.mean() >= 0.99
    live = same & (a.tracks.region <= 10)
    assert live.sum() > 1000
    xa = np.stack([a.tracks.x, a.tracks.y, a.tracks.z])[:, live]
    xb = np.stack([b.tracks.x, b.tracks.y, b.tracks.z])[:, live]
    va = np.stack([a.tracks.vx, a.tracks.vy, a.tracks.vz])[:, live]
    vb = np.stack([b.tracks.vx, b.tracks.vy, b.tracks.vz])[:, live]
    close = (np.abs(xa - xb).max(axis=0) < 1e-6) & (np.linalg.norm(va - vb, axis=0) / np.linalg.norm(va, axis=0) < 1e-4)
    assert close.mean() >= 0.99, close.mean()
    assert np.median(np.abs(xa - xb).max(axis=0)) < 1e-9
    a.close()
    b.close()


def test_tandem_mixed_counts_match_fp64(tandem_small):
    """With gas the two engines draw different random numbers; their census and per-port
    counts agree within a few Poisson standard deviations."""
    a = tandem_small(n=20000, seed=3)
    b = tandem_small(n=20000, seed=3, precision=mq.PREC_MIXED)
    for m in (a, b):
        m.advance(20000)
    ca, cb = a.counts_array().astype(float), b.counts_array().astype(float)
    for col in (0, 1, 2, 15):   # entered, returned, forwarded, lost: summed over ports
        x, y = ca[:, col].sum(), cb[:, col].sum()
        assert abs(x - y) <= 4.0 * np.sqrt(x + y) + 10, (col, x, y)
    ra, rb = _region_counts(a), _region_counts(b)
    for x, y in ((ra[0], rb[0]), (ra[1:10].sum(), rb[1:10].sum()), (ra[10], rb[10]), (ra[11], rb[11])):
        assert abs(x - y) <= 4.0 * np.sqrt(x + y) + 10, (x, y)
    sa, sb = a.last_stats, b.last_stats
    assert abs(sa.track_steps - sb.track_steps) <= 0.02 * sa.track_steps
    a.close()
    b.close()
