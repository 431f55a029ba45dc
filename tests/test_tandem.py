"""Tandem transport on the CPU: the oracle pinned against the reference's own unit tests
(simulation/trapsim/src/geometry.rs:210-231, lib.rs:388-446), the host code (geometry, cube
fields, track launch) against the oracle bit for bit, and the oracle's own invariants
(chunked = unchunked, thread-count independence, the conservation identity of the
reference's routing regression, lib.rs:494-501)."""
import ctypes as C

import numpy as np
import pytest

import multiq_workbench_gb300 as mq
from multiq_workbench_gb300 import tandem as T
from oracle import mqtandem as O

FREE, POST, PLANE, ENT, EXT = 0, 1, 2, 3, 4


def _cubes(code=False, array=False):
    g = mq.CubeGeometry.code_dims() if code else mq.CubeGeometry.as_built()
    g.array = array
    return g, O.cube_from(g.native())


# ------------------------------------------------------------------ reference unit tests


def test_post_counts():   # geometry.rs:211-220
    g, o = _cubes()
    assert O.lib().mqt_n_posts(C.byref(o)) == 488
    assert abs(O.lib().mqt_size(C.byref(o)) - 86.0) < 1e-9
    assert abs(g.size() - 86.0) < 1e-9
    c, oc = _cubes(code=True)
    assert abs(O.lib().mqt_size(C.byref(oc)) - 83.0) < 1e-9
    assert abs(c.size() - 83.0) < 1e-9
    assert abs(c.r0() - 2.6334) < 1e-3
    assert abs(g.r0() - 2.699) < 1e-3


def test_quad_axis_is_open_until_plane():   # geometry.rs:221-231
    g, o = _cubes(code=True)
    x = y = 0.5 * (g.lat(1) + g.lat(2))
    cases = [((x, y, 6.0), FREE), ((x, y, 1.0), PLANE), ((g.lat(1), g.lat(1), 5.0), POST),
             ((g.lat(1), g.lat(1), 1.0), POST), ((g.lat(1) + 2.5, g.lat(1), 1.0), FREE)]
    for p, want in cases:
        assert O.classify(o, p)[0] == want, p
        assert g.classify(p)[0] == want, p


def test_nine_open_mouths_with_solid_board_between():   # lib.rs:390-404
    g, o = _cubes(array=True)
    for i in range(9):
        x, y = O.port_axis(o, i)
        assert (x, y) == g.port_axis(i)
        assert O.lib().mqt_nearest_port(C.byref(o), x, y) == i
        assert g.nearest_port(x, y) == i
        assert O.classify(o, (x, y, g.size() - 0.2))[0] == FREE
        assert g.classify((x, y, g.size() - 0.2))[0] == FREE
    x, y = g.port_axis(0)
    assert O.classify(o, (x + g.pitch, y, g.size() - 0.2))[0] == PLANE
    assert g.classify((x + g.pitch, y, g.size() - 0.2))[0] == PLANE


def test_rejection_preserves_phase_space_and_allows_a_different_port():   # lib.rs:405-445
    s = O.State(1)
    s.rng[0] = 0x9E3779B97F4A7C15
    s.region[0], s.last[0], s.sp[0] = 0, -1, 0
    counts = np.zeros((9, O.NC), np.uint32)
    cp = lambda k: counts[k].ctypes.data_as(C.POINTER(C.c_uint32))
    size, axis = 0.086, 0.008
    c0 = (C.c_double * 2)(0.024, 0.042)
    pos = (0.0242, 0.0419, size + 1e-6)
    s.x[0], s.y[0], s.z[0] = pos
    rng = int(s.rng[0])
    t = s.native()
    O.lib().mqt_enter(C.byref(t), 0, 0, 0, size, c0, axis, cp(0))
    s.vx[0], s.vy[0], s.vz[0] = 3.0, 7.0, -20.0
    s.z[0] = T.Z_RETURN - 1e-6
    O.lib().mqt_leave(C.byref(t), 0, 0, size, c0, axis, cp(0))
    assert s.region[0] == 0
    assert abs(s.x[0] - pos[0]) < 1e-14
    assert abs(s.z[0] - (size - 1e-6)) < 1e-14
    assert (s.vx[0], s.vy[0], s.vz[0]) == (3.0, 7.0, -20.0)
    assert int(s.rng[0]) == rng
    c1 = (C.c_double * 2)(0.04, 0.042)
    s.x[0], s.y[0], s.z[0] = 0.04, 0.042, size + 1e-6
    O.lib().mqt_enter(C.byref(t), 0, 1, 0, size, c1, axis, cp(1))
    assert counts[1][4] == 1   # from_other
    s.z[0] = T.Z_EXIT + 1e-6
    s.vz[0] = 30.0
    O.lib().mqt_leave(C.byref(t), 0, 1, size, c1, axis, cp(1))
    assert s.region[0] == 10
    assert s.vz[0] == -30.0


# ------------------------------------------------------------------ host code vs the oracle


def test_classify_matches_oracle_everywhere():
    rng = np.random.default_rng(7)
    for code, array in ((False, True), (True, False)):
        g, o = _cubes(code, array)
        L = g.size()
        pts = rng.uniform(-12.0, L + 12.0, size=(4000, 3))
        # plus points on lattice lines and planes, where ties of round() live
        lat = np.array([g.lat(i) for i in range(g.n)])
        pts[:500, 0] = rng.choice(lat, 500)
        pts[500:1000, 2] = rng.choice([0.0, g.t_pcb, L - g.t_pcb, L, -g.l_ext, L + g.l_ext], 500)
        for grow in (0.0, 0.4 * 1.0375):
            for p in pts:
                assert g.classify(p, grow) == O.classify(o, p, grow), (p, grow)


def test_track_launch_matches_oracle(tandem_small):
    for mouth in (True, False):
        m = tandem_small(n=257, seed=12345, mouth_start=mouth)
        d = O.desc_from(m.desc)
        s = O.inject(d, 12345, mouth, 257)
        for k, _ in O.TRACK_FIELDS:
            assert np.array_equal(getattr(s, k).view(np.uint8), getattr(m.tracks, k).view(np.uint8)), k
        seam, size, mouths = O.layout(d)
        assert (seam, size) == (m.seam, m.size)
        assert np.array_equal(mouths, m.mouth)
        assert set(np.unique(m.tracks.sp)) <= set(range(5))
        assert np.all(m.tracks.region == 0) and np.all(m.tracks.last == -1)


def test_species_draw_follows_abundance(tandem_small):
    m = tandem_small(n=20000, seed=3)
    w = np.array([h for _, h in T.FIG5C_HEIGHT])
    frac = np.bincount(m.tracks.sp, minlength=5) / 20000
    assert np.all(np.abs(frac - w / w.sum()) < 0.015)


def test_cube_fields_electrodes(tandem_small):
    m = tandem_small(n=1)
    cube = m.cube
    ids = cube.rf[:, 3].astype(int)
    nx, ny, nz = cube.dims
    i, j, k = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    q = (i + nx * (j + ny * k)).ravel()
    sel = q[:: max(1, q.size // 3000)]
    h = cube.h_mm
    for qq in sel:
        ii, jj, kk = qq % nx, (qq // nx) % ny, qq // (nx * ny)
        p = (cube.lo_mm[0] + h * ii, cube.lo_mm[1] + h * jj, cube.lo_mm[2] + h * kk)
        assert m.geom.classify(p, 0.4 * h)[0] == ids[qq]
    phi = cube.wall[:, 3]
    assert np.all(phi[ids == PLANE] == 1.0)
    assert np.all(phi[(ids != PLANE) & (ids != FREE)] == 0.0)
    assert phi.min() >= -1e-6 and phi.max() <= 1.0 + 1e-6
    # wall + entrance + exit bases lie in [0, 1] (the post basis completes them to 1)
    tot = cube.wall[:, 3] + cube.ent[:, 3] + cube.ext[:, 3]
    assert tot.min() >= -1e-5 and tot.max() <= 1.0 + 1e-5
    assert np.all(m.dc[0][:, 3][ids == POST] == np.float32(20.0))


# ------------------------------------------------------------------ oracle invariants


def _census(region):
    return np.bincount(region, minlength=14)


def test_oracle_chunking_and_threads_are_invisible(tandem_small):
    m = tandem_small(n=90, seed=11)
    d = O.desc_from(m.desc)
    a = O.inject(d, 11, True, 90)
    b = a.copy()
    ca = O.advance(d, a, 0, 6000, threads=1)
    cb = O.advance(d, b, 0, 2500, threads=5)
    O.advance(d, b, 2500, 3500, counts=cb, threads=3)
    for k, _ in O.TRACK_FIELDS:
        assert np.array_equal(getattr(a, k).view(np.uint8), getattr(b, k).view(np.uint8)), k
    assert np.array_equal(ca, cb)


@pytest.mark.parametrize("mouth", [True, False])
def test_oracle_routing_conservation(tandem_small, mouth):
    """physical_routing's identities (lib.rs:494-501) on the coarse model."""
    n = 180
    m = tandem_small(n=n, seed=486, mouth_start=mouth)
    d = O.desc_from(m.desc)
    s = O.inject(d, 486, mouth, n)
    cnt = O.advance(d, s, 0, 60000)
    c = _census(s.region)
    split, channel, combine, lost, back, detected = c[0], c[1:10].sum(), c[10], c[11], c[12], c[13]
    assert split + channel + combine + detected + lost + back == n
    entered, returned, forwarded, lost_p, reverse = cnt[:, 0], cnt[:, 1], cnt[:, 2], cnt[:, 15], cnt[:, 14]
    assert (entered + reverse).sum() == (returned + forwarded + lost_p).sum() + channel
    assert cnt[:, 3].sum() == cnt[:, 5:14].sum()          # every revisit has a source port
    assert cnt[:, 16:21].sum() == forwarded.sum()          # every forward has a charge state
    assert (cnt[:, 4] <= cnt[:, 3]).all()
    if mouth:
        assert (entered > 0).all() and returned.sum() > 0
    assert entered.sum() > 0


def test_oracle_rejects_bad_tracks(tandem_small):
    m = tandem_small(n=4)
    d = O.desc_from(m.desc)
    s = O.inject(d, 1, True, 4)
    s.sp[2] = 7
    with pytest.raises(ValueError):
        O.advance(d, s, 0, 10)


def test_frame_census(tandem_small):
    m = tandem_small(n=50)
    m.tracks.region[:] = np.arange(50) % 14
    f = m.frame()
    c = _census(m.tracks.region)
    assert (f.split, f.channel, f.combine, f.lost, f.back, f.detected) == (
        c[0], c[1:10].sum(), c[10], c[11], c[12], c[13])
    assert f.points.shape == (int((m.tracks.region <= 10).sum()), 5)
    assert f.size_mm == pytest.approx(m.size * 1000.0)


def test_port_track_advances_like_the_channel_integrator(tandem_small, s14_coarse):
    """A track inside a driven port advances like the FP64 channel integrator (world.rs:498-536)
    over one 128-step block: position within 1e-12 m, velocity within 1e-7 m/s, equal RNG state
    (the reference's check, lib.rs:458-482).  Both sides are oracles; the drives differ only in
    the rounding of the phase argument."""
    from oracle import mqref as R
    m = tandem_small(n=1, seed=42)
    d = O.desc_from(m.desc)
    f = s14_coarse
    ph = mq.Physics.correct(m.preset.pressure_pa)
    ph.dt, ph.t_max = T.DT, 3e-3
    sp = m.preset.species[0]
    job = mq.Job(mq.Species(sp.mass, sp.z, sp.ccs), mq.RfAc(m.preset.v_rf, T.F_RF, m.preset.v_ac, m.tones[0] * 1e3), 1, 42)
    b = R.batch(ph, job.drive.v_rf, job.drive.f_rf, f.geom.axis(), f.geom.layers())
    b.rf_phase0 = 1
    ions = R.inject(b, [job], 1)
    ions.ph_ac[0] = 0.0   # the reference's check sets the AC phase offset to 0 (sin 0, cos 1)
    ions.ph_rf[0] = 0.0
    tr = O.State(1)
    tr.x[0], tr.y[0], tr.z[0] = ions.x[0], ions.y[0], ions.z[0]
    tr.vx[0], tr.vy[0], tr.vz[0] = ions.vx[0], ions.vy[0], ions.vz[0]
    tr.rng[0], tr.sp[0], tr.region[0], tr.last[0] = ions.rng[0], 0, 1, -1
    g3 = R.Grid3(f.nx, f.ny, f.nz, f.h, f.rf, f.ac, f.dc_field(T.DC_CAL))
    R.run(g3, b, [job], ions, threads=1, max_more=128)
    cnt = O.advance(d, tr, 0, 128)
    assert ions.status[0] == 0 and ions.steps[0] == 128
    assert tr.region[0] == 1 and not cnt.any()
    for a, c in (("x", "x"), ("y", "y"), ("z", "z")):
        assert abs(getattr(ions, a)[0] - getattr(tr, c)[0]) < 1e-12
    for a in ("vx", "vy", "vz"):
        assert abs(getattr(ions, a)[0] - getattr(tr, a)[0]) < 1e-7
    assert int(ions.rng[0]) == int(tr.rng[0])
