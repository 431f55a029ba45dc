"""GPU parity: the engine (through the C ABI) against the CPU oracle.

* FP64 kernel: final states equal the oracle's bit for bit, for every physics switch
  (thermal / legacy collisions, trilinear / nearest fields, standard / legacy criteria,
  disc / legacy / Gaussian launch, full / half kick, with and without gas), and when a run
  is split into partial runs (resume from returned states).
* Mixed engine: deterministic per ion; on collision-free runs its final states track the
  FP64 states to a stated tolerance; with gas its outcome counts agree with the FP64
  counts within binomial limits.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELDS = ("x", "y", "z", "vx", "vy", "vz", "ph_rf", "ph_ac", "rng", "steps", "ncoll", "leg", "status", "jid")


def _mq():
    import multiq_workbench_gb300 as mq
    return mq


def _oracle_run(f, jobs, ph, dc, max_more=None, state=None):
    from oracle import mqref as R
    g = f.geom
    G = R.Grid3(f.nx, f.ny, f.nz, f.h, f.rf, f.ac, f.dc_field(dc))
    b = R.batch(ph, jobs[0].drive.v_rf, jobs[0].drive.f_rf, g.axis(), g.layers())
    s = state.copy() if state is not None else R.inject(b, jobs, sum(j.n for j in jobs))
    R.run(G, b, jobs, s, max_more=0xFFFFFFFF if max_more is None else max_more)
    return s


def _assert_bitequal(a, b, what):
    for k in FIELDS:
        x, y = getattr(a, k), getattr(b, k)
        if not np.array_equal(np.asarray(x).view(np.uint8), np.asarray(y).view(np.uint8)):
            bad = np.nonzero(np.asarray(x).view(np.uint8).reshape(len(x), -1).any(1) !=
                             np.asarray(y).view(np.uint8).reshape(len(y), -1).any(1))[0]
            diff = np.nonzero(np.asarray(x) != np.asarray(y))[0]
            raise AssertionError(f"{what}: field {k} differs in {len(diff)} ions (first {diff[:5]}, "
                                 f"{np.asarray(x)[diff[:3]]} vs {np.asarray(y)[diff[:3]]})")


def _variants():
    mq = _mq()
    base = dict(pressure_pa=0.133322, temp_k=300.0, dt=1e-7, t_max=3000e-7)
    return {
        "corrected_disc": mq.Physics(**base, launch=mq.LAUNCH_DISC, r_inject_mm=2.0),
        "half_kick_gauss": mq.Physics(**base, legacy_force=True, launch=mq.LAUNCH_GAUSSIAN, sigma_mm=0.1),
        "legacy_all": mq.Physics(True, True, True, True, True, 0.133322, 300.0, 1e-7, 3000e-7, 0.0, mq.LAUNCH_LEGACY),
        "legacy_coll_trilinear": mq.Physics(True, True, False, True, True, 0.133322, 300.0, 1e-7, 3000e-7, 0.0, mq.LAUNCH_LEGACY),
        "thermal_nearest": mq.Physics(legacy_fields=True, legacy_force=True, **base, launch=mq.LAUNCH_GAUSSIAN),
        "no_gas_rf_random": mq.Physics(legacy_force=True, pressure_pa=0.0, temp_k=300.0, dt=1e-7, t_max=3000e-7,
                                       launch=mq.LAUNCH_GAUSSIAN, rf_phase0=False),
        "s14_like": mq.Physics(pressure_pa=0.1, temp_k=300.0, dt=4e-8, t_max=4000 * 4e-8, launch=mq.LAUNCH_DISC),
    }


def _jobs(n=192, legacy_species=False, vac=0.5):
    mq = _mq()
    out = []
    for k, mz in enumerate((493.0, 499.0, 505.0)):
        sp = mq.Species(mz * 5, 5.0, 0.0) if legacy_species else mq.Species(mz, 1.0, 2.95 * mz ** (2 / 3))
        out.append(mq.Job(sp, mq.RfAc(100.0, 500e3, vac, 100e3 + 1e3 * k), n, 1000 + k))
    return out


@pytest.mark.parametrize("name", list(_variants().keys()))
def test_f64_bitexact_vs_oracle(coarse, name):
    mq = _mq()
    ph = _variants()[name]
    jobs = _jobs(legacy_species=name.startswith("legacy"))
    dc = [18.0, 24.0, 15.0, 20.0] if name == "s14_like" else [0.0, 5.0, -5.0, 0.0]
    with mq.Engine(coarse, mq.PREC_F64) as e:
        ions, _ = e.run_batch_ions(jobs, dc, ph)
    ref = _oracle_run(coarse, jobs, ph, dc)
    _assert_bitequal(ions, ref, name)
    assert (ions.status != 0).all()


def test_f64_resume_partial_runs(coarse):
    """mq_run_ions in pieces of 137 steps equals one oracle run (states are the checkpoint)."""
    mq = _mq()
    ph = _variants()["half_kick_gauss"]
    jobs = _jobs(128)
    dc = [0.0, 5.0, -5.0, 0.0]
    ions = mq.inject(coarse, jobs, ph)
    with mq.Engine(coarse, mq.PREC_F64) as e:
        e.set_dc(dc)
        for _ in range(4):
            e.run_ions(jobs, ph, ions, max_more=137)
        from oracle import mqref as R
        s = R.State.from_arrays(ions)
        ref = _oracle_run(coarse, jobs, ph, dc, max_more=137 * 4, state=R.State.from_arrays(mq.inject(coarse, jobs, ph)))
        _assert_bitequal(ions, ref, "after 4 x 137 steps")
        e.run_ions(jobs, ph, ions)
    ref2 = _oracle_run(coarse, jobs, ph, dc, state=s)
    _assert_bitequal(ions, ref2, "resumed to completion")


def test_run_batch_counts_match_states(coarse):
    mq = _mq()
    ph = _variants()["half_kick_gauss"]
    jobs = _jobs(256)
    dc = [0.0, 5.0, -5.0, 0.0]
    for prec in (mq.PREC_F64, mq.PREC_MIXED):
        with mq.Engine(coarse, prec) as e:
            ions = mq.IonStates.empty(sum(j.n for j in jobs))
            out = e.run_batch(jobs, dc, ph, ions_out=ions)
        ref = mq.summarize(ions, len(jobs), ph.dt)
        for a, b in zip(out, ref):
            assert (a.n, a.crashed, a.returned, a.transmitted, a.left, a.timeout) == \
                   (b.n, b.crashed, b.returned, b.transmitted, b.left, b.timeout)
            assert math.isclose(a.mean_time, b.mean_time, rel_tol=1e-12)
            assert math.isclose(a.mean_coll, b.mean_coll, rel_tol=1e-12)


def test_mixed_deterministic(coarse):
    """Per-ion results do not depend on scheduling: two runs (and two launch shapes) agree bitwise."""
    mq = _mq()
    ph = _variants()["half_kick_gauss"]
    jobs = _jobs(512)
    dc = [0.0, 5.0, -5.0, 0.0]
    with mq.Engine(coarse, mq.PREC_MIXED) as e:
        a, _ = e.run_batch_ions(jobs, dc, ph)
        e.set_tuning(blocks_per_sm=2, chunk=700)
        b, _ = e.run_batch_ions(jobs, dc, ph)
    _assert_bitequal(a, b, "mixed run twice")


@pytest.mark.parametrize("name", ["half_kick_gauss", "legacy_all", "legacy_coll_trilinear"])
def test_mixed_requeue_mid_window_is_bitwise(coarse, name):
    """Launches of 701 steps re-queue every surviving ion at a step count that is not a multiple of
    4, so its refill rebuilds the drive state and the Philox blocks of a window already begun (the
    thermal candidates' blocks, or the legacy collisions' two blocks per window): every ion's final
    state equals the single-launch run's bit for bit, for thermal gas and for legacy collisions with
    nearest-node and with trilinear fields."""
    mq = _mq()
    ph = _variants()[name]
    jobs = _jobs(512, legacy_species=name.startswith("legacy"))
    dc = [0.0, 5.0, -5.0, 0.0]
    with mq.Engine(coarse, mq.PREC_MIXED) as e:
        a, _ = e.run_batch_ions(jobs, dc, ph)
        e.set_tuning(chunk=701)
        b, _ = e.run_batch_ions(jobs, dc, ph)
        assert e.last_stats.step_kernel_launches == 5
    _assert_bitequal(a, b, f"{name}: 701-step launches vs one launch")


def test_cell_sort_keeps_every_result(coarse):
    """Putting each launch's live list in the Morton order of the ions' cells (a device counting sort
    before every launch) changes only which ions share a warp: with 700-step launches (so the list is
    re-sorted 4 times per ion lifetime) every ion's final state equals the unsorted single-launch run
    bit for bit, so no ion is lost or stepped twice; the same holds on the CUDA-graph path."""
    mq = _mq()
    ph = _variants()["half_kick_gauss"]
    jobs = _jobs(512)
    dc = [0.0, 5.0, -5.0, 0.0]
    with mq.Engine(coarse, mq.PREC_MIXED) as e:
        a, _ = e.run_batch_ions(jobs, dc, ph)
        e.set_tuning(chunk=700, sort_cells=True, use_graph=False)
        b, _ = e.run_batch_ions(jobs, dc, ph)
        e.set_tuning(use_graph=True)
        c, _ = e.run_batch_ions(jobs, dc, ph)
        assert e.last_stats.graph_replays == 1 and e.last_stats.step_kernel_launches == 5
        e.set_tuning(sort_cells=False)
        d, _ = e.run_batch_ions(jobs, dc, ph)
    _assert_bitequal(a, b, "sorted 700-step launches vs one launch")
    _assert_bitequal(a, c, "sorted launches replayed as a graph")
    _assert_bitequal(a, d, "unsorted graph")


def test_record_widths_agree_bitwise(coarse):
    """48-byte node records (128-bit loads) and 64-byte ones (256-bit loads) hold the same
    values: per-ion results agree bit for bit, with and without the L1 prefetch, and switching
    the width re-packs the records on the next call."""
    mq = _mq()
    ph = _variants()["half_kick_gauss"]
    jobs = _jobs(512)
    dc = [0.0, 5.0, -5.0, 0.0]
    with mq.Engine(coarse, mq.PREC_MIXED) as e:
        assert e.tuning()["wide_records"]          # the default below 1 GB of 48-byte records
        a, _ = e.run_batch_ions(jobs, dc, ph)
        e.set_tuning(wide_records=False)
        b, _ = e.run_batch_ions(jobs, dc, ph)
        e.set_tuning(prefetch=True)
        c, _ = e.run_batch_ions(jobs, dc, ph)
        e.set_tuning(wide_records=True)
        d, _ = e.run_batch_ions(jobs, dc, ph)
    _assert_bitequal(a, b, "wide vs narrow records")
    _assert_bitequal(a, c, "wide vs narrow records with prefetch")
    _assert_bitequal(a, d, "wide records with prefetch")


@pytest.mark.parametrize("name", ["corrected_disc", "half_kick_gauss", "legacy_all"])
def test_mixed_injection_draws(coarse, name):
    """The mixed engine's device injection (a batch of zero steps returns it) makes the FP64
    injection's draws: generator state, job, phases and counters equal bit for bit; from the
    FP32 transforms, positions within 1e-5 cell, velocities within 4e-6 of |v| + the batch's median
    |v| (an FP32 angle carries ~1e-7 absolute error, however slow the ion), and the
    first-collision step count within 1e-5 relative (or 1 step)."""
    import dataclasses
    mq = _mq()
    ph = dataclasses.replace(_variants()[name], t_max=0.0)
    jobs = _jobs(700, legacy_species=(name == "legacy_all"))
    n = sum(j.n for j in jobs)
    with mq.Engine(coarse, mq.PREC_MIXED) as e:
        ref = e.inject(jobs, ph)
        got = mq.IonStates.empty(n)
        out = e.run_batch(jobs, [0.0, 5.0, -5.0, 0.0], ph, ions_out=got)
    assert sum(o.n for o in out) == n
    for k in ("z", "ph_rf", "ph_ac", "rng", "steps", "ncoll", "status", "jid"):
        assert np.array_equal(getattr(got, k), getattr(ref, k)), k
    h = coarse.h
    assert np.abs(got.pos() - ref.pos()).max() <= 1e-5 * h
    vr, vg = ref.vel(), got.vel()
    vn = np.linalg.norm(vr, axis=1)
    assert (np.linalg.norm(vg - vr, axis=1) <= 4e-6 * (vn + np.median(vn))).all()
    lr, lg = ref.leg.astype(np.float64), got.leg.astype(np.float64)
    assert (np.abs(lg - lr) <= np.maximum(1e-5 * lr, 1.0)).all()


def test_ragged_and_empty_jobs(coarse):
    """Jobs of 1, 0, 33, 2, 255 and 64 ions in one batch: the FP64 kernel's states equal the
    oracle's bit for bit, both engines count every job's ions once (the empty job included), and
    a batch whose jobs are all empty returns zero counts."""
    mq = _mq()
    ph = _variants()["half_kick_gauss"]
    dc = [0.0, 5.0, -5.0, 0.0]
    sizes = (1, 0, 33, 2, 255, 64)
    jobs = [mq.Job(mq.Species(mz, 1.0, 2.95 * mz ** (2 / 3)), mq.RfAc(100.0, 500e3, 0.5, 99e3 + 500.0 * k), nn, 500 + k)
            for k, (mz, nn) in enumerate(zip((491.0, 493.0, 497.0, 499.0, 503.0, 507.0), sizes))]
    ref = _oracle_run(coarse, jobs, ph, dc)
    with mq.Engine(coarse, mq.PREC_F64) as e:
        ions, _ = e.run_batch_ions(jobs, dc, ph)
        _assert_bitequal(ions, ref, "ragged FP64 vs oracle")
        out = e.run_batch(jobs, dc, ph)
        assert list(out.n) == list(sizes)
        empty = e.run_batch([mq.Job(j.sp, j.drive, 0, j.seed) for j in jobs], dc, ph)
        assert all(o.n == 0 and o.transmitted == 0 for o in empty)
    with mq.Engine(coarse, mq.PREC_MIXED) as e:
        out = e.run_batch(jobs, dc, ph)
        assert list(out.n) == list(sizes)
        assert all(o.crashed + o.returned + o.transmitted + o.left + o.timeout == o.n for o in out)
        empty = e.run_batch([mq.Job(j.sp, j.drive, 0, j.seed) for j in jobs], dc, ph)
        assert all(o.n == 0 for o in empty)
        # more than 2^32 - 16 ions in one batch is refused before anything is allocated
        huge = [mq.Job(jobs[0].sp, jobs[0].drive, 1 << 31, 1), mq.Job(jobs[0].sp, jobs[0].drive, 1 << 31, 2)]
        with pytest.raises(mq.MqError) as ei:
            e.run_batch(huge, dc, ph)
        assert ei.value.code == -8
        assert list(e.run_batch(jobs, dc, ph).n) == list(sizes)     # still usable


def test_mixed_collision_free_tracks_fp64(coarse):
    """No gas: the mixed engine's compensated FP32 state follows the FP64 trajectory.
    Tolerance: after 300 steps |dx| <= 1e-3 cell and |dv|/|v| <= 1e-4 for ions alive in both."""
    mq = _mq()
    ph = _variants()["no_gas_rf_random"]
    jobs = _jobs(256)
    dc = [0.0, 5.0, -5.0, 0.0]
    ions0 = mq.inject(coarse, jobs, ph)
    a, b = ions0.copy(), ions0.copy()
    with mq.Engine(coarse, mq.PREC_F64) as e:
        e.set_dc(dc)
        e.run_ions(jobs, ph, a, max_more=300)
    with mq.Engine(coarse, mq.PREC_MIXED) as e:
        e.set_dc(dc)
        e.run_ions(jobs, ph, b, max_more=300)
    alive = (a.status == 0) & (b.status == 0)
    assert alive.sum() > 100
    h = coarse.h
    dx = np.abs(a.pos()[alive] - b.pos()[alive]).max() / h
    va, vb = a.vel()[alive], b.vel()[alive]
    dv = (np.linalg.norm(va - vb, axis=1) / np.maximum(np.linalg.norm(va, axis=1), 1.0)).max()
    assert dx <= 1e-3, dx
    assert dv <= 1e-4, dv
    same = (a.status == b.status).mean()
    assert same >= 0.99, same


def test_mixed_outcome_counts_vs_fp64(coarse):
    """With gas: per-outcome totals within 5 binomial sigma (pooled) of the FP64 engine."""
    mq = _mq()
    ph = _variants()["half_kick_gauss"]
    jobs = _jobs(2048)
    dc = [0.0, 5.0, -5.0, 0.0]
    with mq.Engine(coarse, mq.PREC_F64) as e:
        o64 = e.run_batch(jobs, dc, ph)
    with mq.Engine(coarse, mq.PREC_MIXED) as e:
        om = e.run_batch(jobs, dc, ph)
    n = sum(o.n for o in o64)
    for k in ("transmitted", "returned", "crashed", "left", "timeout"):
        a = sum(getattr(o, k) for o in om)
        b = sum(getattr(o, k) for o in o64)
        p = (a + b + 1) / (2 * n + 2)
        assert abs(a - b) <= 5 * math.sqrt(2 * n * p * (1 - p)) + 2, (k, a, b)


def test_errors_are_status_codes(coarse):
    mq = _mq()
    ph = _variants()["half_kick_gauss"]
    jobs = _jobs(8)
    bad = jobs + [mq.Job(jobs[0].sp, mq.RfAc(90.0, 500e3, 0.5, 1e5), 8, 1)]
    with mq.Engine(coarse, mq.PREC_MIXED) as e:
        with pytest.raises(mq.MqError) as ei:
            e.run_batch(bad, [0, 5, -5, 0], ph)
        assert ei.value.code == -5 and "RF drive must be shared" in str(ei.value)
        with pytest.raises(mq.MqError) as ei:
            e.run_batch([], [0, 5, -5, 0], ph)
        assert ei.value.code == -1
        with pytest.raises(mq.MqError):
            e.set_tuning(blocks_per_sm=9)
        # the engine stays usable after errors
        out = e.run_batch(jobs, [0, 5, -5, 0], ph)
        assert sum(o.n for o in out) == sum(j.n for j in jobs)


def test_default_shape_on_a_small_grid(coarse):
    """3 resident blocks per SM below 1 GB of node records (the larger grids are in
    test_gpu_fullsize.py)."""
    mq = _mq()
    with mq.Engine(coarse, mq.PREC_MIXED) as e:
        assert e.tuning()["blocks_per_sm"] == 3


def test_autotune_picks_a_valid_shape(coarse):
    mq = _mq()
    ph = _variants()["half_kick_gauss"]
    jobs = _jobs(256)
    with mq.Engine(coarse, mq.PREC_MIXED) as e:
        t, rate = e.autotune(jobs, [0, 5, -5, 0], ph, sample_per_job=64)
        assert t["blocks_per_sm"] in (1, 2, 3) and t["chunk"] > 0 and rate > 0
