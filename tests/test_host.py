"""Host-side logic without a GPU: injection parity with the oracle, physics presets, the C
ABI's exported symbols and its refusal paths, and job sharding across ranks."""
import ctypes as C
import os
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


@pytest.mark.parametrize("launch,legacy,rf0", [(0, False, True), (1, True, True), (2, False, False), (2, False, True)])
def test_host_injection_equals_oracle(coarse, launch, legacy, rf0):
    import multiq_workbench_gb300 as mq
    from oracle import mqref as R
    ph = mq.Physics(legacy_collisions=legacy, legacy_injection=legacy, pressure_pa=0.133322, dt=1e-7, t_max=1e-3,
                    r_inject_mm=2.0, launch=launch, sigma_mm=0.1, rf_phase0=rf0)
    jobs = [mq.Job(mq.Species(499.0 * z, z, 185.6 if z == 1 else 0.0), mq.RfAc(100.0, 500e3, 0.5, 1e5), 300, 17 + int(z))
            for z in (1.0, 5.0)]
    ions = mq.inject(coarse, jobs, ph)
    g = coarse.geom
    s = R.inject(R.batch(ph, 100.0, 500e3, g.axis(), g.layers()), jobs, 600)
    for k, _ in R.FIELDS:
        assert np.array_equal(getattr(ions, k).view(np.uint8), getattr(s, k).view(np.uint8)), k
    if launch == 2:
        r = np.hypot(ions.x - g.axis() * 1e-3, ions.y - g.axis() * 1e-3)
        assert 0.08e-3 < np.sqrt((r ** 2).mean() / 2) < 0.12e-3       # sigma 0.1 mm per axis
    if rf0:
        assert (ions.ph_rf == 0).all()


def test_physics_presets_follow_chsim(monkeypatch):
    import multiq_workbench_gb300 as mq
    leg = mq.Physics.legacy(0.1333)
    assert (leg.legacy_force, leg.legacy_collisions, leg.legacy_fields, leg.legacy_injection, leg.legacy_criteria) == (True,) * 5
    assert (leg.dt, leg.t_max, leg.r_inject_mm) == (1e-7, 1.0, 0.0)
    monkeypatch.delenv("CHSIM_DT_DIV", raising=False)
    cor = mq.Physics.correct(0.1)
    assert (cor.dt, cor.t_max, cor.r_inject_mm) == (4e-8, 0.02, 2.0)
    monkeypatch.setenv("CHSIM_DT_DIV", "100")
    assert mq.Physics.correct(0.1).dt == 2e-8


def _declared_functions():
    names = []
    for h in (ROOT / "include").glob("*.h"):
        txt = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names += re.findall(r"\b(mq_[a-z0-9_]+)\s*\(", txt)
    return sorted(set(names))


def test_library_exports_every_declared_symbol(built):
    from multiq_workbench_gb300 import _native as N
    L = N.lib()
    names = _declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_abi_refusals_without_device(coarse):
    """Engine creation reports a status code (never aborts); with no device it is MQ_ERR_NO_DEVICE."""
    import multiq_workbench_gb300 as mq
    from multiq_workbench_gb300 import _native as N
    L = N.lib()
    h = C.c_void_p()
    desc = coarse.grid_desc()
    assert L.mq_engine_create(None, 0, 0, C.byref(h)) == -1
    assert L.mq_engine_create(C.byref(desc), 7, 0, C.byref(h)) == -1
    if mq.device_count() == 0:
        assert L.mq_engine_create(C.byref(desc), 1, 0, C.byref(h)) == -6
        with pytest.raises(mq.MqError):
            mq.Engine(coarse)
    # injection with a bad total and an RF mismatch is refused
    ph = mq.Physics(pressure_pa=0.1)
    jobs = [mq.Job(mq.Species(499.0, 1.0, 185.6), mq.RfAc(100.0, 500e3, 0.5, 1e5), 4, 1),
            mq.Job(mq.Species(499.0, 1.0, 185.6), mq.RfAc(90.0, 500e3, 0.5, 1e5), 4, 2)]
    with pytest.raises(mq.MqError) as ei:
        mq.inject(coarse, jobs, ph)
    assert ei.value.code == -5


def test_summarize_c_matches_oracle(built):
    import multiq_workbench_gb300 as mq
    from oracle import mqref as R
    rng = np.random.default_rng(5)
    n = 1000
    ions = mq.IonStates.empty(n)
    ions.status[:] = rng.integers(0, 6, n)
    ions.jid[:] = rng.integers(0, 7, n)
    ions.ncoll[:] = rng.integers(0, 100, n)
    ions.steps[:] = rng.integers(0, 20000, n)
    a = mq.summarize(ions, 7, 1e-7)
    s = R.State.from_arrays(ions)
    b = R.Batch()
    b.dt = 1e-7
    o = R.summarize(s, b, 7)
    for x, y in zip(a, o):
        assert (x.n, x.crashed, x.returned, x.transmitted, x.left, x.timeout) == \
               (y["n"], y["crashed"], y["returned"], y["transmitted"], y["left"], y["timeout"])
        assert x.mean_coll == y["mean_coll"] and x.mean_time == y["mean_time"]


def test_l2_probe_refusals_without_device(built):
    import ctypes as C
    import multiq_workbench_gb300 as mq
    from multiq_workbench_gb300 import _native as N
    g = C.c_double(0.0)
    assert N.lib().mq_measure_l2_read_gbs(0, 200 << 20, 10, C.byref(g)) == -1      # above 96 MiB
    assert N.lib().mq_measure_l2_read_gbs(0, 32 << 20, 10, None) == -1
    if mq.device_count() == 0:
        assert N.lib().mq_measure_l2_read_gbs(0, 32 << 20, 10, C.byref(g)) == -6


def test_fault_injection_needs_an_engine(built):
    from multiq_workbench_gb300 import _native as N
    assert N.lib().mq_engine_inject_fault(None, 1) == -1


def test_noalloc_entry_refuses_bad_jobs_and_physics(built):
    """The allocation-free entry point applies the job and physics checks of every other entry
    point before it touches a device: zero mass, zero charge, negative CCS, zero temperature,
    negative pressure or t_max, and a batch whose RF drives differ are refused (the pointers are
    never dereferenced: the checks come first)."""
    import dataclasses
    import multiq_workbench_gb300 as mq
    from multiq_workbench_gb300 import _native as N
    from multiq_workbench_gb300.channel import jobs_native
    grid = N.mq_dev_grid()
    grid.nx = grid.ny = grid.nz = 8
    grid.h = 1e-3
    grid.rf4 = grid.ac4 = grid.dc4 = 1
    io = N.mq_ions()
    for k, _ in mq.channel.ION_FIELDS:
        setattr(io, k, 1)
    good = mq.Physics(pressure_pa=0.1)
    drive = mq.RfAc(100.0, 500e3, 0.5, 1e5)

    def call(jobs, ph):
        return N.lib().mq_run_ions_device_noalloc(C.byref(grid), jobs_native(jobs), len(jobs), C.byref(ph.native()),
                                                  C.byref(io), 4, 10, None, None)
    for sp in (mq.Species(0.0, 1.0, 185.6), mq.Species(499.0, 0.0, 185.6), mq.Species(499.0, 1.0, -1.0)):
        assert call([mq.Job(sp, drive, 4, 1)], good) == -1, sp
    sp = mq.Species(499.0, 1.0, 185.6)
    for bad in (dict(temp_k=0.0), dict(pressure_pa=-1.0), dict(t_max=-1e-6), dict(dt=0.0)):
        assert call([mq.Job(sp, drive, 4, 1)], dataclasses.replace(good, **bad)) == -1, bad
    assert call([mq.Job(sp, drive, 2, 1), mq.Job(sp, mq.RfAc(90.0, 500e3, 0.5, 1e5), 2, 2)], good) == -5


def test_hash_ions_is_fnv1a_over_the_fields(built):
    """check.hash_ions (native FNV-1a 64, check.rs:95-99) equals the byte-by-byte definition."""
    import multiq_workbench_gb300 as mq
    from multiq_workbench_gb300 import check
    ions = mq.IonStates.empty(300)
    rng = np.random.default_rng(11)
    for name, _ in mq.channel.ION_FIELDS:
        a = getattr(ions, name)
        a.view(np.uint8)[:] = rng.integers(0, 256, a.nbytes, dtype=np.uint8)
    h = 1469598103934665603
    for b in b"".join(np.ascontiguousarray(getattr(ions, n)).tobytes() for n, _ in mq.channel.ION_FIELDS):
        h = ((h ^ b) * 1099511628211) & 0xFFFFFFFFFFFFFFFF
    assert check.hash_ions(ions) == h
