"""Failure detection on the device path, with every failure made on the host (nothing faults,
traps or hangs the GPU): an exhausted launch budget is reported by the watchdog from the real
survivor count and the states come back resumable; allocation and launch failures come back as
status codes; a grid larger than the device is refused at creation; the engine stays usable and
gives the same results as before after each failure."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELDS = ("x", "y", "z", "vx", "vy", "vz", "ph_rf", "ph_ac", "rng", "steps", "ncoll", "leg", "status", "jid")


def _setup():
    import multiq_workbench_gb300 as mq
    ph = mq.Physics(legacy_force=True, pressure_pa=0.133322, temp_k=300.0, dt=1e-7, t_max=3000e-7,
                    launch=mq.LAUNCH_GAUSSIAN, sigma_mm=0.1)
    jobs = [mq.Job(mq.Species(mz, 1.0, 2.95 * mz ** (2 / 3)), mq.RfAc(100.0, 500e3, 0.5, 100e3 + 1e3 * k), 128, 70 + k)
            for k, mz in enumerate((493.0, 499.0, 505.0))]
    return mq, ph, jobs, [0.0, 5.0, -5.0, 0.0]


def _same(a, b):
    return all(np.array_equal(np.asarray(getattr(a, k)).view(np.uint8), np.asarray(getattr(b, k)).view(np.uint8))
               for k in FIELDS)


@pytest.mark.parametrize("prec", ["f64", "mixed"])
def test_watchdog_reports_survivors_and_states_resume(coarse, prec):
    mq, ph, jobs, dc = _setup()
    p = mq.PREC_F64 if prec == "f64" else mq.PREC_MIXED
    with mq.Engine(coarse, p) as e:
        e.set_dc(dc)
        ref = e.inject(jobs, ph)
        e.run_ions(jobs, ph, ref)                      # uninterrupted
        ions = e.inject(jobs, ph)
        e.inject_fault(mq.FAULT_LAUNCH_BUDGET)
        with pytest.raises(mq.MqError) as ei:
            e.run_ions(jobs, ph, ions)
        assert ei.value.code == -4 and "live ions" in str(ei.value)
        live = ions.status == 0
        assert live.any() and np.all(ions.steps[live] == 16) and np.all(ions.steps <= 16)
        e.run_ions(jobs, ph, ions)                     # resume to completion
        assert np.all(ions.status != 0)
        if p == mq.PREC_F64:
            assert _same(ions, ref)                    # the FP64 state is an exact checkpoint
        else:
            assert abs(int((ions.status == 3).sum()) - int((ref.status == 3).sum())) <= 3 * np.sqrt(len(ions)) + 5


@pytest.mark.parametrize("prec", ["f64", "mixed"])
def test_alloc_and_launch_failures_are_status_codes(coarse, prec):
    mq, ph, jobs, dc = _setup()
    p = mq.PREC_F64 if prec == "f64" else mq.PREC_MIXED
    with mq.Engine(coarse, p) as e:
        good, _ = e.run_batch_ions(jobs, dc, ph)
        for kind, code in ((mq.FAULT_ALLOC, -3), (mq.FAULT_LAUNCH, -2), (mq.FAULT_LAUNCH_BUDGET, -4)):
            e.inject_fault(kind)
            with pytest.raises(mq.MqError) as ei:
                e.run_batch(jobs, dc, ph)
            assert ei.value.code == code, (kind, str(ei.value))
            again, _ = e.run_batch_ions(jobs, dc, ph)   # usable, and the same results as before
            assert _same(again, good), kind
        e.inject_fault(mq.FAULT_ALLOC)
        e.inject_fault(mq.FAULT_NONE)                  # cleared: the next call runs
        e.run_batch(jobs, dc, ph)
        with pytest.raises(mq.MqError):
            e.inject_fault(7)


def test_grid_larger_than_the_device_is_refused(built):
    """Engine creation on a 4096^3 grid (1.1 TB per field): the FP64 engine fails at the first device
    allocation, before any host array is read, with MQ_ERR_NOMEM; the mixed engine refuses it before
    that with MQ_ERR_TOO_LARGE (its record offsets are 32-bit)."""
    import ctypes as C
    from multiq_workbench_gb300 import _native as N
    small = np.zeros(16, np.float32)
    g = N.mq_grid_desc()
    g.nx = g.ny = g.nz = 4096
    g.h = 1e-4
    g.rf4 = g.ac4 = small.ctypes.data
    h = C.c_void_p()
    assert N.lib().mq_engine_create(C.byref(g), 0, 0, C.byref(h)) == -3
    assert not h.value
    assert N.lib().mq_engine_create(C.byref(g), 1, 0, C.byref(h)) == -8
    assert not h.value
