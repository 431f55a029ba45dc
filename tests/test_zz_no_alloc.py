"""The allocation-free FP64 stepping call (mq_run_ions_device_noalloc).

It exists for callers that cannot allocate device memory themselves - code running inside a
host framework or plugin host that owns every device allocation, or that must not call
cudaMalloc on its path.  Here the test plays that caller: it owns the device arrays (made
with torch), and the call must advance the states exactly like the engine's FP64 entry point
(mq_run_ions with MQ_PREC_F64), bit for bit, on two calls in a row that share the library's
static scratch array.  This file is collected last so a failure here leaves every other
test already run.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELDS = ("x", "y", "z", "vx", "vy", "vz", "ph_rf", "ph_ac", "rng", "steps", "ncoll", "leg", "status", "jid")


@pytest.fixture(scope="module")
def setup():
    import __graft_entry__ as ge
    ge.build()
    import multiq_workbench_gb300 as mq
    g = mq.Geom.with_spacing(0.4)
    f = mq.Fields.build(g, bases=[0, 1, 3, 4])
    dc = [0.0, 5.0, -5.0, 0.0]
    ph = mq.Physics(legacy_force=True, pressure_pa=0.133322, dt=1e-7, t_max=3000e-7, launch=mq.LAUNCH_GAUSSIAN,
                    sigma_mm=0.1)
    jobs = [mq.Job(mq.Species(m, 1.0, 2.95 * m ** (2 / 3)), mq.RfAc(100.0, 500e3, 0.5, 100e3 + 1e3 * k), 200, 70 + k)
            for k, m in enumerate((493.0, 499.0, 505.0))]
    return mq, f, dc, ph, jobs


def _device_call(mq, f, dc, ph, jobs, host_ions, max_more):
    """Copy states to caller-owned device memory, run the allocation-free call, copy back."""
    import torch
    from multiq_workbench_gb300 import _native as N
    dev = {k: torch.from_numpy(np.ascontiguousarray(getattr(host_ions, k))).cuda() for k in FIELDS}
    rf = torch.from_numpy(f.rf).cuda()
    ac = torch.from_numpy(f.ac).cuda()
    dcf = torch.from_numpy(f.dc_field(dc)).cuda()
    grid = N.mq_dev_grid()
    grid.nx, grid.ny, grid.nz, grid.h = f.nx, f.ny, f.nz, f.h
    grid.rf4, grid.ac4, grid.dc4 = rf.data_ptr(), ac.data_ptr(), dcf.data_ptr()
    grid.axis_mm = f.geom.axis()
    for i, v in enumerate(f.geom.layers()):
        grid.layers_mm[i] = v
    io = N.mq_ions()
    for k in FIELDS:
        setattr(io, k, dev[k].data_ptr())
    steps = C.c_uint64(0)
    torch.cuda.synchronize()
    from multiq_workbench_gb300.channel import jobs_native
    code = N.lib().mq_run_ions_device_noalloc(C.byref(grid), jobs_native(jobs), len(jobs), C.byref(ph.native()),
                                              C.byref(io), len(host_ions), max_more, None, C.byref(steps))
    assert code == 0, code
    out = host_ions.copy()
    for k in FIELDS:
        getattr(out, k)[:] = dev[k].cpu().numpy()
    return out, int(steps.value)


def _same(a, b, what):
    for k in FIELDS:
        x, y = getattr(a, k), getattr(b, k)
        assert np.array_equal(x.view(np.uint8), y.view(np.uint8)), f"{what}: {k} differs"


def test_noalloc_matches_fp64_entry_point_on_two_calls(setup):
    mq, f, dc, ph, jobs = setup
    start = mq.inject(f, jobs, ph)
    ref = start.copy()
    with mq.Engine(f, mq.PREC_F64) as e:
        e.set_dc(dc)
        s1 = e.run_ions(jobs, ph, ref, max_more=400)
        ref1 = ref.copy()
        s2 = e.run_ions(jobs, ph, ref)
    got1, n1 = _device_call(mq, f, dc, ph, jobs, start, 400)          # first call: 400 steps
    _same(got1, ref1, "first call")
    assert n1 == s1.ion_steps
    got2, n2 = _device_call(mq, f, dc, ph, jobs, got1, 0xFFFFFFFF)    # second call: to completion
    _same(got2, ref, "second call")
    assert n2 == s2.ion_steps
    assert (got2.status != 0).all()


def test_noalloc_refuses_an_ion_whose_job_index_is_out_of_range(setup):
    """The states are device memory, so the call checks every ion's job index on the device before
    stepping: one index equal to njobs makes it return MQ_ERR_INVALID with the states untouched,
    and the next call with good indices runs as before."""
    import torch
    mq, f, dc, ph, jobs = setup
    from multiq_workbench_gb300 import _native as N
    from multiq_workbench_gb300.channel import jobs_native
    start = mq.inject(f, jobs, ph)
    bad = start.copy()
    bad.jid[17] = len(jobs)
    dev = {k: torch.from_numpy(np.ascontiguousarray(getattr(bad, k))).cuda() for k in FIELDS}
    rf, ac, dcf = (torch.from_numpy(a).cuda() for a in (f.rf, f.ac, f.dc_field(dc)))
    grid = N.mq_dev_grid()
    grid.nx, grid.ny, grid.nz, grid.h = f.nx, f.ny, f.nz, f.h
    grid.rf4, grid.ac4, grid.dc4 = rf.data_ptr(), ac.data_ptr(), dcf.data_ptr()
    grid.axis_mm = f.geom.axis()
    for i, v in enumerate(f.geom.layers()):
        grid.layers_mm[i] = v
    io = N.mq_ions()
    for k in FIELDS:
        setattr(io, k, dev[k].data_ptr())
    torch.cuda.synchronize()
    code = N.lib().mq_run_ions_device_noalloc(C.byref(grid), jobs_native(jobs), len(jobs), C.byref(ph.native()),
                                              C.byref(io), len(start), 100, None, None)
    assert code == -1     # MQ_ERR_INVALID
    for k in FIELDS:
        assert np.array_equal(dev[k].cpu().numpy().view(np.uint8), getattr(bad, k).view(np.uint8)), k
    got, _ = _device_call(mq, f, dc, ph, jobs, start, 100)
    ref = start.copy()
    with mq.Engine(f, mq.PREC_F64) as e:
        e.set_dc(dc)
        e.run_ions(jobs, ph, ref, max_more=100)
    _same(got, ref, "after a refused call")


def test_noalloc_rejects_batches_beyond_its_scratch(setup):
    mq, f, dc, ph, jobs = setup
    from multiq_workbench_gb300 import _native as N
    from multiq_workbench_gb300.channel import jobs_native
    many = [mq.Job(jobs[0].sp, jobs[0].drive, 1, k) for k in range(4097)]
    grid = N.mq_dev_grid()
    grid.nx = grid.ny = grid.nz = 8
    grid.h = 1e-3
    grid.rf4 = grid.ac4 = grid.dc4 = 1      # never dereferenced: the size check comes first
    io = N.mq_ions()
    for k in FIELDS:
        setattr(io, k, 1)
    code = N.lib().mq_run_ions_device_noalloc(C.byref(grid), jobs_native(many), len(many), C.byref(ph.native()),
                                              C.byref(io), 4097, 10, None, None)
    assert code == -8     # MQ_ERR_TOO_LARGE
