"""The mixed engine's loss-surface test at the resolution of its double-float position.

The mixed engine holds positions as FP32 double-floats (about 48 bits) and crosses the exit and
return planes on the full double-float against double-float thresholds.  Here ions sit within
+-2e-9 m of a plane - closer than one FP32 ulp of the position in grid units - with no field and
no gas, so one step moves them by exactly their velocity: the FP64 kernel's classification after
that step is then the exact one, and the mixed engine must reproduce it for every ion.  A numpy
restatement of a test on the FP32 high part alone misclassifies some of these ions, which shows the
placement is fine enough to tell the two apart.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SPACING = 2e-12      # m between neighbouring ions' distances to the plane
PER_SIDE = 1000      # ions on each side of each plane


def _run(coarse, legacy_criteria: bool):
    import multiq_workbench_gb300 as mq
    ph = mq.Physics(legacy_criteria=legacy_criteria, legacy_force=True, pressure_pa=0.0, temp_k=300.0, dt=1e-7,
                    t_max=1e-3, launch=mq.LAUNCH_GAUSSIAN, sigma_mm=0.1)
    g = coarse.geom
    if legacy_criteria:
        z_exit, z_ret = 23.7e-3, 1.0e-3
    else:
        z_exit, z_ret = g.layers()[4] * 1e-3, 0.5e-3
    off = (np.arange(-PER_SIDE, PER_SIDE) + 0.5) * SPACING          # signed distance to the plane after the step
    n = 2 * len(off)
    jobs = [mq.Job(mq.Species(499.0, 1.0, 185.6), mq.RfAc(0.0, 500e3, 0.0, 100e3), n, 3)]
    ions = mq.inject(coarse, jobs, ph)
    step = 1e-6                                                        # |v| dt
    ions.x[:] = g.axis() * 1e-3
    ions.y[:] = g.axis() * 1e-3
    ions.vx[:] = 0.0
    ions.vy[:] = 0.0
    ions.z[:len(off)] = z_exit + off - step                            # moving +z onto the exit plane
    ions.vz[:len(off)] = step / ph.dt
    ions.z[len(off):] = z_ret + off + step                             # moving -z onto the return plane
    ions.vz[len(off):] = -step / ph.dt
    dc = [0.0, 0.0, 0.0, 0.0]
    out = {}
    for prec in (mq.PREC_F64, mq.PREC_MIXED):
        s = ions.copy()
        with mq.Engine(coarse, prec) as e:
            e.set_dc(dc)
            e.run_ions(jobs, ph, s, max_more=1)
        out[prec] = s
    return out[mq.PREC_F64], out[mq.PREC_MIXED], z_exit, z_ret, off, coarse.h


@pytest.mark.parametrize("legacy_criteria", [False, True], ids=["standard", "legacy"])
def test_mixed_crossing_matches_fp64_within_an_fp32_ulp(coarse, legacy_criteria):
    a, b, z_exit, z_ret, off, h = _run(coarse, legacy_criteria)
    m = len(off)
    # FP64: exactly the ions beyond each plane have left through it
    assert np.array_equal(a.status[:m] == 3, off > 0)
    assert np.array_equal(a.status[m:] == 2, off < 0)
    # the rest stay alive, or (legacy exit plane at 23.7 mm, beyond this grid's last node layer at
    # 23.6 mm) leave the box just short of the plane
    assert np.isin(a.status, (0, 2, 3, 4)).all()
    # the mixed engine classifies every ion as the FP64 kernel does
    diff = np.nonzero(a.status != b.status)[0]
    assert len(diff) == 0, (len(diff), diff[:8], a.status[diff[:8]], b.status[diff[:8]])
    # a test on the FP32 high part alone would not: positions rounded to FP32 grid units against the
    # thresholds rounded to FP32
    zx = (np.float64(z_exit) + off) / h
    zr = (np.float64(z_ret) + off) / h
    hi_exit = zx.astype(np.float32) > np.float32(z_exit / h)
    hi_ret = zr.astype(np.float32) < np.float32(z_ret / h)
    wrong = int((hi_exit != (off > 0)).sum() + (hi_ret != (off < 0)).sum())
    assert wrong > 0
