"""Workloads for the bounds-checked build: run with MQ_LIB pointing at libmqgb_check.so (the test
tests/test_gpu_check.py does this in a subprocess).  Runs the check self-test, then every stepping
kernel on small cases (channel FP64 and mixed engines over the physics switches, states with NaN
positions and states on the box faces, the tandem FP64 and mixed engines with ports on their own
grids), and prints one JSON line with the check records."""
import ctypes as C
import json
import sys
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parent.parent))

import multiq_workbench_gb300 as mq  # noqa: E402
from multiq_workbench_gb300 import _native as N  # noqa: E402


def status(reset=0):
    en, hits, site = C.c_int32(), C.c_uint32(), C.c_uint32()
    idx, lim = C.c_uint64(), C.c_uint64()
    rc = N.lib().mq_check_status(0, reset, C.byref(en), C.byref(hits), C.byref(site), C.byref(idx), C.byref(lim))
    return dict(rc=rc, enabled=en.value, hits=hits.value, site=site.value, index=idx.value, limit=lim.value)


def main():
    out = {}
    status(reset=1)
    assert N.lib().mq_check_selftest(0) == 0
    out["selftest"] = status(reset=1)

    g = mq.Geom.with_spacing(0.4)
    f = mq.Fields.build(g, bases=[0, 1, 2, 3, 4, 5], cache=False)
    dc = [0.0, 5.0, -5.0, 0.0]
    base = dict(pressure_pa=0.133322, temp_k=300.0, dt=1e-7, t_max=2000e-7)
    variants = [
        mq.Physics(**base, launch=mq.LAUNCH_DISC, r_inject_mm=2.0),
        mq.Physics(**base, legacy_force=True, launch=mq.LAUNCH_GAUSSIAN, sigma_mm=0.1),
        mq.Physics(True, True, True, True, True, 0.133322, 300.0, 1e-7, 2000e-7, 0.0, mq.LAUNCH_LEGACY),
        mq.Physics(legacy_fields=True, legacy_force=True, **base, launch=mq.LAUNCH_GAUSSIAN),
        mq.Physics(legacy_force=True, pressure_pa=0.0, temp_k=300.0, dt=1e-7, t_max=2000e-7, launch=mq.LAUNCH_GAUSSIAN,
                   rf_phase0=False),
    ]
    jobs = [mq.Job(mq.Species(mz, 1.0, 2.95 * mz ** (2 / 3)), mq.RfAc(100.0, 500e3, 0.5, 100e3 + 1e3 * k), 256, 30 + k)
            for k, mz in enumerate((493.0, 499.0, 505.0))]
    for prec in (mq.PREC_F64, mq.PREC_MIXED):
        with mq.Engine(f, prec) as e:
            for ph in variants:
                e.run_batch(jobs, dc, ph)
            # states that sit on the box faces, outside it, or are NaN: they must end without a
            # gather out of range
            e.set_dc(dc)
            ions = e.inject(jobs, variants[1])
            k = len(ions)
            lim = np.array([(f.nx - 1) * f.h, (f.ny - 1) * f.h, (f.nz - 1) * f.h])
            ions.x[: k // 4] = lim[0]
            ions.y[k // 4: k // 2] = 0.0
            ions.z[k // 2: k // 2 + 16] = lim[2] + 1e-3
            ions.x[k - 32:] = np.nan
            ions.vz[k - 64: k - 32] = np.nan
            e.run_ions(jobs, variants[1], ions)
    out["channel"] = status(reset=1)

    s14 = mq.Fields.build(mq.Geom.s14(h_mm=0.4, n_xy=40), cache=False)
    pg = mq.PortGrid.from_fields(s14)
    for prec in (0, 1):
        m = mq.TandemModel(mq.DEFAULT_TONES, n=512, seed=486, mouth_start=True, channel=s14, cube_h=2.0,
                           port_grids=[pg] + [pg.replica() for _ in range(8)], precision=prec)
        for _ in range(4):
            m.advance(500)
        m.close()
    out["tandem"] = status(reset=1)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
