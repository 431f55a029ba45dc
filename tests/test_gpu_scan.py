"""Scan drivers and self-checks on the GPU: a batch gives every ion bit for bit the state it gets
when its job runs alone (chsim check.rs:25-38), for both engines; the result cache serves a
repeated scan without running it."""
import pytest

import multiq_workbench_gb300 as mq
from multiq_workbench_gb300 import check, scan

pytestmark = pytest.mark.gpu


def _jobs(n=40):
    drive = mq.RfAc(100.0, 500e3, 0.5, 100e3)
    return [mq.Job(mq.Species(mz * 5.0, 5.0, 0.0), drive, n, 1000 + int(mz)) for mz in (491.0, 499.0, 507.0)] + \
           [mq.Job(mq.Species(mz, 1.0, 2.95 * mz ** (2 / 3)), mq.RfAc(100.0, 500e3, 0.5, f), n, 7 + k)
            for k, (mz, f) in enumerate(((495.0, 99e3), (501.0, 101e3)))]


@pytest.mark.parametrize("prec", [mq.PREC_F64, mq.PREC_MIXED])
def test_batch_equals_jobs_run_alone(coarse, prec):
    ph = mq.Physics.legacy(0.133322)
    ph.t_max = 3000 * ph.dt
    with mq.Engine(coarse, prec) as e:
        d = check.check_case(e, _jobs(), [0.0, 5.0, -5.0, 0.0], ph)
    assert d["differ"] == 0, d


def test_thermal_gas_batch_equals_jobs_run_alone(coarse):
    ph = mq.Physics(legacy_force=True, pressure_pa=0.133322, dt=1e-7, t_max=3000e-7, launch=mq.LAUNCH_GAUSSIAN)
    with mq.Engine(coarse, mq.PREC_MIXED) as e:
        d = check.check_case(e, _jobs(), [0.0, 5.0, -5.0, 0.0], ph)
    assert d["differ"] == 0, d


def test_cached_scan_reruns_nothing(coarse, tmp_path):
    ph = mq.Physics.legacy(0.133322)
    ph.t_max = 2000 * ph.dt
    path = tmp_path / "results.tsv"
    with mq.Engine(coarse, mq.PREC_MIXED) as e:
        a = scan.adaptive_scan(e, coarse.geom, mq.Species(2495.0, 5.0, 0.0), mq.RfAc(100.0, 500e3, 0.5, 0.0),
                               [0.0, 5.0, -5.0, 0.0], ph, 90.0, 110.0, 5.0, 64, 128, 0.0, 1, path, log=False)
        n_lines = len(path.read_text().splitlines())
        b = scan.adaptive_scan(e, coarse.geom, mq.Species(2495.0, 5.0, 0.0), mq.RfAc(100.0, 500e3, 0.5, 0.0),
                               [0.0, 5.0, -5.0, 0.0], ph, 90.0, 110.0, 5.0, 64, 128, 0.0, 1, path, log=False)
    assert a == b and len(path.read_text().splitlines()) == n_lines
    assert len(a) >= 5
