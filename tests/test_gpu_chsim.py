"""The chsim command line on the device: the legacy Fig. 4 scan (config 1: 26 m/z x 1000 ions in one
batch) on the FP64 kernel reproduces the oracle's committed per-m/z counts exactly, and on the
mixed engine peaks at the same m/z with the same width; check-tiled finds no ion that differs from
its job run alone; the S14 scan and the hash command run end to end."""
import json
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PINS = json.loads((Path(__file__).parent / "golden" / "pins.json").read_text())


@pytest.fixture(scope="module")
def channel_0p1(built):
    import multiq_workbench_gb300 as mq
    return mq.Fields.build(mq.Geom(), cache=False, device=0)


def test_legacy_fig4_on_both_engines(channel_0p1):
    import multiq_workbench_gb300 as mq
    from multiq_workbench_gb300 import chsim as CH
    ms = PINS["mass_scan"]
    assert [j.sp.mass / 5.0 for j in CH.fig4_jobs(1)][:len(ms["mz"])] == [float(m) for m in ms["mz"]]
    ph = mq.Physics.legacy(1e-3 * 133.322)
    jobs = CH.fig4_jobs(ms["ions_per_mass"])
    with mq.Engine(channel_0p1, mq.PREC_F64) as e:
        out = e.run_batch(jobs, CH.FIG4_DC, ph)
    assert [int(o.transmitted) for o in out][:len(ms["mz"])] == ms["oracle_legacy"]
    with mq.Engine(channel_0p1, mq.PREC_MIXED) as e:
        pk, py, w = CH.cmd_legacy_fig4(e, ms["ions_per_mass"])
    ys = [t / ms["ions_per_mass"] for t in ms["oracle_legacy"]]
    pk0, py0, w0 = CH.fwhm([float(m) for m in ms["mz"]], ys)
    assert abs(pk - pk0) <= 2.0 and abs(w - w0) <= 2.0 and abs(py - py0) < 0.06, ((pk, py, w), (pk0, py0, w0))


def test_check_tiled_and_hash_and_s14(built, capsys):
    from multiq_workbench_gb300 import chsim as CH
    assert CH.cmd_check_tiled(40, False, 0) == 0
    h1 = CH.cmd_hash(40, False, 0)
    h2 = CH.cmd_hash(40, False, 0)
    assert len(h1) == 9 and h1 == h2
    pk, py, w = CH.cmd_s14(["s14", "0.1", "200"], False, 0)
    assert 70.0 <= pk <= 110.0 and np.isfinite(w)
    text = capsys.readouterr().out
    assert "check-tiled: PASS" in text and "resonance: peak" in text
