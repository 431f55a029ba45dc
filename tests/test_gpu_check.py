"""The bounds-checked debug build (-DMQ_CHECK): its self-test records the one index it plants at
its limit (no memory is touched), and every stepping kernel, run over the physics switches, over
states on and outside the box faces or NaN, and through the tandem with nine port grids, computes
no gather or work-queue index out of range."""
import json
import os
import subprocess
import sys
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

HERE = Path(__file__).resolve().parent


def test_check_build_finds_no_out_of_range_index(built):
    from multiq_workbench_gb300 import build as B
    lib = B.build(check=True)
    env = dict(os.environ, MQ_LIB=str(lib))
    r = subprocess.run([sys.executable, str(HERE / "check_workloads.py")], env=env, capture_output=True, text=True,
                       timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    rec = json.loads(r.stdout.strip().splitlines()[-1])
    st = rec["selftest"]
    assert st["rc"] == 0 and st["enabled"] == 1 and st["hits"] == 1 and st["site"] == 99
    assert st["index"] == 7 and st["limit"] == 7
    for part in ("channel", "tandem"):
        assert rec[part]["enabled"] == 1 and rec[part]["hits"] == 0, (part, rec[part])


def test_normal_build_reports_checks_off(built):
    import ctypes as C
    from multiq_workbench_gb300 import _native as N
    en, hits, site = C.c_int32(), C.c_uint32(), C.c_uint32()
    idx, lim = C.c_uint64(), C.c_uint64()
    assert N.lib().mq_check_selftest(0) == 0
    assert N.lib().mq_check_status(0, 1, C.byref(en), C.byref(hits), C.byref(site), C.byref(idx), C.byref(lim)) == 0
    assert en.value == 0 and hits.value == 0
