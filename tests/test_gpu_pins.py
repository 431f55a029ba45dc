"""The device engines at the reference's published S14 point (simulation/mqviz/src/validate.rs:97-112:
chsim's GPU counts for 100,000 ions, seed 4242, Physics::correct(0.1), t_max 3 ms, the calibrated S14
channel and drive): the FP64 kernel reproduces the oracle's committed counts exactly (it is
bit-exact with the oracle on the same grid, and the grid solved on the GPU is bit-identical to the
host's); both engines meet the reference's own bar against chsim's counts (|pull| <= 2 on its rows
T, C, R and T/(T+C), validate.rs:119-135), and the mixed engine, an independent random stream,
agrees with the FP64 kernel at the 95% level (one chi-square over the four outcome classes)."""
import json
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

PINS = json.loads((Path(__file__).parent / "golden" / "pins.json").read_text())


def _as_rows(c):
    return {"transmitted": c.trans, "crashed_or_left": c.crash, "returned": c.ret, "timeout": c.timeout}


def test_s14_point_on_the_device(built):
    import multiq_workbench_gb300 as mq
    from multiq_workbench_gb300 import validate as V
    s = PINS["s14_chsim_gpu"]
    assert V.REF_CHSIM_GPU == (s["n"], s["transmitted"], s["crashed_or_left"], s["returned"], s["timeout"])
    f = V.s14_fields(device=0)
    with mq.Engine(f, mq.PREC_F64) as e:
        c64 = V.run_engine(e, s["n"], 4242, rf_phase0=True)
    assert _as_rows(c64) == {k: s["oracle"][k] for k in _as_rows(c64)}, (c64, s["oracle"])
    with mq.Engine(f, mq.PREC_MIXED) as e:
        cm = V.run_engine(e, s["n"], 4242, rf_phase0=True)
    metal = V.embedded_metal()
    # the reference's own rows and bar: T, C, R and T/(T+C), |pull| <= 2 (validate.rs:119-135)
    for c in (c64, cm):
        for row in V.rows(c, metal):
            assert abs(row.pull()) <= 2.0, (row.name, row.live, row.refv, row.pull())
    # the mixed engine (an independent random stream) against the FP64 kernel at the 95% level: one
    # chi-square over the four classes (transmitted, crashed or left, returned, timeout), p >= 0.05
    r = V.compare_classes({"t": cm.trans, "c": cm.crash, "r": cm.ret, "to": cm.timeout},
                          {"t": c64.trans, "c": c64.crash, "r": c64.ret, "to": c64.timeout})
    print(f"PARITY S14 point: FP64 T {c64.trans} C+L {c64.crash} R {c64.ret} TO {c64.timeout}; mixed T {cm.trans} "
          f"C+L {cm.crash} R {cm.ret} TO {cm.timeout}; mixed vs FP64 chi2 {r['chi2']:.2f} dof {r['dof']} p {r['p']:.3f}; "
          "pulls vs chsim (T, C, R, T/(T+C)): FP64 "
          + " ".join(f"{row.pull():+.2f}" for row in V.rows(c64, metal)) + ", mixed "
          + " ".join(f"{row.pull():+.2f}" for row in V.rows(cm, metal)))
    assert r["p"] >= 0.05, r
