"""The validation tables of simulation/mqviz/src/validate.rs:13-21,114-135 on the CPU: binomial
errors, T/(T+C) and its error, pulls with errors in quadrature, the 'ok' / 'DIFF' mark."""
import math

from multiq_workbench_gb300 import validate as V


def test_counts_and_rows():
    a = V.Counts(1000, 200, 50, 700, 50)
    assert a.frac(a.trans) == 0.2 and math.isclose(a.se(a.trans), math.sqrt(0.2 * 0.8 / 1000))
    assert math.isclose(a.t_over_tc(), 0.8) and math.isclose(a.se_eff(), math.sqrt(0.8 * 0.2 / 250))
    r = V.rows(a, a)
    assert [x.name for x in r] == ["transmitted", "crashed", "returned", "T/(T+C)"]
    assert all(x.pull() == 0.0 for x in r)
    b = V.Counts(1000, 260, 50, 640, 50)
    p = V.rows(b, a)[0].pull()
    assert math.isclose(p, (0.26 - 0.2) / math.sqrt(0.26 * 0.74 / 1000 + 0.2 * 0.8 / 1000))
    t = V.table("t", "b", "a", b, a)
    assert "DIFF" in t.splitlines()[2] and t.splitlines()[3].endswith("ok")


def test_embedded_reference_counts_and_point():
    m = V.embedded_metal()
    assert (m.n, m.trans, m.crash, m.ret, m.timeout) == (100_000, 19_669, 3_412, 75_797, 1_122)
    assert m.trans + m.crash + m.ret + m.timeout == m.n
    ph = V.point_physics(True)
    assert ph.t_max == 3e-3 and ph.pressure_pa == 0.1 and ph.rf_phase0
    assert not V.point_physics(False).rf_phase0
