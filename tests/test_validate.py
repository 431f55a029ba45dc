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


def test_chi2_survival_matches_scipy():
    stats = __import__("pytest").importorskip("scipy.stats")
    for dof in (1, 2, 3, 4, 7, 24, 36, 100):
        for x in (0.01, 0.5, 1.0, 3.0, 7.5, 20.0, 40.0, 80.0, 150.0):
            assert math.isclose(V.chi2_sf(x, dof), stats.chi2.sf(x, dof), rel_tol=1e-9, abs_tol=1e-12), (dof, x)
    assert V.chi2_sf(3.0, 0) == 1.0


def test_class_comparison_is_the_contingency_chi2():
    stats = __import__("pytest").importorskip("scipy.stats")
    a = {"crashed": 400, "returned": 300, "transmitted": 250, "left": 50, "timeout": 0}
    b = {"crashed": 420, "returned": 280, "transmitted": 240, "left": 60, "timeout": 0}
    r = V.compare_classes(a, b)
    c = stats.chi2_contingency([[400, 300, 250, 50], [420, 280, 240, 60]], correction=False)
    assert math.isclose(r["chi2"], c[0], rel_tol=1e-12) and r["dof"] == 3 and math.isclose(r["p"], c[1], rel_tol=1e-9)
    p = 820 / 2000
    assert math.isclose(r["classes"]["crashed"]["pull"], (0.4 - 0.42) / math.sqrt(p * (1 - p) * 2 / 1000))
    assert "timeout" not in r["classes"]
    # identical tables: chi2 0, p 1; one class only: no degrees of freedom
    assert V.compare_classes(a, a)["p"] == 1.0
    assert V.compare_classes({"crashed": 5}, {"crashed": 5})["dof"] == 0
    j = V.compare_jobs([a, a], [b, a])
    assert math.isclose(j["chi2"], r["chi2"]) and j["dof"] == 6


def test_paired_comparison_is_bowkers_symmetry_test():
    import numpy as np
    a = np.array([1, 1, 2, 2, 2, 3, 3, 1, 2, 3])
    b = np.array([1, 2, 2, 1, 1, 3, 2, 1, 2, 3])
    r = V.compare_paired(a, b)
    # off-diagonal pairs: (1,2): n12 = 1, n21 = 2; (2,3): n23 = 0, n32 = 1
    assert math.isclose(r["bowker"], (1 - 2) ** 2 / 3 + (0 - 1) ** 2 / 1) and r["dof"] == 2
    assert math.isclose(r["agree"], 0.6)
    assert V.compare_paired(a, a)["p"] == 1.0 and V.compare_paired(a, a)["dof"] == 0
