"""Resonance fits and the secular-frequency terrain (CPU).  The fit tests restate the reference's own
(simulation/mqviz/src/fit.rs:274-381) with its generator and seeds, so the synthetic scans are the
same draws the reference's tests make; the Mathieu exponent is pinned against a direct Floquet
integration of the Mathieu equation."""
import math

import numpy as np
import pytest

from multiq_workbench_gb300 import fit as F

XS = [70.0 + i for i in range(31)]


def synth(shape, truth, rng, nper):
    """fit.rs:278-283: 31 points 70..100 kHz, nper ions each, k ~ binomial(nper, model)."""
    ps = [min(max(F.model(shape, truth, x), 0.0), 1.0) for x in XS]
    ks = rng.binomial([nper] * len(XS), ps)
    return XS, ks, [nper] * len(XS)


def test_recovers_noiseless_lorentzian_exactly(built):
    truth = [0.01, 0.2, 83.0, 9.0]
    ys = [F.model(F.LORENTZ, truth, x) for x in XS]
    f = F.fit_shape_sigma(F.LORENTZ, XS, ys, [0.01] * len(XS))
    assert f is not None
    for k in range(4):
        assert abs(f.p[k] - truth[k]) < 1e-6 * max(abs(truth[k]), 1.0), (f.p, truth)
    assert f.chi2 < 1e-9


def test_lorentzian_parameters_and_uncertainties_cover(built):
    """400 scans of 31 points x 700 ions (R = 83/9): +-1 sigma covers the truth 68 % of the time for
    every parameter and for R, and the mean bias is small against the error (fit.rs:296-320)."""
    truth = [0.01, 0.2, 83.0, 9.0]
    r_true = truth[2] / truth[3]
    rng = F.Rng(2024)
    hit = [0] * 5
    dev, err = [0.0] * 4, [0.0] * 4
    used = 0
    for _ in range(400):
        xs, ks, ns = synth(F.LORENTZ, truth, rng, 700)
        used += 1
        fl = F.fit_binomial_shape(F.LORENTZ, xs, ks, ns, 0, 1)
        if fl is None:
            continue
        for k in range(4):
            hit[k] += abs(fl.p[k] - truth[k]) <= fl.e[k]
            dev[k] += fl.p[k] - truth[k]
            err[k] += fl.e[k]
        hit[4] += abs(fl.r - r_true) <= fl.r_err
    cov = [h / used for h in hit]
    for i, c in enumerate(cov):
        assert abs(c - 0.6827) < 0.075, (i, cov)
    for k in range(4):
        assert abs(dev[k] / err[k]) < 0.25, (k, dev[k] / err[k])


def test_gaussian_is_chosen_for_gaussian_data_and_recovers_width(built):
    truth = [0.0, 0.3, 83.0, 8.0]
    rng = F.Rng(77)
    wins = w_ok = 0
    for _ in range(60):
        xs, ks, ns = synth(F.GAUSS, truth, rng, 1500)
        f = F.fit_binomial_curve(xs, ks, ns, 0, 1)
        if f.shape == F.GAUSS:
            wins += 1
            w_ok += abs(f.p[3] - truth[3]) < 4.0 * f.e[3]
    assert wins / 60 > 0.8
    assert w_ok / wins > 0.95


def test_bootstrap_error_on_r_agrees_with_covariance(built):
    truth = [0.01, 0.2, 83.0, 9.0]
    rng = F.Rng(5)
    xs, ks, ns = synth(F.LORENTZ, truth, rng, 700)
    f = F.fit_binomial_curve(xs, ks, ns, 200, 3)
    mean, sd = f.r_boot
    assert abs(sd / f.r_err - 1.0) < 0.35, (sd, f.r_err)
    assert abs(mean - f.r) < 3 * sd and f.f0_boot > 0


def test_a_flat_scan_is_not_called_a_resonance_and_a_real_one_is(built):
    rng = F.Rng(404)
    xs = [35.0 + i for i in range(31)]
    false_pos = 0
    for _ in range(300):
        ks = rng.binomial([1000] * 31, [0.004] * 31)
        f = F.fit_binomial_curve(xs, ks, [1000] * 31, 0, 1)
        if f is not None and F.is_significant(f, xs):
            false_pos += 1
    assert false_pos / 300 < 0.03, false_pos
    found = 0
    for _ in range(100):
        ps = [min(max(F.model(F.LORENTZ, [0.004, 0.04, 52.7, 1.5], x), 0.0), 1.0) for x in xs]
        ks = rng.binomial([1000] * 31, ps)
        f = F.fit_binomial_curve(xs, ks, [1000] * 31, 0, 1)
        if F.is_significant(f, xs) and abs(f.p[2] - 52.7) < 0.5:
            found += 1
    assert found >= 95, found


def test_r_in_mz_terms(built):
    mz, f0, fw = 863.5, 83.0, 9.0
    _, _, r, _ = F.r_mz(mz, -f0 / mz, fw, 0.5)
    assert abs(r - f0 / fw) < 1e-9


def test_fit_refusals(built):
    assert F.fit_binomial_curve(XS[:5], [1] * 5, [10] * 5) is None          # fewer than 6 points
    assert F.fit_binomial_curve(XS, [0] * 31, [0] * 31) is None             # no ions anywhere
    assert F.fit_shape_sigma(F.LORENTZ, XS[:4], [0.0] * 4, [1.0] * 4) is None


def _floquet_beta(a, q):
    """beta from the trace of the Mathieu monodromy matrix over one period pi:
    cos(pi beta) = (y1(pi) + y2'(pi)) / 2 for u'' + (a - 2 q cos 2t) u = 0."""
    from scipy.integrate import solve_ivp

    def rhs(t, y):
        k = a - 2.0 * q * math.cos(2.0 * t)
        return [y[1], -k * y[0], y[3], -k * y[2]]
    s = solve_ivp(rhs, (0.0, math.pi), [1.0, 0.0, 0.0, 1.0], method="DOP853", rtol=1e-12, atol=1e-13)
    tr = s.y[0, -1] + s.y[3, -1]
    return math.acos(tr / 2.0) / math.pi


@pytest.mark.parametrize("a,q", [(0.0, 0.05), (0.0, 0.3), (0.0, 0.706), (0.0, 0.85), (-0.02, 0.4), (0.05, 0.5)])
def test_mathieu_beta_matches_floquet_integration(built, a, q):
    pytest.importorskip("scipy")
    assert abs(F.mathieu_beta(a, q) - _floquet_beta(a, q)) < 1e-6


def test_secular_frequency_limits(built):
    qm = 2 * 1.602176634e-19 / (2 * 863.473 * 1.6605390666e-27)
    assert math.isnan(F.sec_freq_khz(0.0, 0.0, qm, 70.0))          # a + q^2/2 = 0: untrapped
    # an RF gradient with q = 0.3 and no DC: f = beta(0, 0.3) * f_rf / 2
    om = 2 * math.pi * 500e3
    g = 0.3 * om * om / (2 * qm * 70.0)
    assert abs(F.sec_freq_khz(g, 0.0, qm, 70.0) - F.mathieu_beta(0.0, 0.3) * 250.0) < 1e-9
    g_hi = 0.96 * om * om / (2 * qm * 70.0)
    assert math.isnan(F.sec_freq_khz(g_hi, 0.0, qm, 70.0))         # q > 0.95


def test_terrain_along_the_channel(built, s14_coarse):
    """The S14 channel's secular-frequency terrain: trapped along the body, a plateau near the
    calibrated excitation frequency, lighter ions higher, and d f / d(m/z) close to -f / (m/z)
    (the pure-RF scaling, which the DC gradients perturb)."""
    from types import SimpleNamespace as NS
    T = F.TerrainTables(s14_coarse)
    assert T.n > 150 and abs(T.z_mm[0] - 0.3) < 1e-12 and T.z_mm[T.n - 1] < 20.0
    sp = [NS(mass=2 * 863.473, z=2.0), NS(mass=2 * 874.466, z=2.0)]
    dc = [18.0, 24.0, 15.0, 20.0]
    t = T.compute(sp, 70.0, dc)
    p0, p1 = t.plateau(0), t.plateau(1)
    assert 70.0 < p0 < 100.0 and p1 < p0
    body = (t.z_mm > 4.0) & (t.z_mm < 12.0)
    assert np.all(np.isfinite(t.fx[0][body])) and np.all(np.isfinite(t.fy[0][body]))
    s = T.dfdmz(sp[0], 70.0, dc)
    assert s < 0 and abs(s / (-p0 / 863.473) - 1.0) < 0.25
    assert t.nearest(p1 - 0.01) == 1 and t.nearest(p0 + 5) == 0
    z = F.Terrain.crossings(t.z_mm, t.fx[0], 0.5 * p0)
    assert len(z) >= 1 and all(0.3 <= c <= 20.0 for c in z)
