"""The chsim command line on the CPU: FWHM by interpolation (channel.rs:511-520), the r0 fit of the
RF basis near the axis on an exact quadrupole potential, the trajectory secular frequency against
the Mathieu exponent in an exact quadrupole field, the on-axis DC profile, and the diagnostics of
the default channel."""
import io
import math
from types import SimpleNamespace as NS

import numpy as np

import multiq_workbench_gb300 as mq
from multiq_workbench_gb300 import chsim as CH
from multiq_workbench_gb300 import fit as F


def test_fwhm():
    xs = [0.0, 1.0, 2.0, 3.0, 4.0]
    ys = [0.0, 0.5, 1.0, 0.5, 0.0]
    assert CH.fwhm(xs, ys) == (2.0, 1.0, 2.0)
    pk, py, w = CH.fwhm([1.0, 2.0, 3.0], [0.2, 0.9, 0.1])
    lo = 1.0 + (0.45 - 0.2) / (0.9 - 0.2)
    hi = 2.0 + (0.9 - 0.45) / (0.9 - 0.1)
    assert (pk, py) == (2.0, 0.9) and math.isclose(w, hi - lo)


def _quad(h_mm=0.1, n=101, nz=5, r0_mm=2.0):
    """An exact quadrupole: phi = -2 X Y / r0^2 per volt about the axis, E = -grad phi."""
    h = h_mm * 1e-3
    a = (n // 2) * h
    r0 = r0_mm * 1e-3
    i = np.arange(n) * h - a
    X, Y = np.meshgrid(i, i, indexing="xy")        # X varies along the last (x) index
    rf = np.zeros((nz, n, n, 4), np.float32)
    rf[..., 0] = (2.0 * Y / r0 ** 2)[None]
    rf[..., 1] = (2.0 * X / r0 ** 2)[None]
    phi = (-2.0 * X * Y / r0 ** 2)
    w = 5
    c = n // 2
    near = np.repeat(phi[None, c - w:c + w + 1, c - w:c + w + 1], nz, axis=0)
    geom = NS(h_mm=h_mm, axis=lambda: a * 1e3)
    return NS(rf=rf.reshape(-1, 4), nx=n, ny=n, nz=nz, h=h, geom=geom, rf_phi_near=near), r0


def test_r0_fit_on_an_exact_quadrupole(built):
    f, r0 = _quad()
    assert math.isclose(CH.r0_fit(f, 0.2, 5), r0 * 1e3, rel_tol=1e-9)


def test_secular_frequency_follows_the_mathieu_exponent(built):
    f, r0 = _quad()
    sp = mq.Species(500.0, 1.0, 0.0)
    qm = sp.z * CH.QE / (sp.mass * CH.AMU)
    om = 2 * math.pi * 500e3
    v = 0.3 * om * om * r0 ** 2 / (4.0 * qm)           # q = 4 qm V / (Omega^2 r0^2) = 0.3
    got = CH.secular_freq(f, sp, v, 500e3, 0.2, False)
    want = F.mathieu_beta(0.0, 0.3) * 500e3 / 2.0
    assert abs(got / want - 1.0) < 0.01, (got, want)
    # half force: q halves
    got_h = CH.secular_freq(f, sp, v, 500e3, 0.2, True)
    assert abs(got_h / (F.mathieu_beta(0.0, 0.15) * 250e3) - 1.0) < 0.01
    # an unstable drive (q > 0.908) leaves the window: NaN
    assert math.isnan(CH.secular_freq(f, sp, v * 1.0 / 0.3, 500e3, 0.2, False))


def test_channel_diagnostics(built, coarse):
    out = io.StringIO()
    rows = CH.r0_profile(coarse, out)
    assert len(rows) == 7 and "RF field check" in out.getvalue()
    ax = coarse.dc_phi_axis(CH.FIG4_DC)
    assert len(ax) == coarse.nz and ax[0][0] == 0.0
    # the plate at +5 V raises the axis potential to a maximum at the plate, between the end of Q1
    # and the start of the downstream section (layers 1 and 3)
    zmax, pmax = max(ax, key=lambda t: t[1])
    lay = coarse.geom.layers()
    assert pmax > 0.1 and lay[1] - 1.0 <= zmax <= lay[3] + 1.0, (zmax, pmax, lay)
    closed, opened = CH.s14_dc(coarse, None)
    assert closed == [18.0, 24.0, 15.0, 20.0] and opened == [18.0, 19.0, 15.0, 20.0]
    jobs = CH.fig4_jobs(10)
    assert len(jobs) == 26 and jobs[0].sp.mass == 475.0 * 5 and jobs[12].seed == 1499


def test_usage_and_unavailable(capsys):
    assert CH.main([]) == 2
    assert CH.main(["compare-theirs"]) == 1
