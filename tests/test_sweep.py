"""Sweep driver on the CPU: frequency grid and cohort split as the reference's sweep builds them
(simulation/mqviz/src/engine.rs:420-431), one batch for all cohorts, and the per-species fit
pipeline of analysis.rs:37-58, driven by a stand-in engine with a known resonance."""
import math

import numpy as np

import multiq_workbench_gb300 as mq
from multiq_workbench_gb300 import fit as F
from multiq_workbench_gb300 import sweep as W


def test_frequency_grid_and_apportioning():
    assert W.SweepCfg(70.0, 100.0, 1.0).freqs() == [70.0 + i for i in range(31)]
    assert len(W.SweepCfg(0.0, 500.0, 1.0).freqs()) == 101          # capped at 101 points
    assert W.SweepCfg(83.0, 83.0, 0.5).freqs() == [83.0]
    # the point count is round((hi - lo) / step), half away from zero, so a grid may end past hi
    assert len(W.SweepCfg(70.0, 71.0, 0.4).freqs()) == 4
    assert W.SweepCfg(80.0, 70.0, 1.0).freqs() == [80.0]
    assert W.apportion(2000, [0.95, 0.05]) == [1900, 100]
    fig5 = W.SweepPreset.fig5()
    n = W.apportion(1000, [s.weight for s in fig5.species])
    assert sum(n) == 1000 and n[2] == max(n)
    assert W.apportion(0, [1, 2]) == [0, 0]


class FakeEngine:
    """run_batch stand-in: transmission is a Lorentzian in f_ac per charge state, drawn binomially."""

    def __init__(self, f0_by_z, width=3.0, peak=0.3, base=0.01):
        self.calls = []
        self.f0, self.w, self.peak, self.base = f0_by_z, width, peak, base
        self.rng = F.Rng(11)

    def run_batch(self, jobs, dc, ph):
        self.calls.append(list(jobs))
        out = []
        for j in jobs:
            f = j.drive.f_ac / 1e3
            p = F.model(F.LORENTZ, [self.base, self.peak, self.f0[int(j.sp.z)], self.w], f)
            t = int(self.rng.binomial([j.n], [p])[0])
            c = (j.n - t) // 3
            out.append(mq.Outcome(j.n, c - 5, j.n - t - c, t, 5, 0, 1.0, 1e-4))
        return out


def test_run_sweep_and_fit_pipeline():
    pre = W.SweepPreset.fig5()
    f0 = {6: 40.0, 7: 46.0, 8: 52.7, 9: 58.0, 10: 63.0}
    eng = FakeEngine(f0)
    cfg = W.SweepCfg(*pre.sweep, ions_per_point=4000)
    sv = W.run_sweep(eng, pre.species, cfg, pre.v_rf, pre.v_ac, pre.dc(), W.sweep_physics(pre.pressure_pa), seed=100)
    assert len(eng.calls) == 1                                    # every cohort in one batch
    jobs = eng.calls[0]
    assert len(jobs) == 31 * 5 and all(j.drive.v_rf == 56.0 and j.drive.v_ac == 0.2 for j in jobs)
    assert [j.seed for j in jobs[:6]] == [100, 101, 102, 103, 104, 105]
    assert sv.counts.shape == (31, 5, 4) and np.all(sv.counts.sum(axis=2) == np.array(
        [W.apportion(4000, [s.weight for s in pre.species])] * 31))
    k, n = sv.frac(0, 2)
    assert n == sv.counts[0, 2].sum() and k == sv.counts[0, 2, 0]
    # slopes given directly: f ~ 1/(m/z) gives d f / d(m/z) = -f0 / (m/z)
    slopes = [-f0[int(s.z)] / s.mz() for s in pre.species]
    fits = W.fit_sweep(sv, pre.species, None, pre.v_rf, pre.dc(), boot=50, seed=7, dfdmz=slopes)
    for s, sp in enumerate(pre.species):
        ft = fits[s]
        assert ft is not None, sp.label
        assert abs(ft.fit.p[2] - f0[int(sp.z)]) < 4 * ft.fit.e[2] + 1e-9
        # with the slope -f / (m/z) of a pure 1/(m/z) mapping, R in m/z is f / FWHM at that f
        assert abs(ft.r_mz[0] - f0[int(sp.z)] / ft.fit.p[3]) < 1e-9 * ft.r_mz[0]
        assert ft.min_ions == W.apportion(4000, [x.weight for x in pre.species])[s]
    csv = W.sweep_csv(sv)
    assert csv.splitlines()[0].startswith("f_khz,6+:T,6+:C") and len(csv.splitlines()) == 32


def test_flat_species_is_skipped():
    pre = W.SweepPreset.custom()
    eng = FakeEngine({2: 84.0}, peak=0.0, base=0.001)
    sv = W.run_sweep(eng, pre.species, W.SweepCfg(70.0, 100.0, 1.0, 500), 70.0, 0.35, pre.dc(), W.sweep_physics(0.1))
    assert W.fit_sweep(sv, pre.species, None, 70.0, pre.dc(), dfdmz=[-0.1]) == [None]
