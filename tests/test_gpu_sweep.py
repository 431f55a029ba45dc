"""Sweeps on the device: every cohort of a frequency sweep runs as one batch, and the resonance fit
turns the counts into R.  The FP64 engine's sweep counts equal the CPU oracle's exactly; the mixed
engine's fitted resonance (f0, FWHM, R) agrees with the FP64 engine's within 3 combined sigma."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


class OracleEngine:
    """run_batch over the CPU oracle."""

    def __init__(self, f):
        self.f = f

    def run_batch(self, jobs, dc, ph):
        import multiq_workbench_gb300 as mq
        from oracle import mqref as R
        f, g = self.f, self.f.geom
        G = R.Grid3(f.nx, f.ny, f.nz, f.h, f.rf, f.ac, f.dc_field(dc))
        b = R.batch(ph, jobs[0].drive.v_rf, jobs[0].drive.f_rf, g.axis(), g.layers())
        s = R.inject(b, jobs, sum(j.n for j in jobs))
        R.run(G, b, jobs, s)
        return [mq.Outcome(**o) for o in R.summarize(s, b, len(jobs))]


def test_fp64_sweep_counts_equal_the_oracle(s14_coarse):
    import multiq_workbench_gb300 as mq
    from multiq_workbench_gb300 import sweep as W
    pre = W.SweepPreset.s14()
    cfg = W.SweepCfg(78.0, 92.0, 2.0, ions_per_point=200)
    ph = W.sweep_physics(pre.pressure_pa)
    with mq.Engine(s14_coarse, precision=mq.PREC_F64) as eng:
        dev = W.run_sweep(eng, pre.species, cfg, pre.v_rf, pre.v_ac, pre.dc(), ph, seed=31)
    ref = W.run_sweep(OracleEngine(s14_coarse), pre.species, cfg, pre.v_rf, pre.v_ac, pre.dc(), ph, seed=31)
    assert dev.counts.shape == (8, 2, 4)
    assert np.array_equal(dev.counts, ref.counts)


def test_mixed_sweep_fit_agrees_with_fp64(s14_coarse):
    import multiq_workbench_gb300 as mq
    from multiq_workbench_gb300 import fit as F
    from multiq_workbench_gb300 import sweep as W
    pre = W.SweepPreset.s14()
    cfg = W.SweepCfg(*pre.sweep, ions_per_point=2000)
    ph = W.sweep_physics(pre.pressure_pa)
    T = F.TerrainTables(s14_coarse)
    fits = {}
    for prec in (mq.PREC_MIXED, mq.PREC_F64):
        with mq.Engine(s14_coarse, precision=prec) as eng:
            sv = W.run_sweep(eng, pre.species, cfg, pre.v_rf, pre.v_ac, pre.dc(), ph, seed=5)
        assert sv.counts.sum() == 31 * 2000
        fits[prec] = W.fit_sweep(sv, pre.species, T, pre.v_rf, pre.dc(), boot=0, seed=1)
    a, b = fits[mq.PREC_MIXED][0], fits[mq.PREC_F64][0]
    assert a is not None and b is not None
    assert 70.0 < a.fit.p[2] < 100.0 and a.dfdmz < 0
    for k in (2, 3):                          # f0, FWHM
        pull = (a.fit.p[k] - b.fit.p[k]) / math.hypot(a.fit.e[k], b.fit.e[k])
        assert abs(pull) <= 3.0, (k, a.fit.p[k], b.fit.p[k], pull)
    pull_r = (a.r_f[0] - b.r_f[0]) / math.hypot(a.r_f[1], b.r_f[1])
    assert abs(pull_r) <= 3.0, (a.r_f, b.r_f)
