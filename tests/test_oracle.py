"""The CPU oracle itself: deterministic math, reproducibility of the committed fixtures on
this host, and the summary semantics of chsim ``summarize``."""
import ctypes as C
import math
from pathlib import Path

import numpy as np
import pytest

FIX = Path(__file__).parent / "golden" / "oracle_coarse.npz"


def test_log_within_two_ulp(built):
    from oracle import mqref as R
    L = R.lib()
    rng = np.random.default_rng(3)
    xs = np.concatenate([rng.random(20000), 10 ** rng.uniform(-300, 0, 20000), [1.0, 0.5, 1e-300, 1e-7, 2 ** -24]])
    worst = max(abs(L.mqr_log(float(x)) - math.log(x)) / math.ulp(math.log(x)) if x != 1.0 else abs(L.mqr_log(1.0))
                for x in xs)
    assert worst <= 2.0


def test_sincos2pi_accuracy(built):
    from oracle import mqref as R
    L = R.lib()
    s, c = C.c_double(), C.c_double()
    rng = np.random.default_rng(4)
    for u in np.concatenate([rng.random(20000), [0.0, 0.25, 0.5, 0.75, 0.125, 1 - 2 ** -53]]):
        L.mqr_sincos2pi(float(u), C.byref(s), C.byref(c))
        assert abs(s.value - math.sin(2 * math.pi * u)) <= 1e-15
        assert abs(c.value - math.cos(2 * math.pi * u)) <= 1e-15
    L.mqr_sincos2pi(0.25, C.byref(s), C.byref(c))
    assert s.value == 1.0 and c.value == 0.0


def test_splitmix_reference_value(built):
    from oracle import mqref as R
    # SplitMix64 of 0 (Steele, Lea, Flood 2014 / world.rs:397-402)
    assert R.lib().mqr_splitmix(0) == 0xE220A8397B1DCDAF


def test_coarse_fixture_reproduces_bitwise(built):
    """The oracle's final states on the 0.4 mm grid equal the committed fixture on this host."""
    import multiq_workbench_gb300 as mq
    from oracle import mqref as R
    fx = np.load(FIX)
    g = mq.Geom.with_spacing(0.4)
    f = mq.Fields.build(g, cache=False)
    drive = [mq.RfAc(100.0, 500e3, 0.5, 100e3 + 1e3 * k) for k in range(3)]
    variants = {
        "half_kick_gauss": (mq.Physics(legacy_force=True, pressure_pa=0.133322, dt=1e-7, t_max=3000e-7,
                                       launch=mq.LAUNCH_GAUSSIAN, sigma_mm=0.1), False, [0.0, 5.0, -5.0, 0.0]),
        "legacy_all": (mq.Physics(True, True, True, True, True, 0.133322, 300.0, 1e-7, 3000e-7, 0.0, mq.LAUNCH_LEGACY), True,
                       [0.0, 5.0, -5.0, 0.0]),
        "s14_like": (mq.Physics(pressure_pa=0.1, dt=4e-8, t_max=4000 * 4e-8, launch=mq.LAUNCH_DISC), False,
                     [18.0, 24.0, 15.0, 20.0]),
    }
    for name, (ph, legsp, dc) in variants.items():
        jobs = []
        for k, mz in enumerate((493.0, 499.0, 505.0)):
            sp = mq.Species(mz * 5, 5.0, 0.0) if legsp else mq.Species(mz, 1.0, 2.95 * mz ** (2 / 3))
            jobs.append(mq.Job(sp, drive[k], 64, 1000 + k))
        G = R.Grid3(f.nx, f.ny, f.nz, f.h, f.rf, f.ac, f.dc_field(dc))
        b = R.batch(ph, 100.0, 500e3, g.axis(), g.layers())
        s = R.inject(b, jobs, 192)
        R.run(G, b, jobs, s)
        for k, _ in R.FIELDS:
            a, ref = getattr(s, k), fx[f"{name}.{k}"]
            assert np.array_equal(a.view(np.uint8), ref.view(np.uint8)), (name, k)


def test_summarize_counts_and_means(built):
    from oracle import mqref as R
    s = R.State(6)
    s.status[:] = [1, 2, 3, 4, 5, 0]
    s.jid[:] = [0, 0, 0, 1, 1, 1]
    s.ncoll[:] = [1, 2, 3, 4, 5, 6]
    s.steps[:] = [10, 20, 30, 40, 50, 60]

    class P:
        pass
    b = R.Batch()
    b.dt = 1e-7
    out = R.summarize(s, b, 2)
    assert (out[0]["crashed"], out[0]["returned"], out[0]["transmitted"]) == (1, 1, 1)
    assert (out[1]["left"], out[1]["timeout"], out[1]["n"]) == (1, 2, 3)   # status 0 counts as timeout (channel.rs:501)
    assert out[0]["mean_coll"] == 2.0 and math.isclose(out[1]["mean_time"], 50 * 1e-7)


def _rows(c):
    """Outcome fractions with binomial errors and T/(T+C), as simulation/mqviz/src/validate.rs:119-126 tabulates them."""
    n = max(c["n"], 1)
    out = {}
    for k in ("transmitted", "crashed", "returned"):
        p = c[k] / n
        out[k] = (p, math.sqrt(p * (1 - p) / n))
    m = max(c["transmitted"] + c["crashed"], 1)
    p = c["transmitted"] / m
    out["T/(T+C)"] = (p, math.sqrt(p * (1 - p) / m))
    return out


@pytest.mark.parametrize("rf0", [True, False])
def test_independent_form_agrees_with_table_form(s14_coarse, rf0):
    """The independent per-ion FP64 loop (validate.rs:49-94: own seeding, own time accumulator, a
    trilinear pass per field, inline collisions) and the table-driven integrator give the same
    outcome fractions within the reference's own bar, |pull| <= 2 on every row (validate.rs:128-135),
    on the coarse S14 grid at an excited point with crashes, 8000 ions each, t_max 3 ms."""
    import multiq_workbench_gb300 as mq
    from oracle import mqref as R
    f = s14_coarse
    g = mq.Geom.s14(h_mm=0.4, n_xy=40)
    lay = g.layers()
    dc = [18.0, 24.0, 15.0, 20.0]
    sp = mq.Species(499.0 * 5, 5.0, 2.95 * 499 ** (2 / 3) * 3)
    G = R.Grid3(f.nx, f.ny, f.nz, f.h, f.rf, f.ac, f.dc_field(dc))
    n, tmax = 8000, 3e-3
    ind = R.run_independent(G, sp, 70.0, 500e3, 3.0, 84.25e3, 0.1, 4e-8, tmax, g.axis(), lay[4] * 1e-3, 0.5e-3, n,
                            777, rf_phase0=rf0)
    ph = mq.Physics(pressure_pa=0.1, dt=4e-8, t_max=tmax, launch=mq.LAUNCH_DISC, r_inject_mm=2.0, rf_phase0=rf0)
    b = R.batch(ph, 70.0, 500e3, g.axis(), lay)
    jobs = [mq.Job(sp, mq.RfAc(70.0, 500e3, 3.0, 84.25e3), n, 777)]
    s = R.inject(b, jobs, n)
    R.run(G, b, jobs, s)
    o = R.summarize(s, b, 1)[0]
    tab = dict(n=o["n"], transmitted=o["transmitted"], crashed=o["crashed"] + o["left"], returned=o["returned"])
    assert ind["n"] == n and ind["crashed"] > 50 and ind["transmitted"] > 50
    assert ind["transmitted"] + ind["crashed"] + ind["returned"] + ind["timeout"] == n
    a, r = _rows(ind), _rows(tab)
    for k in a:
        pull = (a[k][0] - r[k][0]) / max(math.hypot(a[k][1], r[k][1]), 1e-300)
        assert abs(pull) <= 2.0, (k, a[k], r[k], pull)
