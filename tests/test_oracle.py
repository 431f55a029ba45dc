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
