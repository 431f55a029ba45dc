"""The mixed engines' thermal-collision sampler against the reference's, as algorithms (numpy, CPU).

The reference (simulation/mqviz/src/world.rs:473-488) draws null-collision candidates at the rate
n sigma (|v| + 6 s) per unit time, the gas partner V from the Maxwellian f (per-component spread s)
and accepts with |v - V| / (|v| + 6 s). The mixed engines (mqx::thermal_partner in
csrc/mq_mixmath.h) draw candidates at n sigma (|v| + E|V|), E|V| = 2 sqrt(2/pi) s, the partner from
the mixture q(V) = f(V) (|v| + |V|) / (|v| + E|V|) (the Maxwellian with probability
|v| / (|v| + E|V|), else the speed-weighted Maxwellian whose speed r has r^2 / 2 s^2 ~ Gamma(2, 1)),
and accept with |v - V| / (|v| + |V|). Both must give the collision rate n sigma E|v - V| and the
same distribution of the partner among accepted candidates; this restates both in numpy and
compares them by Monte Carlo at three ion speeds. (The device sampler itself is held to the FP64
kernel, which uses the reference's sampler, by the 95% gates of the GPU tests.)
"""
import numpy as np

N = 400_000
E_V = 2.0 * np.sqrt(2.0 / np.pi)   # E|V| / s for a 3-D Maxwellian


def _reference(rng, v, s):
    vm = np.linalg.norm(v)
    V = rng.normal(0.0, s, (N, 3))
    g = np.linalg.norm(v - V, axis=1)
    acc = rng.random(N) * (vm + 6.0 * s) < g
    return (vm + 6.0 * s) * acc.mean(), V[acc], acc.mean()


def _majorant(rng, v, s):
    vm = np.linalg.norm(v)
    ev = E_V * s
    from_f = rng.random(N) * (vm + ev) < vm
    Vf = rng.normal(0.0, s, (N, 3))
    r = s * np.sqrt(-2.0 * np.log(rng.random(N) * rng.random(N)))
    ct = 2.0 * rng.random(N) - 1.0
    st = np.sqrt(1.0 - ct * ct)
    ph = 2.0 * np.pi * rng.random(N)
    Vw = np.stack([r * st * np.cos(ph), r * st * np.sin(ph), r * ct], 1)
    V = np.where(from_f[:, None], Vf, Vw)
    g = np.linalg.norm(v - V, axis=1)
    acc = rng.random(N) * (vm + np.linalg.norm(V, axis=1)) < g
    return (vm + ev) * acc.mean(), V[acc], acc.mean()


def test_majorant_sampler_matches_the_reference_sampler():
    rng = np.random.default_rng(2024)
    s = 1.0
    for speed in (0.2, 1.0, 3.0):
        v = np.array([speed, 0.0, 0.0])
        exact = np.linalg.norm(v - rng.normal(0.0, s, (4 * N, 3)), axis=1).mean()   # E|v - V|
        rate_ref, V_ref, acc_ref = _reference(rng, v, s)
        rate_maj, V_maj, acc_maj = _majorant(rng, v, s)
        # the collision rate (per n sigma): both samplers give E|v - V|, to Monte Carlo precision
        assert abs(rate_ref / exact - 1.0) < 0.01, (speed, rate_ref, exact)
        assert abs(rate_maj / exact - 1.0) < 0.01, (speed, rate_maj, exact)
        # the partner among accepted candidates: mean along v, mean speed, mean square across v
        for f in (lambda V: V[:, 0], lambda V: np.linalg.norm(V, axis=1), lambda V: V[:, 1] ** 2 + V[:, 2] ** 2):
            a, b = f(V_ref), f(V_maj)
            se = np.sqrt(a.var() / len(a) + b.var() / len(b))
            assert abs(a.mean() - b.mean()) < 5.0 * se, (speed, a.mean(), b.mean(), se)
        # and the majorant wastes far fewer candidates
        assert acc_maj > 1.9 * acc_ref, (speed, acc_maj, acc_ref)
