"""The run statistics of leswht_gb300.stats on inputs with known answers
(CPU): the Strouhal estimator on a sampled sinusoid with an uneven time
step, the channel Nusselt number of a laminar profile, the cylinder
Nusselt number's normalisation, and mean/rms from dt-weighted sums."""
import math

import numpy as np
import pytest

from leswht_gb300 import cases, stats


def test_strouhal_of_a_sinusoid_with_uneven_steps():
    rng = np.random.default_rng(3)
    dt = 0.05 * (1.0 + 0.3 * rng.random(600))
    t = 10.0 + np.cumsum(dt)
    lift = 0.4 * np.sin(2 * math.pi * 0.21 * t + 0.3) + 0.02
    st = stats.strouhal(t, lift)
    assert st == pytest.approx(0.21, rel=1e-2)


def test_strouhal_needs_two_periods():
    t = np.linspace(0.0, 6.0, 400)          # 1.2 periods of St = 0.2
    assert stats.strouhal(t, np.sin(2 * math.pi * 0.2 * t)) is None
    assert stats.strouhal(t, np.zeros_like(t)) is None


def test_channel_nusselt_of_the_laminar_profile():
    # U = 1.5 (1 - y^2), T = 1 - y^2 with T = 0 at the walls: the wall
    # gradient is 2, the mixed-mean temperature 0.8, so Nu = 2 * 2 / 0.8 = 5
    g = cases.channel(4, 256, 4).grid
    y = np.asarray(g.ymp[1:g.n2m + 1])
    sh = (g.n3m, g.n2m, g.n1m)
    U = np.broadcast_to((1.5 * (1 - y ** 2))[None, :, None], sh)
    T = np.broadcast_to((1 - y ** 2)[None, :, None], sh)
    assert stats.channel_nusselt(T, U, g) == pytest.approx(5.0, rel=2e-3)


def test_cylinder_nusselt_normalisation():
    # heat rate of a unit-Nusselt body: pi D Lz dT / (Re Pr)
    q = math.pi * 1.0 * math.pi * 1.0 / (3900.0 * 0.71)
    assert stats.cylinder_nusselt(q, 3900.0, 0.71, 1.0, math.pi, 1.0) == pytest.approx(1.0, rel=1e-14)


def test_mean_and_rms_from_weighted_sums():
    rng = np.random.default_rng(5)
    sh = (2, 3, 4)
    samples = [rng.standard_normal(sh) for _ in range(50)]
    dts = rng.random(50) + 0.5
    win = dts.sum()
    avg = {}
    for name, f in (("uavg", lambda s: s), ("vavg", lambda s: 2 * s), ("wavg", lambda s: -s), ("pavg", lambda s: s),
                    ("uu", lambda s: s * s), ("vv", lambda s: 4 * s * s), ("ww", lambda s: s * s),
                    ("p2avg", lambda s: s * s)):
        avg[name] = sum(d * f(s) for d, s in zip(dts, samples))
    m = stats.mean_and_rms(avg, win)
    mean = sum(d * s for d, s in zip(dts, samples)) / win
    var = sum(d * (s - mean) ** 2 for d, s in zip(dts, samples)) / win
    assert np.allclose(m["u"], mean) and np.allclose(m["u_rms"], np.sqrt(var))
    assert np.allclose(m["v_rms"], 2 * np.sqrt(var))
