"""The shedding analysis of the configuration timings (the crossing-count
Strouhal estimate of karman_shedding.mjs:94-114) on synthetic probe
signals; no GPU."""
import math

import numpy as np

from tsl_array_n_gb300.configs import strouhal


def test_strouhal_of_a_sinusoid():
    dt, every, diameter, speed, st = 1.0 / 512, 2, 0.125, 1.0, 0.2
    f = st * speed / diameter
    t = np.arange(0, 6000, every) * dt
    rng = np.random.default_rng(0)
    sig = 0.3 * np.sin(2 * math.pi * f * t + 0.4) + 0.01 * rng.standard_normal(t.size)
    got, crossings = strouhal(sig, every, dt, diameter, speed)
    assert crossings > 10
    assert abs(got - st) < 0.02 * st


def test_strouhal_of_a_steady_wake_is_none():
    sig = np.full(500, 0.02) + 1e-9 * np.arange(500)
    got, crossings = strouhal(sig, 2, 1.0 / 512, 0.125, 1.0)
    assert got is None and crossings <= 1
