"""PGSE gradient waveforms for the KSPACE scheme (host only): rectangular and
trapezoidal (finite-ramp) lobes, their areas and the b-value their k(t)
gives, against the Stejskal-Tanner expressions."""
import math

import numpy as np
import pytest

GAMMA = 2.675e8


def wave(*a, **k):
    import initializator_gb300 as bt
    return bt.kspace_waveform_pgse(*a, **k)


def b_value(w, dt, refocus_t):
    """b = int k(t)^2 dt for the z waveform, the sign of the spin phase
    flipped by the 180 pulse at refocus_t (k piecewise linear within steps)."""
    g = w[:, 2].copy()
    t = (np.arange(len(g)) + 0.5) * dt
    g[t > refocus_t] *= -1.0
    k = np.concatenate([[0.0], np.cumsum(GAMMA * g * dt)])
    # exact integral of a piecewise-linear k over each step
    return float(np.sum(dt * (k[:-1] ** 2 + k[:-1] * k[1:] + k[1:] ** 2) / 3.0))


def test_rectangular_lobes_unchanged_with_zero_ramp():
    """Without ramps the waveform is each step's overlap with the two
    rectangular lobes, bit for bit (the form earlier runs used)."""
    dt = 1e-5
    a = wave(4000, dt, 0.1, 2.055e-3, 20e-3)
    b = wave(4000, dt, 0.1, 2.055e-3, 20e-3, ramp=0.0)
    assert np.array_equal(a, b)
    # each step's value is the rectangular lobes' overlap with it
    t0 = np.arange(4000) * dt
    t1 = t0 + dt

    def overlap(lo, hi):
        return np.clip(np.minimum(t1, hi) - np.maximum(t0, lo), 0.0, None) / dt

    expect = 0.1 * (overlap(0.0, 2.055e-3) + overlap(20e-3, 20e-3 + 2.055e-3))
    assert np.array_equal(a[:, 2], expect) and not a[:, :2].any()
    # a lobe edge inside a step: that step carries the lobe's fraction of it
    i = int(2.055e-3 / dt)
    assert math.isclose(a[i, 2], 0.1 * 0.5, rel_tol=1e-9)


@pytest.mark.parametrize("ramp", [0.0, 0.2e-3, 0.5e-3])
def test_lobe_areas_and_bounds(ramp):
    dt, g, delta, Delta = 1e-5, 0.1, 2e-3, 20e-3
    w = wave(2500, dt, g, delta, Delta, ramp=ramp)
    z = w[:, 2]
    assert np.all(z >= 0.0) and np.all(z <= g * (1 + 1e-12))
    split = int(10e-3 / dt)
    for part in (z[:split], z[split:]):
        assert math.isclose(part.sum() * dt, g * (delta - ramp), rel_tol=1e-12)


@pytest.mark.parametrize("ramp", [0.0, 0.3e-3])
def test_b_value_matches_stejskal_tanner(ramp):
    """Trapezoids of rise time e, lobe start-of-rise to start-of-fall d:
    b = gamma^2 G^2 (d^2 (Delta - d/3) + e^3/30 - d e^2/6)."""
    dt, g, delta, Delta = 1e-6, 0.1, 2e-3, 20e-3
    w = wave(int(24e-3 / dt), dt, g, delta, Delta, ramp=ramp)
    d, e = delta - ramp, ramp
    ref = GAMMA ** 2 * g ** 2 * (d * d * (Delta - d / 3) + e ** 3 / 30 - d * e * e / 6)
    assert math.isclose(b_value(w, dt, Delta / 2), ref, rel_tol=1e-3)


def test_rejects_ramps_longer_than_half_a_lobe():
    with pytest.raises(ValueError):
        wave(100, 1e-5, 0.1, 1e-3, 5e-3, ramp=0.6e-3)
