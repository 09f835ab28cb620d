"""The noise bound of the hybrid mode's KS check (surrogate.ks_noise_bound):
the Dvoretzky-Kiefer-Wolfowitz bound on the KS distance of an empirical CDF
from its own distribution, and how often samples of a perfect surrogate
exceed it."""
import math

import numpy as np
import pytest

from neutrinotelescopes_gb300.surrogate import HybridSimulator, ks_distance, ks_noise_bound


def test_bound_values():
    assert math.isclose(ks_noise_bound(40_000, 0.95), math.sqrt(math.log(40.0) / 80_000), rel_tol=1e-12)
    assert abs(ks_noise_bound(40_000, 0.95) - 0.00679) < 1e-5
    assert ks_noise_bound(40_000, 0.0) == 0.0
    assert ks_noise_bound(0, 0.95) == math.inf
    assert ks_noise_bound(10_000, 0.99) > ks_noise_bound(10_000, 0.95) > ks_noise_bound(40_000, 0.95)
    for bad in (1.0, 1.5, -0.1):
        with pytest.raises(ValueError):
            ks_noise_bound(1000, bad)


def test_perfect_samples_exceed_the_bound_rarely():
    """n uniform samples against the uniform CDF: the KS distance exceeds
    eps(n) in at most 5 % of the trials at 95 % confidence (the bound is
    conservative: about 4 % here)."""
    rng = np.random.default_rng(3)
    n, trials = 2000, 1000
    eps = ks_noise_bound(n, 0.95)
    i = np.arange(1, n + 1)
    over = 0
    for _ in range(trials):
        u = np.sort(rng.uniform(size=n))
        d = max(np.max(i / n - u), np.max(u - (i - 1) / n))
        over += d > eps
    assert over / trials <= 0.05 + 3 * math.sqrt(0.05 * 0.95 / trials)


def test_non_finite_cdf_fails_the_check():
    """A model CDF with a NaN (a diverged flow) gives a NaN distance, and a
    NaN distance with MC hits present is a failed check; without MC hits a
    check decides nothing."""
    u = np.linspace(0.001, 0.999, 500)
    assert abs(ks_distance(u) - 0.001) < 1e-3
    bad = u.copy()
    bad[-1] = np.nan
    assert math.isnan(ks_distance(bad))
    bad = u.copy()
    bad[0] = np.inf
    assert math.isnan(ks_distance(bad))
    sim = HybridSimulator.__new__(HybridSimulator)
    sim.ks_threshold, sim.ks_confidence = 0.02, 0.95
    assert sim.ks_fails(float("nan"), 40_000)
    assert not sim.ks_fails(float("nan"), 0)
    assert not sim.ks_fails(0.02, 40_000)
    assert sim.ks_fails(0.02 + ks_noise_bound(40_000, 0.95) + 1e-6, 40_000)
