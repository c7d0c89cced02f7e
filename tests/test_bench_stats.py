"""The autocorrelation estimators bench.py uses for ESS/s: the windowed tau_int
and the blocking estimate that catches rare long excursions."""
from __future__ import annotations

import numpy as np

from test_bench_dist import _bench


def _ar1(rng, n, rho):
    e = rng.standard_normal(n) * np.sqrt(1 - rho * rho)
    x = np.empty(n)
    x[0] = rng.standard_normal()
    for i in range(1, n):
        x[i] = rho * x[i - 1] + e[i]
    return x


def test_estimators_agree_on_ar1():
    b = _bench()
    rng = np.random.default_rng(5)
    x = _ar1(rng, 400_000, 0.9)
    exact = (1 + 0.9) / (2 * (1 - 0.9))
    assert abs(b.tau_int(x) - exact) < 0.1 * exact
    assert abs(b.tau_blocking(x) - exact) < 0.5 * exact   # 19 degrees of freedom
    assert abs(b.tau_int(rng.standard_normal(100_000)) - 0.5) < 0.05


def test_blocking_sees_the_slow_component_the_window_misses():
    """A fast component plus a small, very slow one (the shape of a sticky
    independence chain): the windowed sum stops after a few fast times; the
    block means see the slow drift."""
    b = _bench()
    rng = np.random.default_rng(6)
    n = 400_000
    x = rng.standard_normal(n) + 0.3 * _ar1(rng, n, 0.9999)
    w, bl = b.tau_int(x), b.tau_blocking(x)
    assert w < 5.0
    assert bl > 20 * w, (w, bl)


def test_jackknife_error_of_white_noise():
    b = _bench()
    rng = np.random.default_rng(7)
    x = rng.standard_normal(200_000)
    err = b.jackknife_mean_err(x)
    assert abs(err - 1 / np.sqrt(len(x))) < 0.4 / np.sqrt(len(x))
