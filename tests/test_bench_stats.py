"""Host-side parts of bench.py: the autocorrelation estimators it uses for ESS/s
(the windowed tau_int and the blocking estimate that catches rare long
excursions) and the JSON line of its reference arm."""
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


def test_reference_arm_line_keeps_the_contract():
    """`bench.py --impl reference` (host CPU, no GPU): one JSON line with the
    headline's metric, unit and workload, a cpu_baseline describing the run and
    an e2e entry with no host-device bytes."""
    import json
    import subprocess
    import sys

    from conftest import ROOT

    b = _bench()
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference",
                          "--steps", "2", "--warmup", "3", "--ref-seconds", "2"],
                         capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == b.METRIC and d["unit"] == "flips/ns"
    assert d["config"]["workload"] == b.WORKLOAD and d["higher_is_better"] is True
    assert d["value"] > 0 and d["steps"] == 2 and d["warmup"] == 3
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == d["value"]
    e = d["e2e"]
    assert e["value"] == d["value"] and e["h2d_bytes_per_step"] == 0 == e["d2h_bytes_per_step"]


def test_tau_int_matches_the_reference_estimator():
    """bench.tau_int (FFT autocorrelation) against the reference's own
    `integrated_autocorrelation_time(autocorrelation(x))` of
    analysis/scripts/reproduce_validation.py, evaluated on seeded series by
    tests/golden/make_tau_golden.py."""
    from conftest import ROOT

    b = _bench()
    g = np.load(ROOT / "tests" / "golden" / "tau_golden.npz")
    for x, t in zip(g["series"], g["tau"]):
        assert abs(b.tau_int(x) - t) <= 1e-9 * max(1.0, t), (b.tau_int(x), t)
