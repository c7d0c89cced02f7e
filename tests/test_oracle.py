"""Pins the CPU oracle against the reference's own fixtures and known answers
(no GPU).  The oracle is then the checker for the GPU parity tests."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import golden_summary, read_csv


def test_exact_enumeration_matches_reference_table(oracle):
    """Our enumeration reproduces the reference's committed 4x4 exact values
    (exact_enumeration_comparison.csv, from reproduce_validation.py:88-140)."""
    rows = read_csv("exact_enumeration_comparison.csv")
    temps = [r["T"] for r in rows]
    ours = oracle.exact_enumeration(4, 2, temps)
    for r, o in zip(rows, ours):
        assert abs(o["E"] - r["E_exact"]) < 1e-10
        assert abs(o["M"] - r["M_exact"]) < 1e-10
        assert abs(o["M2"] - r["M2_exact"]) < 1e-10
        assert abs(o["M4"] - r["M4_exact"]) < 1e-10
        assert abs(o["Cv"] - r["Cv_exact"]) < 1e-9
        assert abs(o["chi"] - r["chi_conn_exact"]) < 1e-9


def test_onsager_formulas_match_reference_table(oracle):
    rows = [r for r in read_csv("onsager_comparison.csv") if r["n"] == 16][:10]
    for r in rows:
        assert abs(oracle.onsager_energy(r["T"]) - r["E_exact"]) < 1e-12
        assert abs(oracle.onsager_magnetization(r["T"]) - r["M_exact"]) < 1e-12


def test_reference_cpu_path_2d_exact_enumeration(oracle):
    """Random-site Metropolis (metropolis.rs:8-27) on 4x4 agrees with exact
    enumeration within the reference's validation thresholds
    (validation_metrics.csv: |dE| <= 0.02, |dM| <= 0.01)."""
    for T in (1.5, 2.3, 3.0):
        e, m = oracle.ref_run(4, 2, T, seed=7, warmup=2000, samples=60000)
        ex = oracle.exact_enumeration(4, 2, [T])[0]
        assert abs(e.mean() - ex["E"]) < 0.02
        assert abs(m.mean() - ex["M"]) < 0.01


def test_reference_cpu_path_onsager(oracle):
    """2D L=32 below Tc: E within the reference's Onsager threshold (0.01)."""
    for T in (1.6, 2.0):
        e, m = oracle.ref_run(32, 2, T, seed=11, warmup=1000, samples=3000)
        assert abs(e.mean() - oracle.onsager_energy(T)) < 0.01
        assert abs(m.mean() - oracle.onsager_magnetization(T)) < 0.03


def test_checkerboard_replay_3d_exact_enumeration(oracle):
    """The checkerboard/Philox replay (the GPU's bit-exact oracle) samples the
    Boltzmann distribution of a 2x2x2 periodic cube (all 256 states)."""
    L, dim = 2, 3
    for T in (2.0, 5.0):
        pt = oracle.IsingPT(L, dim, 1, [T], seed=3)
        pt.warmup(500)
        rt, rb, rm = pt.sample(200000, 1 << 30, 1)
        n = L ** 3
        e = -rb[:, 0] / n
        m = np.abs(rm[:, 0]) / n
        ex = oracle.exact_enumeration(L, dim, [T])[0]
        assert abs(e.mean() - ex["E"]) < 0.02
        assert abs(m.mean() - ex["M"]) < 0.01


def test_checkerboard_replay_known_limits(oracle):
    """known_limits_summary.csv: 3D ground state E=-3, |m|=1 at T=0.1 from an
    ordered start; high-T energy near 0."""
    pt = oracle.IsingPT(8, 3, 1, [0.1], seed=5)
    pt.spins[:] = 1
    pt.warmup(50)
    b, m = oracle.measure(pt.replica_spins(0), 8)
    assert -b / 512 == -3.0 and abs(m) / 512 == 1.0
    pt = oracle.IsingPT(8, 3, 1, [50.0], seed=5)
    pt.warmup(200)
    rt, rb, rm = pt.sample(2000, 1 << 30, 1)
    assert abs((-rb[:, 0] / 512).mean()) < 0.1


def test_checkerboard_replay_pt_matches_reference_gpu_csv(oracle):
    """PT replay of the reference's production grid (32 replicas on
    [4.40, 4.62], exchange 10, measure 5) for L=8 agrees with the reference's
    own GPU result (gpu_fss_ising_N8_summary.csv) within combined jackknife
    errors."""
    from helpers import pt_summary
    g = golden_summary("ising", 8)
    temps = [4.40 + (4.62 - 4.40) * i / 31 for i in range(32)]
    pt = oracle.IsingPT(8, 3, 32, temps, seed=42)
    pt.warmup(1000)
    pt.reset_sampling()
    rt, rb, rm = pt.sample(20000, 10, 5)
    s = pt_summary(rt, -rb.astype(float), rm, 8, temps, dim=3)
    for key in ("E", "M", "M2", "chi"):
        z = (s[key] - g[key]) / np.sqrt(s[key + "_err"] ** 2 + g[key + "_err"] ** 2)
        assert np.all(np.abs(z) < 5.0), (key, z)
        assert np.mean(z ** 2) < 3.0, (key, np.mean(z ** 2))


def test_exchange_bijectivity(oracle):
    """parallel_tempering.rs:52-66: labels stay a permutation."""
    R = 9
    betas = 1.0 / np.linspace(4.0, 5.0, R)
    rng = np.random.default_rng(0)
    r2t = np.arange(R, dtype=np.int32)
    t2r = np.arange(R, dtype=np.int32)
    for k in range(200):
        en = rng.normal(-1000, 50, R)
        oracle.exchange(betas, en, r2t, t2r, k % 2, 42, 8, k)
        assert sorted(r2t) == list(range(R))
        assert all(t2r[r2t[r]] == r for r in range(R))


def test_jackknife_constant_series(oracle):
    out = oracle.jackknife(np.full(100, -1.5), np.full(100, 0.25), 0.2, 512, 20)
    assert out[0] == -1.5 and out[1] == 0.0 and out[2] == 0.25 and out[8] == 0.0
