"""GPU parity of the O(3)/O(2) path against the FP64 oracle replay (same Philox
words, FP32 on the device) and statistical agreement with the reference's own
GPU summaries.

Tolerances (FP32 device arithmetic vs FP64 oracle):
  hot start 2e-6 per component; overrelaxation 1e-5 per component;
  Metropolis 1e-5 per component except sites whose acceptance test falls
  within rounding of the threshold (at most 0.1% of sites);
  observables 2e-6 relative to the number of bonds."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import golden_summary

pytestmark = pytest.mark.gpu


def grid(tmin, tmax, n):
    return [tmin + (tmax - tmin) * i / (n - 1) for i in range(n)]


@pytest.mark.parametrize("nc", [3, 2])
def test_hot_start_matches_oracle(gpu, oracle, nc):
    sizes = [4, 6, 8, 16]
    b = gpu.ContinuousBatch(sizes, 2, nc, seed=77)
    for s, L in enumerate(sizes):
        for r in range(2):
            g = b.get_spins(s, r).astype(np.float64).reshape(-1)
            o = oracle.cont_hot_start(L, nc, 77, r)
            assert np.max(np.abs(g - o)) < 2e-6


@pytest.mark.parametrize("sizes", [[4, 6, 8, 10, 16], [4, 8, 12, 16]])
@pytest.mark.parametrize("nc", [3, 2])
def test_halfsweeps_match_oracle(gpu, oracle, nc, sizes):
    """Sizes all multiples of 4 run the two-site column kernels; a size that
    is not runs the one-site kernels."""
    R, seed, J = 2, 5, 1.0
    temps = [1.2, 2.0] if nc == 3 else [1.8, 2.5]
    delta = 0.7 if nc == 3 else 1.3
    b = gpu.ContinuousBatch(sizes, R, nc, seed=seed)
    b.set_temperatures(temps, J=J)
    for s, L in enumerate(sizes):
        for r in range(R):
            st = b.get_spins(s, r).astype(np.float64).reshape(-1)
            # overrelaxation colour 0, then Metropolis colour 1, then measure
            o = st.copy()
            oracle.cont_overrelax(o, L, nc, 0, J)
            oracle.cont_metropolis(o, L, nc, 1, seed, r, 0, 1.0 / temps[r], J, delta)
            b._ref = getattr(b, "_ref", {})
            b._ref[(s, r)] = o
    b.overrelax(0)
    b.metropolis(1, delta)
    e, m, hb = b.measure()
    for s, L in enumerate(sizes):
        n = L ** 3
        for r in range(R):
            g = b.get_spins(s, r).astype(np.float64).reshape(-1, nc)
            o = b._ref[(s, r)].reshape(-1, nc)
            bad = np.any(np.abs(g - o) > 1e-5, axis=1)
            assert bad.sum() <= max(1, n // 1000), (L, r, bad.sum())
            q = oracle.cont_measure(g.reshape(-1), L, nc)
            k = s * R + r
            tol = 2e-6 * 3 * n
            assert abs(e[k] - q[0]) < tol
            assert np.all(np.abs(m[k, :nc] - q[1:1 + nc]) < tol)
            assert np.all(np.abs(hb[k] - q[4:10]) < tol)


@pytest.mark.parametrize("nc", [3, 2])
def test_two_site_kernels_match_one_site(gpu, nc):
    """Random streams are keyed per (L, replica), so L = 8 and 16 evolve the
    same in a batch of multiples of 4 (two-site overrelaxation and Metropolis
    kernels) and in one with an L = 6 added last (one-site kernels): bit for
    bit, through sweeps, exchanges and renormalisation."""
    R, temps = 2, ([1.3, 1.6] if nc == 3 else [1.9, 2.4])
    out = []
    for sizes in ([8, 16], [8, 16, 6]):
        b = gpu.ContinuousBatch(sizes, R, nc, seed=31)
        b.set_temperatures(temps)
        for _ in range(3):
            b.overrelax(0)
            b.overrelax(1)
            b.metropolis(0, 0.6)
            b.metropolis(1, 0.6)
        # exchange and renormalisation (every 2 sweeps) through the PT loop
        b.pt_run(6, 3, 3, delta=0.6, n_overrelax=1, renorm_every=2)
        out.append([b.get_spins(si, r) for si in range(2) for r in range(R)])
        b.close()
    for x, y in zip(out[0], out[1]):
        assert np.array_equal(x, y)


@pytest.mark.parametrize("nc", [3, 2])
def test_fused_measurement_matches_separate_pass(gpu, nc):
    """Measured PT sweeps fuse the measurement into the colour-1 Metropolis
    half-sweep (sizes multiples of 4): records (slots, E, M, bond sums) and
    spins equal those of the separate measurement pass bit for bit, through
    exchanges and a renormalisation sweep."""
    sizes, R = [8, 12, 16], 3
    temps = [1.3, 1.45, 1.6] if nc == 3 else [1.9, 2.2, 2.5]
    out = []
    for fused in (True, False):
        b = gpu.ContinuousBatch(sizes, R, nc, seed=61)
        b.set_fused_measure(fused)
        b.set_temperatures(temps)
        b.sweep(4, 0.6, 2)
        b.reset_sampling()
        rec = b.pt_run(40, 4, 2, delta=0.6, n_overrelax=2, renorm_every=10)
        out.append((rec, [b.get_spins(s_, r) for s_ in range(3) for r in range(R)],
                    b.metropolis_accepted()))
        b.close()
    for x, y in zip(out[0][0], out[1][0]):
        assert np.array_equal(x, y)
    for x, y in zip(out[0][1], out[1][1]):
        assert np.array_equal(x, y)
    assert np.array_equal(out[0][2], out[1][2])


@pytest.mark.parametrize("nc", [3, 2])
def test_overrelaxation_conserves_energy(gpu, nc):
    """overrelax.rs:74-86 (1e-8 in FP64); FP32 device: relative 1e-5."""
    b = gpu.ContinuousBatch([16, 32], 3, nc, seed=9)
    b.set_temperatures([1.4, 1.45, 1.5])
    b.sweep(20, 0.5, 0)
    e0, _, _ = b.measure()
    for _ in range(10):
        b.overrelax(0)
        b.overrelax(1)
    e1, _, _ = b.measure()
    n = np.repeat([16 ** 3, 32 ** 3], 3) * 3
    assert np.all(np.abs(e1 - e0) / n < 1e-5)


def test_renormalisation_and_determinism(gpu):
    runs = []
    for _ in range(2):
        b = gpu.ContinuousBatch([8, 16], 4, 3, seed=21)
        b.set_temperatures(grid(1.4, 1.5, 4))
        b.sweep(30, 0.5, 4)
        b.reset_sampling()
        rec = b.pt_run(200, 10, 5, delta=0.5, n_overrelax=4, renorm_every=100)
        runs.append((rec, b.get_spins(1, 2)))
    (r0, s0), (r1, s1) = runs
    for a, c in zip(r0, r1):
        assert np.array_equal(a, c)
    assert np.array_equal(s0, s1)
    # renormalisation happened at global sweep 229 (sweep counter 30 + 200)
    norms = np.linalg.norm(s0.astype(np.float64), axis=1)
    assert np.max(np.abs(norms - 1)) < 1e-5


def test_xy_ordered_helicity_limits(gpu):
    """All spins aligned: C_a = N per axis, S_a = 0 and E = -3N (ground state)."""
    L = 8
    b = gpu.ContinuousBatch([L], 1, 2, seed=1)
    b.set_temperatures([0.05])
    b.set_spins(0, 0, np.tile([1.0, 0.0], (L ** 3, 1)).astype(np.float32))
    e, m, hb = b.measure()
    n = L ** 3
    assert abs(e[0] + 3 * n) < 1e-3 and np.allclose(hb[0, :3], n) and np.allclose(hb[0, 3:], 0)


@pytest.mark.parametrize("model,nc,tmin,tmax,L", [("heisenberg", 3, 1.35, 1.55, 8),
                                                  ("heisenberg", 3, 1.35, 1.55, 16),
                                                  ("xy", 2, 2.10, 2.30, 8),
                                                  ("xy", 2, 2.10, 2.30, 16)])
def test_pt_statistics_match_reference_gpu_csv(gpu, model, nc, tmin, tmax, L):
    """Reference production grid (scripts/run_gpu_publication.sh:31-50: 20
    replicas, overrelax 5, delta 0.5, exchange 10, measure 5): E, |M|, M2, chi
    agree with the reference's own GPU summary within combined errors."""
    from helpers import pt_summary
    g = golden_summary(model, L)
    R = 20
    temps = grid(tmin, tmax, R)
    b = gpu.ContinuousBatch([L], R, nc, seed=314)
    b.set_temperatures(temps)
    b.sweep(3000, 0.5, 5)
    b.reset_sampling()
    rt, re, rm, rh = b.pt_run(30000, 10, 5, delta=0.5, n_overrelax=5, renorm_every=100)
    mabs = np.linalg.norm(rm, axis=2)
    s = pt_summary(rt, re, mabs, L, temps, dim=3, n_comp_m=True)
    for key in ("E", "M", "M2", "chi"):
        z = (s[key] - g[key]) / np.sqrt(s[key + "_err"] ** 2 + g[key + "_err"] ** 2)
        assert np.all(np.abs(z) < 5.5), (key, z)
        assert np.mean(z ** 2) < 3.5, (key, np.mean(z ** 2))


def test_continuous_lattice_mirror(gpu, oracle):
    lat = gpu.ContinuousGpuLattice(8, 3, 42)
    for _ in range(50):
        lat.sweep(1 / 1.45, 1.0, 0.5, 5)
    e, mx, my, mz = lat.measure_gpu(1.0)
    assert np.isfinite([e, mx, my, mz]).all() and e / 512 < -0.5
