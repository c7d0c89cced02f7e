"""GPU parity of the Ising path: bit-exact against the CPU checkerboard/Philox
replay (spins, integer bond sums and magnetisations, PT records, exchange
labels), then size-independent properties at the production sizes and
statistical agreement with the reference's own GPU summaries."""
from __future__ import annotations

import ctypes
import subprocess

import numpy as np
import pytest

from conftest import ROOT, golden_summary

pytestmark = pytest.mark.gpu

TEMPS3 = [4.40 + (4.62 - 4.40) * i / 31 for i in range(32)]


def grid(tmin, tmax, n):
    return [tmin + (tmax - tmin) * i / (n - 1) for i in range(n)]


# ------------------------------------------------------------ Philox pin
def test_philox_matches_curand(gpu, oracle, tmp_path):
    """The oracle's Philox4x32-10 equals curand's block function."""
    so = tmp_path / "libcp.so"
    subprocess.run(["nvcc", "-gencode=arch=compute_103a,code=sm_103a", "-shared", "-Xcompiler",
                    "-fPIC", "-o", str(so), str(ROOT / "tests/cuda/philox_curand.cu")], check=True)
    lib = ctypes.CDLL(str(so))
    rng = np.random.default_rng(0)
    n = 4096
    ctr = rng.integers(0, 2 ** 32, (n, 4), dtype=np.uint64).astype(np.uint32)
    key = rng.integers(0, 2 ** 32, (n, 2), dtype=np.uint64).astype(np.uint32)
    ctr[0] = 0
    key[0] = 0
    ctr[1] = 0xFFFFFFFF
    key[1] = 0xFFFFFFFF
    out = np.zeros((n, 4), np.uint32)
    p = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    assert lib.curand_philox_blocks(p(ctr), p(key), p(out), n) == 0
    for i in range(n):
        assert np.array_equal(oracle.philox(ctr[i], key[i]), out[i]), i


# ------------------------------------------------------------ bit-exact
@pytest.mark.parametrize("dim,sizes", [(3, [2, 4, 6, 8, 10, 16, 32]), (2, [4, 6, 8, 16, 32, 64])])
def test_hot_start_bit_exact(gpu, oracle, dim, sizes):
    b = gpu.IsingBatch(sizes, 3, seed=1234567890123, dim=dim)
    for s, L in enumerate(sizes):
        for r in range(3):
            assert np.array_equal(b.get_spins(s, r), oracle.hot_start(L, dim, 1234567890123, r))


@pytest.mark.parametrize("dim,sizes,h", [(3, [2, 4, 6, 8, 10, 16, 32], 0.0),
                                         (3, [8, 12, 24, 32, 40, 48, 64], 0.0),
                                         (3, [4, 8, 16, 24], 0.35),
                                         (2, [4, 6, 8, 16, 32, 48, 64, 80], 0.0)])
def test_sweeps_bit_exact(gpu, oracle, dim, sizes, h):
    """Every size of a batch advances in the one half-sweep launch (rolling,
    flat and site-block tasks side by side; 3D L = 24, 40, 48 and 2D L = 48,
    80 are flat tasks with rows of a non-power-of-two number of words) and
    matches the oracle bit for bit."""
    R, seed, J = 3, 42, 1.0
    temps = [2.0, 4.5, 7.0] if dim == 3 else [1.5, 2.269, 3.5]
    b = gpu.IsingBatch(sizes, R, seed=seed, dim=dim)
    b.set_temperatures(temps, J=J, h=h)
    ref = {(s, r): oracle.hot_start(L, dim, seed, r) for s, L in enumerate(sizes) for r in range(R)}
    thr = [oracle.thresholds(dim, 1.0 / T, J, h) for T in temps]
    for sweep in range(7):
        b.step(1)
        for (s, r), sp in ref.items():
            for c in (0, 1):
                oracle.halfsweep(sp, sizes[s], dim, c, seed, r, sweep, thr[r])
    bond, mag = b.measure()
    for (s, r), sp in ref.items():
        assert np.array_equal(b.get_spins(s, r), sp), (sizes[s], r)
        ob, om = oracle.measure(sp, sizes[s], dim)
        assert bond[s * R + r] == ob and mag[s * R + r] == om


@pytest.mark.parametrize("dim,sizes,R", [(3, [8, 12, 16, 32], 5), (2, [16, 32, 64], 17)])
def test_resident_pt_matches_graph_cycle(gpu, dim, sizes, R):
    """Small lattices run pt_run in one cooperative resident launch (sweeps,
    measurements, exchanges at a grid barrier); the CUDA-graph cycle of
    separate launches gives the same records, ladder, acceptances and spins
    bit for bit, also across calls that split the exchange period."""
    temps = grid(4.3, 4.7, R) if dim == 3 else grid(2.1, 2.5, R)
    out = []
    for resident in (True, False):
        b = gpu.IsingBatch(sizes, R, seed=77, dim=dim)
        b.set_resident_pt(resident)
        b.set_temperatures(temps)
        b.step(7)
        b.reset_sampling()
        parts = [b.pt_run(n, 10, 3) for n in (37, 100, 13)]
        rec = [np.concatenate([p_[i] for p_ in parts]) for i in range(3)]
        out.append((rec, b.r2t(), b.accepted(), b.sweep_counter(),
                    [b.get_spins(s_, r) for s_ in range(len(sizes)) for r in range(R)]))
        b.close()
    (ra, ta, aa, sa, pa), (rb, tb, ab, sb, pb) = out
    for x, y in zip(ra, rb):
        assert np.array_equal(x, y)
    assert np.array_equal(ta, tb) and np.array_equal(aa, ab) and sa == sb
    assert aa.sum() > 0
    for x, y in zip(pa, pb):
        assert np.array_equal(x, y)


def test_set_spins_roundtrip_and_ordered_limits(gpu, oracle):
    """Ground state: E = -3 (3D) / -2 (2D) per site, |m| = 1 at T = 0.1
    (known_limits_summary.csv, observables.rs:189-216)."""
    for dim, sizes, e0 in [(3, [8, 16], -3.0), (2, [16, 32], -2.0)]:
        b = gpu.IsingBatch(sizes, 2, seed=5, dim=dim)
        b.set_temperatures([0.1, 0.1])
        for s, L in enumerate(sizes):
            for r in range(2):
                b.set_spins(s, r, np.ones(L ** dim, np.int8))
                assert np.all(b.get_spins(s, r) == 1)
        b.step(100)
        bond, mag = b.measure()
        for s, L in enumerate(sizes):
            n = L ** dim
            for r in range(2):
                assert -bond[s * 2 + r] / n == e0 and abs(mag[s * 2 + r]) / n == 1.0


@pytest.mark.parametrize("ee,me", [(10, 5), (3, 2), (1, 1), (7, 3)])
def test_pt_run_bit_exact(gpu, oracle, ee, me):
    """Records (slot, bond, mag), exchange labels and final spins of a PT run
    through the CUDA graph equal the oracle's replay."""
    sizes, R, dim, seed = [8, 12, 16], 8, 3, 99
    temps = grid(4.3, 4.7, R)
    b = gpu.IsingBatch(sizes, R, seed=seed, dim=dim)
    b.set_temperatures(temps)
    b.step(15)
    b.reset_sampling()
    parts = [b.pt_run(n, ee, me) for n in (23, 40, 1, 36)]
    rt = np.concatenate([p[0] for p in parts])
    rb = np.concatenate([p[1] for p in parts])
    rm = np.concatenate([p[2] for p in parts])
    r2t = b.r2t()
    for s, L in enumerate(sizes):
        pt = oracle.IsingPT(L, dim, R, temps, seed)
        pt.warmup(15)
        pt.reset_sampling()
        ot, ob, om = pt.sample(100, ee, me)
        sl = slice(s * R, (s + 1) * R)
        assert rt.shape[0] == ot.shape[0]
        assert np.array_equal(rt[:, sl], ot)
        assert np.array_equal(rb[:, sl], ob)
        assert np.array_equal(rm[:, sl], om)
        assert np.array_equal(r2t[sl], pt.r2t)
        for r in range(R):
            assert np.array_equal(b.get_spins(s, r), pt.replica_spins(r))
    acc = b.accepted()
    assert np.all(acc > 0)


def test_uneven_sizes_pt_matches_oracle(gpu, oracle):
    """Sizes that are not powers of two run as flat word tasks (L = 24, 48:
    multiples of 8) or site-block tasks (L = 12, 20: one Philox block's 16
    sites per thread), here in the graph cycle (the resident kernel is
    switched off): records with the fused E/M sums, exchanges and final spins
    equal the oracle's PT replay."""
    sizes, R, dim, seed = [12, 24, 48, 20], 2, 3, 31
    temps = grid(4.4, 4.6, R)
    b = gpu.IsingBatch(sizes, R, seed=seed, dim=dim)
    b.set_resident_pt(False)
    b.set_temperatures(temps)
    b.step(3)
    b.reset_sampling()
    rt, rb, rm = b.pt_run(20, 5, 2)
    r2t = b.r2t()
    for s, L in enumerate(sizes):
        pt = oracle.IsingPT(L, dim, R, temps, seed)
        pt.warmup(3)
        pt.reset_sampling()
        ot, ob, om = pt.sample(20, 5, 2)
        sl = slice(s * R, (s + 1) * R)
        assert np.array_equal(rt[:, sl], ot), L
        assert np.array_equal(rb[:, sl], ob), L
        assert np.array_equal(rm[:, sl], om), L
        assert np.array_equal(r2t[sl], pt.r2t), L
        for r in range(R):
            assert np.array_equal(b.get_spins(s, r), pt.replica_spins(r)), (L, r)
    b.close()


def test_largest_sizes_match_oracle(gpu, oracle):
    """The largest lattices: 3D L = 512 (134M sites, flat word tasks with rows of
    64 words) and 2D L = 1024 (rows of 128 words), bit for bit against the
    oracle through sweeps and the measured sums."""
    for dim, L, R, n_sw, T in ((3, 512, 1, 1, 4.5), (2, 1024, 2, 2, 2.3)):
        seed = 5
        b = gpu.IsingBatch([L], R, seed=seed, dim=dim)
        b.set_temperatures([T] * R)
        b.step(n_sw)
        bond, mag = b.measure()
        thr = oracle.thresholds(dim, 1.0 / T)
        for r in range(R):
            sp = oracle.hot_start(L, dim, seed, r)
            for k in range(n_sw):
                for c in (0, 1):
                    oracle.halfsweep(sp, L, dim, c, seed, r, k, thr)
            assert np.array_equal(b.get_spins(0, r), sp), (dim, L, r)
            ob, om = oracle.measure(sp, L, dim)
            assert bond[r] == ob and mag[r] == om, (dim, L, r)
        b.close()


def test_large_flat_batches_group_tasks(gpu, oracle):
    """A 2D batch of at least 8192 flat warp tasks (L = 256 x 32) runs its flat
    tasks four per warp (all loads of a group before any decision); replicas
    across the batch match the oracle bit for bit, and so do the measured
    bond and magnetisation sums."""
    L, R, seed = 256, 32, 11
    temps = grid(2.0, 2.6, R)
    b = gpu.IsingBatch([L], R, seed=seed, dim=2)
    b.set_temperatures(temps)
    b.step(3)
    bond, mag = b.measure()
    for r in (0, 17, 31):
        sp = oracle.hot_start(L, 2, seed, r)
        thr = oracle.thresholds(2, 1.0 / temps[r])
        for k in range(3):
            for c in (0, 1):
                oracle.halfsweep(sp, L, 2, c, seed, r, k, thr)
        assert np.array_equal(b.get_spins(0, r), sp), r
        ob, om = oracle.measure(sp, L, 2)
        assert bond[r] == ob and mag[r] == om, r
    b.close()


def test_exchange_api_matches_oracle(gpu, oracle):
    sizes, R, seed = [8, 16], 6, 7
    temps = grid(4.0, 5.0, R)
    b = gpu.IsingBatch(sizes, R, seed=seed)
    b.set_temperatures(temps)
    betas = 1.0 / np.array(temps)
    r2t_o = [np.arange(R, dtype=np.int32) for _ in sizes]
    t2r_o = [np.arange(R, dtype=np.int32) for _ in sizes]
    for k in range(12):
        b.step(3)
        bond, mag = b.measure()
        acc = b.exchange(k % 2)
        for s, L in enumerate(sizes):
            en = -bond[s * R:(s + 1) * R].astype(np.float64)
            a = oracle.exchange(betas, en, r2t_o[s], t2r_o[s], k % 2, seed, L, k)
            assert a == acc[s]
        got = b.r2t()
        for s in range(len(sizes)):
            assert np.array_equal(got[s * R:(s + 1) * R], r2t_o[s])


# ------------------------------------------------------------ full-size properties
def test_production_size_properties(gpu, oracle):
    """Production configuration (L = 8..128, 32 replicas): fused measurement
    equals the standalone reduction, spins stay +-1, runs are deterministic and
    launch-shape independent, and L = 128 replicas match the replay bit for bit."""
    sizes, R = [8, 16, 32, 64, 128], 32
    a = gpu.IsingBatch(sizes, R, seed=42)
    a.set_temperatures(TEMPS3)
    a.step(20)
    a.reset_sampling()
    rt, rb, rm = a.pt_run(10, 10, 5)
    bond, mag = a.measure()
    assert np.array_equal(rb[-1], bond) and np.array_equal(rm[-1], mag)
    s = a.get_spins(4, 31)
    assert set(np.unique(s)) <= {-1, 1}
    c = gpu.IsingBatch(sizes, R, seed=42)
    c.set_temperatures(TEMPS3)
    c.set_launch(128, 2)
    c.step(20)
    c.reset_sampling()
    rt2, rb2, rm2 = c.pt_run(10, 10, 5)
    assert np.array_equal(rb, rb2) and np.array_equal(rm, rm2) and np.array_equal(rt, rt2)
    for si in (0, 4):
        for r in (0, 17):
            assert np.array_equal(a.get_spins(si, r), c.get_spins(si, r))
    # full-size bit-exactness: L = 128 replicas against the replay
    d = gpu.IsingBatch([128], 2, seed=3)
    d.set_temperatures([4.5, 4.6])
    d.step(2)
    for r, T in enumerate([4.5, 4.6]):
        sp = oracle.hot_start(128, 3, 3, r)
        thr = oracle.thresholds(3, 1.0 / T)
        for k in range(2):
            for colour in (0, 1):
                oracle.halfsweep(sp, 128, 3, colour, 3, r, k, thr)
        assert np.array_equal(d.get_spins(0, r), sp)


@pytest.mark.parametrize("depth", [1, 2, 3])
def test_rolling_sizes_match_replay(gpu, oracle, depth):
    """Every rolling size (L = 32: a warp task is the whole plane; L = 64:
    16-row tasks; L = 256: 4-row tasks, the first/last halo rows of every
    lane group) against the replay, bit for bit, with loads one or two planes
    ahead in registers or through the shared-memory ring (depth 3)."""
    for L in (32, 64, 256):
        d = gpu.IsingBatch([L], 1, seed=5)
        d.set_prefetch(depth)
        d.set_temperatures([4.51])
        d.step(2)
        sp = oracle.hot_start(L, 3, 5, 0)
        thr = oracle.thresholds(3, 1.0 / 4.51)
        for k in range(2):
            for colour in (0, 1):
                oracle.halfsweep(sp, L, 3, colour, 5, 0, k, thr)
        assert np.array_equal(d.get_spins(0, 0), sp), L
        d.close()


def test_prefetch_depth_keeps_results(gpu):
    """Every rolling prefetch form gives the same bits (L = 64 and 128 are
    rolling), through sweeps with fused measurements and exchanges."""
    sizes, R = [64, 128], 2
    out = []
    for depth in (1, 2, 3):
        b = gpu.IsingBatch(sizes, R, seed=13)
        b.set_prefetch(depth)
        b.set_temperatures(grid(4.4, 4.6, R))
        b.step(4)
        _, bb, mm = b.pt_run(6, 3, 2)
        out.append((bb, mm, [b.get_spins(s, r) for s in range(2) for r in range(R)]))
    for o in out[1:]:
        assert np.array_equal(out[0][0], o[0]) and np.array_equal(out[0][1], o[1])
        for x, y in zip(out[0][2], o[2]):
            assert np.array_equal(x, y)


def test_words_per_lane_keep_results(gpu, oracle):
    """3D L >= 32 rolls with four words per lane by default (L = 64: two
    replicas per CTA task, L = 32: eight, so R = 3 leaves tasks part empty;
    at L = 32 a warp task is a whole plane), or with two: the
    same bits, through sweeps with fused measurements and exchanges, with the
    cache prefetch on or off and with dependent or ordinary launches; L = 64
    and L = 128 sweeps also against the oracle."""
    sizes, R = [32, 64, 128, 256], 3
    out = []
    for words, pf, dep in ((4, 0, True), (2, 0, True), (4, 3, True), (4, 0, False)):
        b = gpu.IsingBatch(sizes, R, seed=17)
        b.set_words_per_lane(words)
        b.set_cache_prefetch(2, pf)
        b.set_dependent_launch(dep)
        b.set_temperatures(grid(4.4, 4.6, R))
        b.step(3)
        _, bb, mm = b.pt_run(6, 3, 2)
        out.append((bb, mm, [b.get_spins(s, r) for s in range(4) for r in range(R)]))
        b.close()
    d64 = gpu.IsingBatch([64], 3, seed=29)
    d64.set_temperatures([4.45, 4.5, 4.55])
    sp64 = [d64.get_spins(0, r) for r in range(3)]
    d64.step(1)
    for r in range(3):
        thr64 = oracle.thresholds(3, 1 / [4.45, 4.5, 4.55][r])
        for c in (0, 1):
            oracle.halfsweep(sp64[r], 64, 3, c, 29, r, 0, thr64)
        assert np.array_equal(d64.get_spins(0, r), sp64[r]), r
    d64.close()
    for o in out[1:]:
        assert np.array_equal(out[0][0], o[0]) and np.array_equal(out[0][1], o[1])
        for x, y in zip(out[0][2], o[2]):
            assert np.array_equal(x, y)
    d = gpu.IsingBatch([128], 1, seed=23)
    d.set_temperatures([4.5])
    sp = d.get_spins(0, 0)
    d.step(1)
    thr = oracle.thresholds(3, 1 / 4.5)
    for c in (0, 1):
        oracle.halfsweep(sp, 128, 3, c, 23, 0, 0, thr)
    assert np.array_equal(d.get_spins(0, 0), sp)
    d.close()


def test_autotune_keeps_results(gpu):
    sizes, R = [8, 32, 64], 16
    a = gpu.IsingBatch(sizes, R, seed=1)
    a.set_temperatures(grid(4.4, 4.6, R))
    a.step(5)
    ref = [a.get_spins(2, r) for r in range(R)]
    best = a.autotune()
    assert best[0] in (128, 256, 512) and best[2] in (1, 2, 3)
    for r in range(R):
        assert np.array_equal(a.get_spins(2, r), ref[r])
    assert a.sweep_counter() == 5
    ms = a.time_halfsweep(6)
    assert ms > 0
    for r in range(R):
        assert np.array_equal(a.get_spins(2, r), ref[r])


# ------------------------------------------------------------ statistics
@pytest.mark.parametrize("L", [8, 16])
def test_pt_statistics_match_reference_gpu_csv(gpu, L):
    """Same grid/cadence as the reference's production run
    (scripts/run_gpu_publication.sh:22-29): E, |M|, M2, chi agree with the
    reference's own GPU summary CSV within combined jackknife errors."""
    from helpers import pt_summary
    g = golden_summary("ising", L)
    b = gpu.IsingBatch([L], 32, seed=2024)
    b.set_temperatures(TEMPS3)
    b.step(5000)
    b.reset_sampling()
    rt, rb, rm = b.pt_run(50000, 10, 5)
    s = pt_summary(rt, -rb.astype(float), rm, L, TEMPS3)
    for key in ("E", "M", "M2", "chi"):
        z = (s[key] - g[key]) / np.sqrt(s[key + "_err"] ** 2 + g[key + "_err"] ** 2)
        assert np.all(np.abs(z) < 5.0), (key, z)
        assert np.mean(z ** 2) < 3.0, (key, np.mean(z ** 2))


def test_lattice_gpu_mirror(gpu, oracle):
    """LatticeGpu.step / measure_gpu / energy_gpu mirror lattice_gpu.rs."""
    lat = gpu.LatticeGpu(8, 42)
    sp = oracle.hot_start(8, 3, 42, 0)
    thr = oracle.thresholds(3, 1 / 4.5, 1.0, 0.0)
    for k in range(5):
        lat.step(1 / 4.5, 1.0, 0.0)
        for c in (0, 1):
            oracle.halfsweep(sp, 8, 3, c, 42, 0, k, thr)
    assert np.array_equal(lat.get_spins(), sp)
    bnd, mag = oracle.measure(sp, 8)
    e, m = lat.measure_gpu(1.0)
    assert e == -bnd / 512 and m == abs(mag) / 512
    assert lat.energy_gpu(1.0) == -bnd
