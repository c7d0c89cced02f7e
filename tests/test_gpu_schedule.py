"""isg_ising_run_schedule: temperature schedules without exchange (the sweep
loops of src/cuda/fss_gpu.rs, kz_gpu.rs and coarsening_gpu.rs), checked bit for
bit against the oracle's replay — the cluster-resident kernel (small lattices,
one thread-block cluster per lattice) and the half-sweep fallback (large ones)
— plus the identity with plain sweeps (isg_ising_step)."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _replay(oracle, sizes, dim, R, temps0, seed, temps, n, every, phase):
    out = []
    for L in sizes:
        pt = oracle.IsingPT(L, dim, R, temps0, seed)
        b, m = pt.schedule(temps, n, every, phase)
        out.append((pt, b, m))
    return out


@pytest.mark.parametrize("dim,sizes,R", [
    (3, [4, 6, 8, 12, 20, 28, 32], 3),   # clusters of 1..8 CTAs
    (2, [8, 10, 64, 90], 2),
])
def test_current_temperatures_vs_oracle(gpu, oracle, dim, sizes, R):
    temps0 = [4.3, 4.5, 4.7][:R] if dim == 3 else [2.2, 2.4][:R]
    b = gpu.IsingBatch(sizes, R, seed=21, dim=dim)
    b.set_temperatures(temps0)
    b.step(3)
    rb, rm = b.run_schedule(None, 17, 3, 1)
    want = _replay(oracle, sizes, dim, R, temps0, 21, None, 0, 0, 0)
    for s, (pt, _, _) in enumerate(want):
        pt.warmup(3)
        wb, wm = pt.schedule(None, 17, 3, 1)
        sl = slice(s * R, (s + 1) * R)
        assert rb.shape[0] == 6 and np.array_equal(rb[:, sl], wb) and np.array_equal(rm[:, sl], wm)
        for r in range(R):
            assert np.array_equal(b.get_spins(s, r), pt.replica_spins(r)), (sizes[s], r)


def test_ramp_vs_oracle(gpu, oracle):
    """A linear quench ramp (kz_gpu.rs:28-33): one temperature per sweep."""
    sizes, R = [6, 20, 24], 2
    ramp = [6.0 + (1.0 - 6.0) * (k + 1) / 25 for k in range(25)]
    b = gpu.IsingBatch(sizes, R, seed=5)
    rb, rm = b.run_schedule(ramp, None, 5, 4)
    for s, L in enumerate(sizes):
        pt = oracle.IsingPT(L, 3, R, [6.0] * R, 5)
        wb, wm = pt.schedule(ramp, 25, 5, 4)
        sl = slice(s * R, (s + 1) * R)
        assert np.array_equal(rb[:, sl], wb) and np.array_equal(rm[:, sl], wm), L
        for r in range(R):
            assert np.array_equal(b.get_spins(s, r), pt.replica_spins(r))
    # every slot now holds the last temperature: plain sweeps continue the same chain
    b.step(2)
    for s, L in enumerate(sizes):
        pt = oracle.IsingPT(L, 3, R, [6.0] * R, 5)
        pt.schedule(ramp, 25)
        pt.temps[:] = ramp[-1]
        pt.warmup(2)
        for r in range(R):
            assert np.array_equal(b.get_spins(s, r), pt.replica_spins(r))


def test_large_lattice_fallback_vs_oracle(gpu, oracle):
    """L = 64 and 128 exceed the resident limit: the half-sweep kernels run the
    schedule sweep by sweep with the same stream."""
    sizes, R = [64, 128], 1
    temps = [4.6, 4.5, 4.5, 4.4]
    b = gpu.IsingBatch(sizes, R, seed=8)
    rb, rm = b.run_schedule(temps, None, 2, 1)
    for s, L in enumerate(sizes):
        pt = oracle.IsingPT(L, 3, R, [4.6], 8)
        wb, wm = pt.schedule(temps, 4, 2, 1)
        assert np.array_equal(rb[:, s:s + 1], wb) and np.array_equal(rm[:, s:s + 1], wm)
        assert np.array_equal(b.get_spins(s, 0), pt.replica_spins(0))


def test_schedule_equals_plain_sweeps(gpu):
    sizes, R = [8, 16, 32], 4
    T = [4.4, 4.5, 4.6, 4.7]
    a = gpu.IsingBatch(sizes, R, seed=3)
    a.set_temperatures(T)
    a.step(70)
    c = gpu.IsingBatch(sizes, R, seed=3)
    c.set_temperatures(T)
    c.run_schedule(None, 70)
    for s in range(len(sizes)):
        for r in range(R):
            assert np.array_equal(a.get_spins(s, r), c.get_spins(s, r))
    assert a.sweep_counter() == c.sweep_counter() == 70


def test_schedule_rejects_bad_arguments(gpu):
    b = gpu.IsingBatch([8], 1, seed=1)
    with pytest.raises(gpu.IsingError):
        b.run_schedule(None, 5)          # temperatures not set
    with pytest.raises(gpu.IsingError):
        b.run_schedule([4.5, -1.0], None)
    b.set_temperatures([4.5])
    with pytest.raises(gpu.IsingError):
        b.run_schedule(None, 5, 2, 2)    # phase must be < every
