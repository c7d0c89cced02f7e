"""Statistical checks of the continuous oracle on the CPU.

The oracle's checkerboard XY Metropolis (the device's CMETRO words: sites of
colour index 2j and 2j+1 share Philox block j, words 0/2 and 1/3) samples the
Boltzmann distribution: on a periodic 4^3 lattice its mean energy per site agrees
with the reference's own XY algorithm (single-cluster Wolff, run_xy_jfit,
gpu_jfit.rs:410-524) on the same lattice as a graph, within 5 standard errors; the
O(3) checkerboard oracle agrees with the reference CPU Heisenberg path."""
from __future__ import annotations

import numpy as np
import pytest


def _cubic_edges(L):
    idx = lambda x, y, z: (z * L + y) * L + x  # noqa: E731  (natural index, x fastest)
    e = []
    for z in range(L):
        for y in range(L):
            for x in range(L):
                i = idx(x, y, z)
                e += [(i, idx((x + 1) % L, y, z)), (i, idx(x, (y + 1) % L, z)),
                      (i, idx(x, y, (z + 1) % L))]
    return np.array(e, np.int32)


def _block_err(x, nb=20):
    B = len(x) // nb
    return x[:B * nb].reshape(nb, B).mean(1).std(ddof=1) / np.sqrt(nb)


@pytest.mark.parametrize("T", [1.6, 3.0])
def test_xy_checkerboard_metropolis_matches_wolff(oracle, T):
    L, nc, seed, n = 4, 2, 17, 64
    beta = 1.0 / T
    s = oracle.cont_hot_start(L, nc, seed, 0)
    es = []
    for k in range(42000):
        for colour in (0, 1):
            oracle.cont_metropolis(s, L, nc, colour, seed, 0, k, beta, 1.0, np.pi)
        if k >= 2000:
            es.append(oracle.cont_measure(s, L, nc)[0] / n)
    es = np.array(es)
    ref = oracle.cgraph_ref_pt(n, _cubic_edges(L), nc, [T], 1.0, seed, 2000, 40000, 10 ** 9)
    e_ref = ref[0, 0] / ref[0, 5]
    var_ref = ref[0, 1] / ref[0, 5] - e_ref ** 2
    err_ref = np.sqrt(max(var_ref, 0.0) / ref[0, 5]) * 3.0  # Wolff samples: tau of a few
    err = np.hypot(_block_err(es), err_ref)
    assert abs(es.mean() - e_ref) < 5 * err, (T, es.mean(), e_ref, err)


@pytest.mark.parametrize("T", [1.0, 2.0])
def test_heisenberg_checkerboard_matches_reference_cpu_path(oracle, T):
    """O(3): the checkerboard oracle (cone Metropolis + overrelaxation per colour,
    the device's algorithm) and the reference's CPU path (random-site cone
    Metropolis then sequential overrelaxation, heisenberg/sweep.rs:50-62) agree
    on the mean energy per site of a 4^3 lattice within 5 standard errors."""
    L, nc, seed, n, delta = 4, 3, 23, 64, 0.6
    beta = 1.0 / T
    a = oracle.cont_hot_start(L, nc, seed, 0)
    b = a.copy()
    ea, eb = [], []
    for k in range(22000):
        for colour in (0, 1):
            oracle.cont_metropolis(a, L, nc, colour, seed, 0, k, beta, 1.0, delta)
        for colour in (0, 1):
            oracle.cont_overrelax(a, L, nc, colour, 1.0)
        oracle.cont_ref_sweep(b, L, beta, 1.0, delta, seed, k, 1)
        if k >= 2000:
            ea.append(oracle.cont_measure(a, L, nc)[0] / n)
            eb.append(oracle.cont_measure(b, L, nc)[0] / n)
    ea, eb = np.array(ea), np.array(eb)
    err = np.hypot(_block_err(ea), _block_err(eb))
    assert abs(ea.mean() - eb.mean()) < 5 * err, (T, ea.mean(), eb.mean(), err)
