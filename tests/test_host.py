"""CPU-only checks of the boundary: the C-ABI library loads and exports every
symbol include/isg.h declares, host statistics match the oracle bit for bit,
and host helpers mirror the reference."""
from __future__ import annotations

import ctypes
import re

import numpy as np
import pytest

from conftest import ROOT


def declared_symbols() -> list[str]:
    names = []
    for h in sorted((ROOT / "include").glob("*.h")):
        text = h.read_text()
        names += re.findall(r"^\s*(?:const\s+char\s*\*|int)\s+(isg_\w+)\s*\(", text, re.M)
    return names


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "isg_ising_create" in names and "isg_jackknife" in names
    assert len(names) == len(set(names))


def test_library_exports_every_declared_symbol(pkg):
    lib = ctypes.CDLL(str(pkg.library_path()))
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_version(pkg):
    assert pkg.lib().isg_version() == 100


def test_jackknife_bit_exact_vs_oracle(pkg, oracle):
    rng = np.random.default_rng(1)
    for n, nb in [(1000, 20), (20003, 20), (37, 20), (5, 5), (3, 20)]:
        e = rng.normal(-1.2, 0.05, n)
        m = np.abs(rng.normal(0.4, 0.1, n))
        a = pkg.jackknife_observables(e, m, 1 / 4.5, 4096.0, min(20, n) if nb == 20 else nb)
        b = oracle.jackknife(e, m, 1 / 4.5, 4096.0, min(20, n) if nb == 20 else nb)
        assert np.array_equal(a, b)


def test_jackknife_matches_numpy_restatement(pkg):
    """Independent numpy form of gpu_fss.rs:327-412."""
    rng = np.random.default_rng(2)
    e = rng.normal(-1.0, 0.1, 4000)
    m = np.abs(rng.normal(0.3, 0.1, 4000))
    beta, n3, nb = 0.22, 512.0, 20
    out = pkg.jackknife_observables(e, m, beta, n3, nb)
    bs = len(e) // nb
    e, m = e[:bs * nb], m[:bs * nb]

    def obs(e, m):
        return np.array([e.mean(), m.mean(), (m ** 2).mean(), (m ** 4).mean(),
                         beta ** 2 * ((e ** 2).mean() - e.mean() ** 2) * n3,
                         beta * ((m ** 2).mean() - m.mean() ** 2) * n3])

    full = obs(e, m)
    jk = np.array([obs(np.delete(e, slice(b * bs, (b + 1) * bs)),
                       np.delete(m, slice(b * bs, (b + 1) * bs))) for b in range(nb)])
    err = np.sqrt(((jk - full) ** 2).sum(0) * (nb - 1) / nb)
    np.testing.assert_allclose(out[0::2], full, rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(out[1::2], err, rtol=1e-8, atol=1e-14)


def test_linspace_temperatures(pkg):
    """parallel_tempering.rs:69-76."""
    t = pkg.linspace_temperatures(4.0, 5.0, 5)
    assert len(t) == 5 and abs(t[0] - 4.0) < 1e-10 and abs(t[4] - 5.0) < 1e-10
    assert abs(t[2] - 4.5) < 1e-10
    assert pkg.linspace_temperatures(4.4, 4.6, 1) == [4.4]


def test_binder_limits(pkg):
    """observables.rs:300-312: U4 -> 2/3 in the ordered phase."""
    assert abs(pkg.binder(1.0, 1.0) - 2.0 / 3.0) < 1e-12
    assert pkg.binder(0.0, 0.0) == 0.0


def test_create_rejects_bad_arguments_without_gpu(pkg):
    """Argument checks run before any device call."""
    with pytest.raises(pkg.IsingError) as ei:
        pkg.IsingBatch([7], 2)
    assert ei.value.status == -4 and "odd size" in str(ei.value)
    with pytest.raises(pkg.IsingError) as ei:
        pkg.IsingBatch([8, 8], 2)
    assert ei.value.status == -1
    with pytest.raises(pkg.IsingError):
        pkg.IsingBatch([8], 0)
    with pytest.raises(pkg.IsingError):
        pkg.IsingBatch([8], 2, dim=4)
