"""The annealing finite-size-scaling path (`fss --gpu`: src/cuda/fss_gpu.rs:7-39,
src/bin/fss.rs) — isg_fss_anneal, the Python mirror (run_fss_gpu,
LatticeGpu.measure / domain_wall_density) and the `fss` drop-in driver.

CPU: the driver's flag handling (src/cli.rs messages and exit codes; validation
runs before any device call) and the oracle's replay of the schedule.
GPU: bit-exact observables against the oracle's replay, the reference's own
CLI test (tests/cli.rs:131-186) with --gpu, CSV text against the library, and
the annealed averages against the reference's published PT summaries.
"""
from __future__ import annotations

import subprocess

import numpy as np
import pytest

from conftest import ROOT, golden_summary

BIN = ROOT / "ising-rs_gb300" / "bin" / "fss"


def run(args, cwd=None):
    if not BIN.exists():
        pytest.fail(f"{BIN} not built")
    return subprocess.run([str(BIN), *args], capture_output=True, text=True, cwd=cwd, timeout=600)


@pytest.mark.parametrize("args,frag", [
    (["--steps", "1"], "Error: --steps must be at least 2 (got 1)"),
    (["--tmin", "5", "--tmax", "4"], "Error: --tmin (5) must be less than --tmax (4)"),
    (["--tmin", "0"], "Error: --tmin must be positive (got 0)"),
    (["--samples", "0"], "Error: --samples must be at least 1"),
    (["--warmup", "0"], "Error: --warmup must be at least 1"),
    (["--sizes", "8,1"], "Error: --n must be at least 2 (got 1)"),
    (["--samples", "1e3"], "Error: invalid value '1e3' for --samples: invalid digit found in string"),
    (["--j", "abc"], "Error: invalid value 'abc' for --j: invalid float literal"),
    (["--geometry", "hex"], "Error: unknown geometry 'hex' (expected: square, triangular, cubic)"),
    (["--seed"], "Error: --seed requires a value"),
    (["--gpu", "--sizes", "9"], "even size"),
    (["--sizes", "8"], "pass --gpu"),
    (["--raw", "--gpu"], "Warning: --raw mode does not support --gpu; ignoring --gpu"),
])
def test_rejections(args, frag, tmp_path):
    r = run(["--outdir", str(tmp_path / "o"), *args])
    assert r.returncode == 1 and frag in r.stderr, r.stderr
    assert not (tmp_path / "o").exists()


def test_help_and_unknown_flags(tmp_path):
    r = run(["--help"])
    assert r.returncode == 0 and "--sizes" in r.stderr and "--gpu" in r.stderr
    # a known flag skips the next argument, so '--bogus2' after '--gpu' is not reported
    r = run(["--bogus", "--gpu", "--bogus2", "--steps", "1"])
    assert r.returncode == 1
    assert "Warning: unknown flag '--bogus' (ignored)" in r.stderr
    assert "--bogus2" not in r.stderr


def test_oracle_schedule_shape_and_limits(oracle):
    """The replayed schedule: ascending T rows on the T grid of fss_gpu.rs:20-21,
    and the high-temperature series of the simple-cubic Ising model (t = tanh beta):
    <e> = -3t + O(t^3), N<m^2> = 1 + 6t + 30t^2 + 150t^3 + ..., chi = beta N <m^2>.
    (At much higher T the checkerboard update accepts almost every flip and
    decorrelates slowly, so the check stays at T = 20..40.)"""
    out = oracle.fss_anneal([4, 6], 3, 20.0, 40.0, 3, 1.0, 0.0, 50, 3000, 5)
    assert out.shape == (2, 3, 7)
    assert np.array_equal(out[0, :, 0], [20.0, 20.0 + 20.0 * 1 / 2, 40.0])
    for i, n3 in enumerate((64.0, 216.0)):
        beta = 1.0 / out[i, :, 0]
        t = np.tanh(beta)
        series = 1 + 6 * t + 30 * t * t + 150 * t ** 3
        np.testing.assert_allclose(out[i, :, 1], -3 * t, atol=0.015)
        np.testing.assert_allclose(out[i, :, 3] * n3, series, rtol=0.15)
        np.testing.assert_allclose(out[i, :, 6], beta * series, rtol=0.15)
    # m^4 <= m^2 <= 1 per sample carries to the averages
    assert np.all(out[:, :, 4] <= out[:, :, 3]) and np.all(out[:, :, 3] <= 1.0)


def test_oracle_observables_formula(oracle):
    """measure_observables restates lattice_gpu.rs:205-251 term by term."""
    bond = np.array([-100, -96, -120, 12], np.int64)
    mag = np.array([30, -28, 64, 0], np.int64)
    n3, T, J, h = 64.0, 4.5, 1.0, 0.25
    row = oracle.measure_observables(T, bond, mag, J, h, n3)
    e = (-J * bond - h * mag) / n3
    m = np.abs(mag / n3)
    ms = mag / n3
    beta = 1.0 / T
    want = [T, e.mean(), m.mean(), (m * m).mean(), (m * m * m * m).mean(),
            beta * beta * ((e * e).mean() - e.mean() ** 2) * n3,
            beta * ((ms * ms).mean() - ms.mean() ** 2) * n3]
    np.testing.assert_allclose(row, want, rtol=1e-12, atol=1e-12)


# ----------------------------------------------------------------------------- GPU


@pytest.mark.gpu
@pytest.mark.parametrize("sizes,dim,J,h", [
    ([4, 6, 8, 16], 3, 1.0, 0.0),
    ([8, 32, 64], 2, 0.5, 0.25),
])
def test_anneal_bit_exact_vs_oracle(gpu, oracle, sizes, dim, J, h):
    cfg = gpu.FssConfig(sizes=sizes, j=J, h=h, t_min=3.9 if dim == 3 else 2.0,
                        t_max=4.9 if dim == 3 else 2.6, t_steps=4, warmup_sweeps=6,
                        sample_sweeps=11, seed=7)
    got = gpu.run_fss_gpu(cfg, dim=dim)
    want = oracle.fss_anneal(sizes, dim, cfg.t_min, cfg.t_max, cfg.t_steps, J, h,
                             cfg.warmup_sweeps, cfg.sample_sweeps, cfg.seed)
    for i, (n, rows) in enumerate(got):
        assert n == sizes[i]
        arr = np.array([[o.temperature, o.energy, o.magnetisation, o.m2, o.m4,
                         o.heat_capacity, o.susceptibility] for o in rows])
        assert np.array_equal(arr, want[i]), (n, arr, want[i])


@pytest.mark.gpu
def test_repeated_and_many_sizes(gpu, oracle):
    """A repeated size repeats its rows; more than 16 distinct sizes run in groups
    without changing any size's stream."""
    sizes = [4, 6, 4] + list(range(8, 42, 2))
    cfg = gpu.FssConfig(sizes=sizes, t_min=4.0, t_max=5.0, t_steps=2, warmup_sweeps=2,
                        sample_sweeps=3, seed=11)
    got = {}
    for n, rows in gpu.run_fss_gpu(cfg):
        arr = np.array([[o.temperature, o.energy, o.magnetisation, o.m2, o.m4,
                         o.heat_capacity, o.susceptibility] for o in rows])
        if n in got:
            assert np.array_equal(got[n], arr)
        got[n] = arr
    for n in (4, 40):
        want = oracle.fss_anneal([n], 3, 4.0, 5.0, 2, 1.0, 0.0, 2, 3, 11)[0]
        assert np.array_equal(got[n], want)


@pytest.mark.gpu
def test_lattice_gpu_measure_and_domain_walls(gpu, oracle):
    """LatticeGpu::measure (lattice_gpu.rs:190-251) and domain_wall_density
    (:253-281) on the mirror, against the oracle replay and the reference's host
    wall count on the copied spins."""
    lat = gpu.LatticeGpu(8, 3)
    obs = lat.measure(4.5, 1.0, 0.0, 40)
    pt = oracle.IsingPT(8, 3, 1, [4.5], 3)
    _, b, m = pt.sample(40, 41, 1)
    want = oracle.measure_observables(4.5, b[:, 0], m[:, 0], 1.0, 0.0, 512.0)
    got = [obs.temperature, obs.energy, obs.magnetisation, obs.m2, obs.m4,
           obs.heat_capacity, obs.susceptibility]
    assert got == want
    s = lat.get_spins().reshape(8, 8, 8).astype(np.int64)
    walls = sum(int((s != np.roll(s, -1, axis=a)).sum()) for a in range(3))
    assert lat.domain_wall_density() == walls / (3 * 512)


@pytest.mark.gpu
def test_fss_cli_reference_test_with_gpu(gpu, tmp_path):
    """tests/cli.rs:131-186 (fss_writes_csv_files) with --gpu added."""
    r = run(["--sizes", "4,6", "--geometry", "cubic", "--wolff", "--samples", "10", "--warmup",
             "10", "--tmin", "3.0", "--tmax", "5.0", "--steps", "3", "--seed", "1", "--outdir",
             str(tmp_path), "--gpu"])
    assert r.returncode == 0, r.stderr
    for n in (4, 6):
        lines = (tmp_path / f"fss_N{n}.csv").read_text().strip().splitlines()
        assert lines[0] == "T,E,M,M2,M4,Cv,chi"
        assert len(lines) == 4
        assert all(len(line.split(",")) == 7 for line in lines[1:])


@pytest.mark.gpu
def test_fss_cli_csv_text_matches_library(gpu, tmp_path):
    args = dict(sizes=[8, 10], t_min=4.2, t_max=4.8, t_steps=5, warmup_sweeps=20,
                sample_sweeps=30, seed=99)
    r = run(["--gpu", "--sizes", "8,10", "--tmin", "4.2", "--tmax", "4.8", "--steps", "5",
             "--warmup", "20", "--samples", "30", "--seed", "99", "--outdir", str(tmp_path)])
    assert r.returncode == 0, r.stderr
    assert "GPU mode: CUDA checkerboard Metropolis" in r.stderr and "FSS GPU: N=10" in r.stderr
    for n, rows in gpu.run_fss_gpu(gpu.FssConfig(**args)):
        text = "T,E,M,M2,M4,Cv,chi\n" + "".join(
            f"{o.temperature:.4f},{o.energy:.6f},{o.magnetisation:.6f},{o.m2:.6f},{o.m4:.6f},"
            f"{o.heat_capacity:.6f},{o.susceptibility:.6f}\n" for o in rows)
        assert (tmp_path / f"fss_N{n}.csv").read_text() == text


@pytest.mark.gpu
def test_annealed_averages_vs_reference_pt_summaries(gpu):
    """On the grid of the reference's publication run (32 T on [4.40, 4.62]), the
    annealed <e> and <|m|> of L = 8 and 16 agree with the committed gpu_fss
    summaries (100k-sweep PT) within the statistical error of 20k samples."""
    cfg = gpu.FssConfig(sizes=[8, 16], t_min=4.40, t_max=4.62, t_steps=32,
                        warmup_sweeps=2000, sample_sweeps=20000, seed=42)
    for n, rows in gpu.run_fss_gpu(cfg):
        g = golden_summary("ising", n)
        e = np.array([o.energy for o in rows])
        m = np.array([o.magnetisation for o in rows])
        np.testing.assert_allclose([o.temperature for o in rows], g["T"], atol=5e-7)
        de, dm = e - g["E"], m - g["M"]
        assert np.max(np.abs(de)) < 0.05 and np.max(np.abs(dm)) < 0.06, (n, de, dm)
        assert abs(de.mean()) < 0.008 and abs(dm.mean()) < 0.012, (n, de.mean(), dm.mean())
