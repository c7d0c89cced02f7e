"""The quench protocols: Kibble-Zurek ramps (`kz --gpu`, src/cuda/kz_gpu.rs)
and coarsening after a quench (`coarsening --gpu`, src/cuda/coarsening_gpu.rs)
— isg_kz_sweep / isg_coarsening, the Python mirror and the drop-in drivers.

CPU: the drivers' flag handling (messages and exit codes of src/bin/kz.rs and
src/bin/coarsening.rs; validation runs before any device call) and physics
checks of the oracle's replays.
GPU: bit-exact results against the oracle's replays, and the reference's own
CLI tests (tests/cli.rs:310-475, 862-877) with --gpu.
"""
from __future__ import annotations

import subprocess

import numpy as np
import pytest

from conftest import ROOT

BIN = ROOT / "ising-rs_gb300" / "bin"


def run(name, args):
    exe = BIN / name
    if not exe.exists():
        pytest.fail(f"{exe} not built")
    return subprocess.run([str(exe), *args], capture_output=True, text=True, timeout=600)


@pytest.mark.parametrize("args,frag", [
    (["--n", "1"], "Error: --n must be at least 2 (got 1)"),
    (["--tau-steps", "0"], "Error: --tau-steps must be at least 1"),
    (["--n", "4", "--tau-min", "10", "--tau-max", "100", "--tau-steps", "2", "--trials", "0"],
     "--trials must be at least 1"),
    (["--t-end", "0"], "Error: temperatures must be positive"),
    (["--freeze-temperature", "-1"], "Error: temperatures must be positive"),
    (["--tau-min", "0"], "Error: --tau-min must be >= 1 and <= --tau-max"),
    (["--tau-min", "50", "--tau-max", "10"], "Error: --tau-min must be >= 1 and <= --tau-max"),
    (["--geometry", "square", "--gpu"], "supports only --geometry cubic"),
    (["--n", "4"], "pass --gpu"),
    (["--gpu", "--n", "7"], "even size"),
    (["--trials", "x"], "Error: invalid value 'x' for --trials: invalid digit found in string"),
])
def test_kz_rejections(args, frag, tmp_path):
    r = run("kz", ["--outdir", str(tmp_path / "o"), *args])
    assert r.returncode == 1 and frag in r.stderr, r.stderr
    assert not (tmp_path / "o").exists()


@pytest.mark.parametrize("args,frag", [
    (["--n", "0"], "Error: --n must be at least 2 (got 0)"),
    (["--t-quench", "0"], "Error: temperatures must be positive"),
    (["--steps", "0"], "Error: --steps must be at least 1"),
    (["--sample-every", "0"], "Error: --sample-every must be at least 1"),
    (["--geometry", "hex"], "Error: unknown geometry 'hex' (expected: square, triangular, cubic)"),
    (["--n", "4"], "pass --gpu"),
    (["--gpu", "--n", "5"], "even size"),
])
def test_coarsening_rejections(args, frag, tmp_path):
    r = run("coarsening", ["--outdir", str(tmp_path / "o"), *args])
    assert r.returncode == 1 and frag in r.stderr, r.stderr
    assert not (tmp_path / "o").exists()


def test_help_texts():
    for name in ("kz", "coarsening"):
        r = run(name, ["-h"])
        assert r.returncode == 0 and "--gpu" in r.stderr and "--outdir" in r.stderr


def test_oracle_kz_slower_quench_fewer_walls(oracle):
    """Kibble-Zurek: a slower ramp through Tc leaves fewer domain walls; rho stays
    in [0, 1/2] in expectation and the error is a standard error over trials."""
    out = oracle.kz_sweep(8, 1.0, 6.0, 1.0, [2, 300], 4, 20, 0, 0.01, 42)
    assert 0.0 <= out[1, 0] < out[0, 0] <= 0.6
    assert np.all(out[:, 1] >= 0.0)


def test_oracle_coarsening_walls_decay(oracle):
    """After a quench from T = 10 to 0.5, rho starts near 1/2 (disorder) and
    decreases (Allen-Cahn coarsening)."""
    st, rho = oracle.coarsening(10, 1.0, 10.0, 0.5, 50, 400, 50, 3)
    assert np.array_equal(st, np.arange(8) * 50)
    assert rho[0] > rho[-1] and rho[0] < 0.5 and rho[-1] < 0.25


# ----------------------------------------------------------------------------- GPU


@pytest.mark.gpu
@pytest.mark.parametrize("n,taus,trials,warm,freeze", [
    (6, [3, 10, 25], 3, 4, 2),
    (8, [1, 7], 2, 0, 0),
    (20, [12], 4, 3, 1),
])
def test_kz_bit_exact_vs_oracle(gpu, oracle, n, taus, trials, warm, freeze):
    pts = gpu.run_kz_sweep_gpu(n, "cubic", 1.0, 6.0, 1.0, taus, trials,
                               gpu.KzProtocol(warm, freeze, 0.5), base_seed=42)
    want = oracle.kz_sweep(n, 1.0, 6.0, 1.0, taus, trials, warm, freeze, 0.5, 42)
    got = np.array([[p.rho, p.rho_err] for p in pts])
    assert [p.tau_q for p in pts] == taus and all(p.n_trials == trials for p in pts)
    assert np.array_equal(got, want), (got, want)


@pytest.mark.gpu
def test_coarsening_bit_exact_vs_oracle(gpu, oracle):
    cfg = gpu.CoarseningConfig(n=10, t_high=10.0, t_quench=0.5, warmup_sweeps=5, total_steps=37,
                               sample_every=4, seed=9)
    pts = gpu.run_coarsening_gpu(cfg)
    st, rho = oracle.coarsening(10, 1.0, 10.0, 0.5, 5, 37, 4, 9)
    assert [p.step for p in pts] == st.tolist()
    assert [p.rho for p in pts] == rho.tolist()


@pytest.mark.gpu
def test_kz_cli_reference_tests_with_gpu(gpu, tmp_path):
    """tests/cli.rs:310-417 (kz_writes_csv, kz_supports_single_tau_step) with --gpu."""
    r = run("kz", ["--n", "4", "--geometry", "cubic", "--tau-min", "10", "--tau-max", "100",
                   "--tau-steps", "3", "--trials", "2", "--seed", "1", "--outdir", str(tmp_path),
                   "--gpu"])
    assert r.returncode == 0, r.stderr
    lines = (tmp_path / "kz_N4.csv").read_text().strip().splitlines()
    assert lines[0] == "tau_q,rho,rho_err,n_trials" and len(lines) == 4
    assert [int(x.split(",")[0]) for x in lines[1:]] == [10, 32, 100]
    for line in lines[1:]:
        f = line.split(",")
        assert len(f) == 4 and 0.0 <= float(f[1]) <= 1.0 and 0.0 <= float(f[2]) <= 1.0
        assert int(f[3]) == 2
    pts = gpu.run_kz_sweep_gpu(4, "cubic", 1.0, 6.0, 1.0, [10, 32, 100], 2, base_seed=1)
    assert lines[1:] == [f"{p.tau_q},{p.rho:.8f},{p.rho_err:.8f},2" for p in pts]
    r = run("kz", ["--n", "4", "--geometry", "cubic", "--tau-min", "25", "--tau-max", "25",
                   "--tau-steps", "1", "--trials", "1", "--seed", "2", "--outdir",
                   str(tmp_path / "one"), "--gpu"])
    assert r.returncode == 0, r.stderr
    lines = (tmp_path / "one" / "kz_N4.csv").read_text().strip().splitlines()
    assert len(lines) == 2 and lines[1].startswith("25,")


@pytest.mark.gpu
def test_coarsening_cli_reference_test_with_gpu(gpu, tmp_path):
    """tests/cli.rs:441-475 (coarsening_writes_csv) with --gpu, and the CSV text
    against the library."""
    r = run("coarsening", ["--n", "4", "--geometry", "cubic", "--t-quench", "3.0", "--steps",
                           "50", "--sample-every", "25", "--warmup", "10", "--seed", "1",
                           "--outdir", str(tmp_path), "--gpu"])
    assert r.returncode == 0, r.stderr
    text = (tmp_path / "coarsening_N4_T3.00.csv").read_text()
    pts = gpu.run_coarsening_gpu(gpu.CoarseningConfig(n=4, t_quench=3.0, total_steps=50,
                                                      sample_every=25, warmup_sweeps=10, seed=1))
    assert text == "t,rho\n" + "".join(f"{p.step},{p.rho:.8f}\n" for p in pts)
    assert len(pts) == 2
