"""The gpu_fss drop-in driver: flag validation, messages and exit codes of
src/bin/gpu_fss.rs / src/cli.rs (checked without a GPU: validation runs before
any device call), plus the reference's own GPU smoke test (tests/cli.rs:677-728)
and CSV formats on a GPU."""
from __future__ import annotations

import subprocess

import numpy as np
import pytest

from conftest import ROOT

BIN = ROOT / "ising-rs_gb300" / "bin" / "gpu_fss"


def run(args, cwd=None):
    if not BIN.exists():
        pytest.fail(f"{BIN} not built")
    return subprocess.run([str(BIN), *args], capture_output=True, text=True, cwd=cwd, timeout=600)


@pytest.mark.parametrize("args,frag", [
    (["--tmin", "5", "--tmax", "4"], "Error: --tmin (5) must be less than --tmax (4)"),
    (["--tmin", "-1"], "Error: --tmin must be positive (got -1)"),
    (["--tmax", "0"], "Error: --tmax must be positive (got 0)"),
    (["--tmin", "4.4", "--tmax", "4.4"], "Error: --tmin (4.4) must be less than --tmax (4.4)"),
    (["--samples", "0"], "Error: --samples must be at least 1"),
    (["--warmup", "0"], "Error: --warmup must be at least 1"),
    (["--measure-every", "0"], "Error: --measure-every must be at least 1"),
    (["--replicas", "abc"], "Error: invalid value 'abc' for --replicas: invalid digit found in string"),
    (["--replicas", "-3"], "Error: invalid value '-3' for --replicas: invalid digit found in string"),
    (["--tmin", "x"], "Error: invalid value 'x' for --tmin: invalid float literal"),
    (["--seed", ""], "Error: invalid value '' for --seed: cannot parse integer from empty string"),
    (["--warmup"], "Error: --warmup requires a value"),
])
def test_rejections(args, frag, tmp_path):
    r = run(["--outdir", str(tmp_path), *args])
    assert r.returncode == 1 and frag in r.stderr, r.stderr


def test_unknown_model(tmp_path):
    r = run(["--model", "potts", "--outdir", str(tmp_path)])
    assert r.returncode == 1
    assert "Error: --model must be ising, xy, or heisenberg" in r.stderr
    assert "GPU FSS: model=potts, sizes=[8, 16, 32, 64], T=4.4..4.6, replicas=20" in r.stderr


def test_odd_size_rejected(tmp_path):
    r = run(["--sizes", "7", "--outdir", str(tmp_path)])
    assert r.returncode == 1 and "even size" in r.stderr


def test_unknown_flags_ignored_and_bad_sizes_dropped(tmp_path):
    r = run(["--bogus", "--sizes", "x,,y", "--outdir", str(tmp_path)])
    assert r.returncode == 0, r.stderr
    assert "sizes=[]" in r.stderr


@pytest.mark.gpu
def test_gpu_fss_ising_smoke(gpu, tmp_path):
    """The reference's gpu_fss_ising_smoke (tests/cli.rs:677-728)."""
    r = run(["--model", "ising", "--sizes", "4", "--tmin", "4.4", "--tmax", "4.6", "--replicas",
             "4", "--warmup", "50", "--samples", "100", "--exchange-every", "10", "--outdir",
             str(tmp_path)])
    assert r.returncode == 0, r.stderr
    summary = (tmp_path / "gpu_fss_ising_N4_summary.csv").read_text().splitlines()
    assert len(summary) >= 2 and summary[0].startswith("T,E,")
    assert summary[0] == "T,E,E_err,M,M_err,M2,M2_err,M4,M4_err,Cv,Cv_err,chi,chi_err"
    ts = (tmp_path / "gpu_fss_ising_N4_timeseries.csv").read_text().splitlines()
    assert ts[0] == "temp_idx,E,M" and len(ts) == 1 + 100 * 4
    t, e, m = ts[1].split(",")
    assert len(e.split(".")[1]) == 8 and len(m.split(".")[1]) == 8
    assert "NaN" not in "".join(summary)


@pytest.mark.gpu
@pytest.mark.parametrize("model", ["xy", "heisenberg"])
def test_gpu_fss_continuous_smoke(gpu, tmp_path, model):
    r = run(["--model", model, "--sizes", "4,6", "--tmin", "1.3", "--tmax", "1.6", "--replicas",
             "4", "--warmup", "20", "--samples", "60", "--measure-every", "3", "--outdir",
             str(tmp_path)])
    assert r.returncode == 0, r.stderr
    for n in (4, 6):
        s = (tmp_path / f"gpu_fss_{model}_N{n}_summary.csv").read_text().splitlines()
        assert len(s) == 5 and all(len(row.split(",")) == 13 for row in s)
        ts = (tmp_path / f"gpu_fss_{model}_N{n}_timeseries.csv").read_text().splitlines()
        assert len(ts) == 1 + 20 * 4


@pytest.mark.gpu
def test_gpu_fss_matches_library_records(gpu, oracle, tmp_path):
    """The driver's timeseries equal the oracle's replay of the same run
    (seed 42, all sizes in one batch) formatted as gpu_fss.rs:264."""
    r = run(["--model", "ising", "--sizes", "8,4", "--tmin", "4.4", "--tmax", "4.6",
             "--replicas", "4", "--warmup", "30", "--samples", "40", "--exchange-every", "10",
             "--measure-every", "5", "--outdir", str(tmp_path)])
    assert r.returncode == 0, r.stderr
    temps = [4.4 + (4.6 - 4.4) * i / 3 for i in range(4)]
    for L in (8, 4):
        pt = oracle.IsingPT(L, 3, 4, temps, 42)
        pt.warmup(30)
        pt.reset_sampling()
        ot, ob, om = pt.sample(40, 10, 5)
        n3 = float(L ** 3)
        want = ["temp_idx,E,M"] + [f"{ot[i, rr]},{-ob[i, rr] / n3:.8f},{abs(om[i, rr]) / n3:.8f}"
                                   for i in range(ot.shape[0]) for rr in range(4)]
        got = (tmp_path / f"gpu_fss_ising_N{L}_timeseries.csv").read_text().splitlines()
        assert got == want
