"""The reweighting consumers of the PT timeseries (analysis/scripts/
reweighting.py, analysis/scripts/analyze_gpu_fss.py:86-243): device energy
histograms, GPU WHAM / single-histogram reweighting, and the binary timeseries
and histogram files.

CPU: the oracle's numpy restatement against golden vectors made by the
reference's own reweighting.py (tests/golden/make_reweight_golden.py), the
binary file layouts through the library's host-only writers, argument checks
made before any device call, and the gpu_fss flags.
GPU: the device reweighting against the golden vectors and the oracle (FP64;
relative 1e-9, the sums run in a different order), the histograms bit for bit
against the PT records, WHAM over exact-energy histograms against WHAM over
the samples, and the gpu_fss binary outputs against its text output and the
Python mirror.
"""
from __future__ import annotations

import csv
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

BIN = ROOT / "ising-rs_gb300" / "bin"


def golden():
    d = np.load(GOLDEN / "reweight_golden.npz")
    splits = np.cumsum(d["counts"])[:-1]
    return d, np.split(d["e"], splits), np.split(d["m"], splits)


def synthetic(seed=5, K=5, n=2000, V=512):
    """Overlapping PT-like samples: total energies and |m| per simulation."""
    rng = np.random.default_rng(seed)
    betas = np.linspace(0.21, 0.23, K)
    el, ml = [], []
    for b in betas:
        el.append(rng.normal(-0.9 * V - 9000.0 * (b - 0.21), 25.0, n))
        ml.append(np.clip(rng.normal(0.2 + 12.0 * (b - 0.21), 0.06, n), 0.0, 1.0))
    return el, ml, betas


# ----------------------------------------------------------------- CPU


def test_oracle_matches_reference_reweighting(oracle):
    d, el, ml = golden()
    b = d["betas"]
    np.testing.assert_allclose(oracle.rw_single_histogram(el[1], b[1], 0.2135), d["single_w"],
                               rtol=1e-12, atol=1e-300)
    w, sim = oracle.rw_wham(el, b, 0.2175)
    np.testing.assert_allclose(w, d["wham_w"], rtol=1e-10, atol=1e-300)
    assert np.array_equal(sim, d["sim_idx"])
    T, U = oracle.rw_binder(el, ml, b, d["targets"])
    np.testing.assert_allclose(T, d["T_out"], rtol=1e-15)
    np.testing.assert_allclose(U, d["U_out"], rtol=1e-12)
    assert abs(np.sum(np.concatenate(ml) * w) - float(d["obs_m"])) < 1e-12


def test_oracle_fine_tables_at_simulation_temperatures(oracle):
    """At a simulation's own temperature single-histogram reweighting is the
    plain sample average."""
    el, ml, b = synthetic()
    t = oracle.rw_single_fine(el, ml, b, 1.0 / b, 8)
    for k in range(len(b)):
        assert abs(t["M"][k] - ml[k].mean()) < 1e-12
        assert abs(t["E"][k] - el[k].mean() / 512) < 1e-12
    tw = oracle.rw_wham_fine(el, ml, b, [4.6, 4.65], 8)
    assert np.all(np.isfinite(tw["chi_err"])) and np.all(tw["U"] < 2.0 / 3.0)


def test_timeseries_file_round_trip(pkg, tmp_path):
    p = tmp_path / "ts.bin"
    temps = [4.4, 4.5, 4.6]
    ti = np.array([2, 0, 1, 1], np.int32)
    rp = np.array([0, 1, 2, 3], np.int32)
    E = np.array([-1.25, -1.5, -1.0 / 3.0, 0.0])
    M = np.array([0.5, 0.75, 1.0 / 7.0, 0.0])
    pkg.write_timeseries(p, "heisenberg", 16, temps, ti, rp, E, M)
    raw = p.read_bytes()
    assert raw[:8] == b"ISGTSER1" and len(raw) == 32 + 8 * 3 + 24 * 4
    ts = pkg.read_timeseries(p)
    assert ts["model"] == "heisenberg" and ts["n"] == 16
    assert np.array_equal(ts["temps"], temps)
    r = ts["records"]
    assert np.array_equal(r["temp_idx"], ti) and np.array_equal(r["replica"], rp)
    assert np.array_equal(r["E"], E) and np.array_equal(r["M"], M)
    el, ml, bl = pkg.timeseries_lists(ts)
    assert len(el) == 3 and np.array_equal(el[1], E[[2, 3]] * 16 ** 3)
    np.testing.assert_allclose(bl, 1.0 / np.array(temps))
    with pytest.raises(pkg.IsingError, match="temperature index out of range"):
        pkg.write_timeseries(tmp_path / "bad.bin", "ising", 8, temps, [3], [0], [0.0], [0.0])


def test_histogram_file_round_trip(pkg, tmp_path):
    import ctypes as C
    p = tmp_path / "h.bin"
    temps = np.array([4.4, 4.6])
    lo = np.array([-1536, -1500], np.int64)
    nb = np.array([2, 3], np.int64)
    cnt = np.arange(4 * 5, dtype=np.uint64) * np.uint64(2 ** 33)
    rc = pkg.lib().isg_hist_write(str(p).encode(), 3, 8, 1.5, temps.ctypes.data_as(C.c_void_p), 2,
                                  lo.ctypes.data_as(C.c_void_p), nb.ctypes.data_as(C.c_void_p),
                                  cnt.ctypes.data_as(C.c_void_p))
    assert rc == 0
    h = pkg.read_histograms(p)
    assert h["dim"] == 3 and h["n"] == 8 and h["J"] == 1.5
    assert np.array_equal(h["bonds"][0], [-1536, -1532])
    assert np.array_equal(h["bonds"][1], [-1500, -1496, -1492])
    assert np.array_equal(np.concatenate(h["counters"]).reshape(-1), cnt)


def test_reweighting_argument_checks(pkg):
    with pytest.raises(pkg.IsingError, match="need at least one point"):
        pkg.single_histogram(np.zeros(0), 0.2, 0.21)
    with pytest.raises(pkg.IsingError, match="every simulation needs samples"):
        pkg.wham_reweight([np.ones(3), np.zeros(0)], [0.2, 0.21], 0.2)


@pytest.mark.parametrize("args,frag", [
    (["--timeseries-format", "json"], "Error: --timeseries-format must be csv, bin or both"),
    (["--model", "xy", "--histograms"], "Error: --histograms needs --model ising"),
])
def test_gpu_fss_new_flag_rejections(args, frag, tmp_path):
    r = subprocess.run([str(BIN / "gpu_fss"), "--outdir", str(tmp_path / "o"), *args],
                       capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and frag in r.stderr, r.stderr
    assert not (tmp_path / "o").exists()


# ----------------------------------------------------------------- GPU


@pytest.mark.gpu
def test_gpu_reweighting_matches_reference_golden(gpu):
    d, el, ml = golden()
    b = d["betas"]
    np.testing.assert_allclose(gpu.single_histogram(el[1], b[1], 0.2135), d["single_w"],
                               rtol=1e-9, atol=1e-300)
    w, sim = gpu.wham_reweight(el, b, 0.2175)
    np.testing.assert_allclose(w, d["wham_w"], rtol=1e-9, atol=1e-300)
    assert np.array_equal(sim, d["sim_idx"])
    T, U = gpu.reweight_binder(el, ml, b, d["targets"])
    np.testing.assert_allclose(T, d["T_out"], rtol=1e-15)
    np.testing.assert_allclose(U, d["U_out"], rtol=1e-9)
    assert abs(gpu.reweight_observable(np.concatenate(ml), w) - float(d["obs_m"])) < 1e-9


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["single", "wham"])
def test_gpu_fine_tables_match_oracle(gpu, oracle, kind):
    el, ml, b = synthetic()
    T = np.linspace(4.35, 4.75, 41)
    if kind == "single":
        g = gpu.reweight_single_histogram(el, ml, b, T, 8)
        o = oracle.rw_single_fine(el, ml, b, T, 8)
    else:
        g = gpu.wham_reweight_fine(el, ml, b, T, 8)
        o = oracle.rw_wham_fine(el, ml, b, T, 8)
    for k in o:
        np.testing.assert_allclose(g[k], o[k], rtol=1e-8, atol=1e-12, err_msg=k)


def _records_histogram(rt, rb, rm, s, R, L):
    """Counters of size s accumulated from PT records as the device does."""
    N = float(L) ** 3
    dn = 3 * L ** 3
    out = {}
    sl = slice(s * R, (s + 1) * R)
    for t_row, b_row, m_row in zip(rt[:, sl], rb[:, sl], rm[:, sl]):
        for t, b, m in zip(t_row, b_row, m_row):
            assert (int(b) + dn) % 4 == 0
            m1 = abs(float(m)) / N
            m2 = m1 * m1
            m4 = m2 * m2
            c = out.setdefault((int(t), int(b)), [0, 0, 0, 0])
            c[0] += 1
            c[1] += int(np.rint(m1 * 4294967296.0))
            c[2] += int(np.rint(m2 * 4294967296.0))
            c[3] += int(np.rint(m4 * 4294967296.0))
    return out


@pytest.mark.gpu
def test_device_histograms_match_records(gpu):
    sizes, R = [4, 6, 8], 5
    b = gpu.IsingBatch(sizes, R, seed=17)
    temps = [4.2 + 0.15 * t for t in range(R)]
    b.set_temperatures(temps * len(sizes))
    b.step(30)
    b.reset_sampling()
    # a first chunk runs (and captures its cycle graph) before histograms exist
    b.pt_run(20, 5, 2)
    b.hist_enable()
    recs = [b.pt_run(n, 5, 2) for n in (37, 40, 23)]
    rt = np.concatenate([x[0] for x in recs])
    rb = np.concatenate([x[1] for x in recs])
    rm = np.concatenate([x[2] for x in recs])
    for s, L in enumerate(sizes):
        want = _records_histogram(rt, rb, rm, s, R, L)
        for t in range(R):
            bonds, cnt = b.histogram(s, t)
            got = {(t, int(bb)): [int(v) for v in c] for bb, c in zip(bonds, cnt) if c[0] > 0}
            exp = {k: v for k, v in want.items() if k[0] == t}
            assert got == exp, (L, t)
            assert min(k[1] for k in exp) == bonds[0] and max(k[1] for k in exp) == bonds[-1]
    b.hist_reset()
    assert b.histogram(0, 0)[0].size == 0
    b.hist_enable(False)


@pytest.mark.gpu
def test_wham_on_histograms_equals_wham_on_samples(gpu):
    L, R = 8, 6
    temps = [4.3 + 0.08 * t for t in range(R)]
    b = gpu.IsingBatch([L], R, seed=23)
    b.set_temperatures(temps)
    b.step(500)
    b.reset_sampling()
    b.hist_enable()
    rt, rb, rm = b.pt_run(6000, 10, 1)
    N = float(L) ** 3
    el = [(-rb[rt == t]).astype(np.float64) for t in range(R)]
    ml = [np.abs(rm[rt == t]).astype(np.float64) / N for t in range(R)]
    bonds, cnts = zip(*[b.histogram(0, t) for t in range(R)])
    T = np.linspace(4.3, 4.7, 21)
    h = gpu.wham_histograms(bonds, cnts, temps, 1.0, N, T)
    s = gpu.wham_reweight_fine(el, ml, 1.0 / np.array(temps), T, L)
    for k in ("E", "M", "M2", "M4", "U", "chi_conn", "Cv"):
        np.testing.assert_allclose(h[k], s[k], rtol=1e-8, atol=1e-10, err_msg=k)


@pytest.mark.gpu
def test_gpu_fss_binary_outputs(gpu, tmp_path):
    sizes, R, warm, samp, ee, seed = [4, 6], 4, 20, 60, 5, 11
    r = subprocess.run([str(BIN / "gpu_fss"), "--model", "ising", "--sizes", "4,6",
                        "--replicas", str(R), "--warmup", str(warm), "--samples", str(samp),
                        "--exchange-every", str(ee), "--seed", str(seed), "--tmin", "4.3",
                        "--tmax", "4.6", "--outdir", str(tmp_path), "--timeseries-format",
                        "both", "--histograms"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    temps = gpu.linspace_temperatures(4.3, 4.6, R)
    b = gpu.IsingBatch(sizes, R, seed=seed)
    b.set_temperatures(temps * 2)
    b.step(warm)
    b.reset_sampling()
    b.hist_enable()
    b.pt_run(samp, ee, 1)
    for s, L in enumerate(sizes):
        ts = gpu.read_timeseries(tmp_path / f"gpu_fss_ising_N{L}_timeseries.bin")
        assert ts["model"] == "ising" and ts["n"] == L
        with open(tmp_path / f"gpu_fss_ising_N{L}_timeseries.csv") as f:
            rows = list(csv.DictReader(f))
        rec = ts["records"]
        assert len(rows) == len(rec) == samp * R
        assert np.array_equal(rec["temp_idx"], [int(x["temp_idx"]) for x in rows])
        assert np.max(np.abs(rec["E"] - [float(x["E"]) for x in rows])) <= 5e-9
        assert np.max(np.abs(rec["M"] - [float(x["M"]) for x in rows])) <= 5e-9
        h = gpu.read_histograms(tmp_path / f"gpu_fss_ising_N{L}_hist.bin")
        assert np.allclose(h["temps"], temps)
        for t in range(R):
            bonds, cnt = b.histogram(s, t)
            assert np.array_equal(h["bonds"][t], bonds) and np.array_equal(h["counters"][t], cnt)
