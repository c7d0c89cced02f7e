"""Ising parallel tempering on a graph: `gpu_jfit --model ising`
(src/bin/gpu_jfit.rs:172-297, graphs from src/graph.rs) — isg_graph_*, the
Python mirror (GraphDef, GraphBatch) and the gpu_jfit drop-in driver.

CPU: the graph readers and builders, the greedy colouring, the oracle's two
algorithms (the device replay and the reference's random-site sweeps with one
shared generator) against exact enumeration, the device replay against the
reference algorithm, create-time validation (before any device call) and the
driver's flag handling.
GPU: records, spins, ladder and acceptance count bit-exact against the
oracle's replay on BCC, FCC and diluted cubic graphs (one graph above 32768
nodes), the reference algorithm's averages reproduced statistically, and the
driver's CSV reproduced from the Python mirror's records.
"""
from __future__ import annotations

import math
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT

BIN = ROOT / "ising-rs_gb300" / "bin"


def run(args):
    exe = BIN / "gpu_jfit"
    if not exe.exists():
        pytest.fail(f"{exe} not built")
    return subprocess.run([str(exe), *args], capture_output=True, text=True, timeout=600)


def exact_averages(n, edges, T, J=1.0):
    """<e>, <|m|>, <m^2> per node of the Ising model on a small graph by
    enumerating its 2^n states."""
    e = np.asarray(edges).reshape(-1, 2)
    s = 1 - 2 * ((np.arange(2 ** n)[:, None] >> np.arange(n)[None, :]) & 1)
    bond = (s[:, e[:, 0]] * s[:, e[:, 1]]).sum(1).astype(np.float64)
    mag = s.sum(1).astype(np.float64)
    E = -J * bond
    w = np.exp(-(E - E.min()) / T)
    w /= w.sum()
    return (w * E).sum() / n, (w * np.abs(mag)).sum() / n, (w * mag * mag).sum() / n / n


# a 9-node test graph: triangle-rich, degrees 2..5, not bipartite
SMALL_N = 9
SMALL_EDGES = [(0, 1), (1, 2), (2, 0), (2, 3), (3, 4), (4, 5), (5, 3), (5, 6), (6, 7),
               (7, 8), (8, 6), (0, 8), (1, 4), (2, 6)]


# ----------------------------------------------------------------- CPU


def test_graph_builders_match_reference_shapes(pkg):
    G = pkg.GraphDef
    g = G.bcc(4)
    assert g.n_nodes == 128 and len(g.edges) == 512 and set(g.degrees()) == {8}
    g = G.fcc(4)
    assert g.n_nodes == 256 and len(g.edges) == 1536 and set(g.degrees()) == {12}
    for p, m in [(0.0, 24000), (0.1, 21600), (0.3, 16800), (0.5, 12000)]:
        g = G.diluted_cubic(20, p, seed=7)
        assert g.n_nodes == 8000 and len(g.edges) == m and g.degrees().max() <= 6
    for g in (G.bcc(2), G.fcc(2), G.bcc(3), G.fcc(3)):
        key = np.sort(g.edges, 1)
        assert len(np.unique(key, axis=0)) == len(key), "duplicate bond"
        assert np.all(g.edges[:, 0] != g.edges[:, 1])
        assert len(g.edges) * 2 == g.degrees().sum()


def test_graph_readers(pkg):
    G = pkg.GraphDef
    g = G.from_json('{"n_nodes": 4, "edges": [[0,1],[1, 2], [2,3]]}')
    assert g.n_nodes == 4 and g.edges.tolist() == [[0, 1], [1, 2], [2, 3]]
    g2 = G.from_json(G.bcc(2).to_json())
    assert g2.n_nodes == 16 and np.array_equal(g2.edges, G.bcc(2).edges)
    for text, msg in [('{"edges": []}', "missing n_nodes"),
                      ('{"n_nodes": -1, "edges": []}', "missing n_nodes"),
                      ('{"n_nodes": 3}', "missing edges"),
                      ('{"n_nodes": 3, "edges": [5]}', "edge entry is not a 2-element array"),
                      ('{"n_nodes": 3, "edges": [[0,1,2]]}', "edge entry must have exactly 2"),
                      ('{"n_nodes": 3, "edges": [[0,1.5]]}', "edge index is not an integer")]:
        with pytest.raises(ValueError, match=msg):
            G.from_json(text)
    g = G.from_edge_csv("# comment\n0,1\n\n 1 , 5 \n")
    assert g.n_nodes == 6 and g.edges.tolist() == [[0, 1], [1, 5]]
    with pytest.raises(ValueError, match="bad edge line: 7"):
        G.from_edge_csv("0,1\n7\n")


def _greedy(n, edges):
    adj = [[] for _ in range(n)]
    for a, b in edges:
        adj[a].append(b)
        adj[b].append(a)
    col = [-1] * n
    for v in range(n):
        used = {col[u] for u in adj[v] if col[u] >= 0}
        c = 0
        while c in used:
            c += 1
        col[v] = c
    return col


@pytest.mark.parametrize("kind", ["small", "bcc3", "fcc2", "fcc3", "dil6"])
def test_colouring_proper_and_greedy(pkg, oracle, kind):
    G = pkg.GraphDef
    g = {"small": G(SMALL_N, SMALL_EDGES), "bcc3": G.bcc(3), "fcc2": G.fcc(2),
         "fcc3": G.fcc(3), "dil6": G.diluted_cubic(6, 0.3, seed=1)}[kind]
    k, col = oracle.graph_colouring(g.n_nodes, g.edges)
    assert col.tolist() == _greedy(g.n_nodes, g.edges.tolist())
    assert k == max(col) + 1
    assert np.all(col[g.edges[:, 0]] != col[g.edges[:, 1]])
    if kind == "bcc3":
        assert k == 2  # bipartite: corners first, then centres


@pytest.mark.parametrize("T", [2.5, 4.0])
def test_oracle_replay_matches_exact_enumeration(oracle, T):
    R, sweeps = 2, 60000
    pt = oracle.GraphPT(SMALL_N, SMALL_EDGES, R, [T, T], seed=11)
    pt.warmup(200)
    pt.reset_sampling()
    _, rb, rm = pt.sample(sweeps, 1 << 30, 1)
    e = -rb.astype(np.float64) / SMALL_N
    m = np.abs(rm.astype(np.float64)) / SMALL_N
    ee, em, _ = exact_averages(SMALL_N, SMALL_EDGES, T)
    blocks = 60
    for series, exact in ((e, ee), (m, em)):
        bm = series.reshape(blocks, -1, R).mean(axis=1).reshape(-1)
        err = bm.std(ddof=1) / math.sqrt(len(bm))
        assert abs(bm.mean() - exact) < 5 * err + 1e-3, (bm.mean(), exact, err)


@pytest.mark.parametrize("T", [2.5, 4.0])
def test_oracle_reference_algorithm_matches_exact_enumeration(oracle, T):
    R = 3
    out = oracle.graph_ref_pt(SMALL_N, SMALL_EDGES, [T] * R, 1.0, 5, 200, 60000, 1 << 30)
    ee, em, em2 = exact_averages(SMALL_N, SMALL_EDGES, T)
    cnt = out[:, 5]
    assert np.all(cnt == 60000)
    np.testing.assert_allclose(out[:, 0] / cnt, ee, atol=0.02)
    np.testing.assert_allclose(out[:, 2] / cnt, em, atol=0.015)
    np.testing.assert_allclose(out[:, 3] / cnt, em2, atol=0.015)


def test_oracle_replay_matches_reference_algorithm_on_bcc(pkg, oracle):
    """Colour-class sweeps with Philox against random-site sweeps with one
    shared Xoshiro256++: the same ladder, the same per-temperature averages."""
    g = pkg.GraphDef.bcc(3)
    temps = [5.0, 6.0, 7.0, 8.0]
    R, warm, samp, ee = len(temps), 500, 30000, 10
    ref = oracle.graph_ref_pt(g.n_nodes, g.edges, temps, 1.0, 3, warm, samp, ee)
    pt = oracle.GraphPT(g.n_nodes, g.edges, R, temps, seed=3)
    pt.warmup(warm)
    pt.reset_sampling()
    rt, rb, rm = pt.sample(samp, ee, 1)
    n = g.n_nodes
    for t in range(R):
        sel = rt == t
        e = (-rb[sel] / n).mean()
        m = (np.abs(rm[sel]) / n).mean()
        assert abs(e - ref[t, 0] / ref[t, 5]) < 0.03, (t, e, ref[t, 0] / ref[t, 5])
        assert abs(m - ref[t, 2] / ref[t, 5]) < 0.03, (t, m, ref[t, 2] / ref[t, 5])
    assert pt.accepted[0] > 0


@pytest.mark.parametrize("n,edges,R,frag", [
    (0, [], 2, "n_nodes must be 1..65536"),
    (65537, [], 2, "n_nodes must be 1..65536"),
    (3, [(0, 3)], 2, "names a node outside 0..2"),
    (3, [(1, 1)], 2, "self-loop at node 1"),
    (14, [(0, k) for k in range(1, 14)], 2, "node 0 has degree 13 (at most 12)"),
    (3, [(0, 1)], 0, "replicas must be 1..1024"),
    (3, [(0, 1)], 1025, "replicas must be 1..1024"),
])
def test_graph_create_rejections(pkg, n, edges, R, frag):
    with pytest.raises(pkg.IsingError, match=re.escape(frag)):
        pkg.GraphBatch(n, np.array(edges, np.int32).reshape(-1, 2), R)


@pytest.mark.parametrize("args,frag", [
    ([], "Error: --graph <path.json> is required"),
    (["--graph", "g.json", "--tmin", "0"], "Error: --tmin must be positive (got 0)"),
    (["--graph", "g.json", "--tmin", "7", "--tmax", "6"],
     "Error: --tmin (7) must be less than --tmax (6)"),
    (["--graph", "g.json", "--warmup", "0"], "Error: --warmup must be at least 1"),
    (["--graph", "g.json", "--samples", "0"], "Error: --samples must be at least 1"),
    (["--graph", "g.json", "--replicas", "x"],
     "Error: invalid value 'x' for --replicas: invalid digit found in string"),
    (["--graph", "missing.json"],
     "Error: failed to read graph file missing.json: No such file or directory (os error 2)"),
])
def test_jfit_rejections(args, frag, tmp_path):
    r = subprocess.run([str(BIN / "gpu_jfit"), "--outdir", str(tmp_path / "o"), *args],
                       capture_output=True, text=True, timeout=60, cwd=tmp_path)
    assert r.returncode == 1 and frag in r.stderr, r.stderr
    assert not (tmp_path / "o").exists()


def test_jfit_bad_json_and_models(pkg, tmp_path):
    bad = tmp_path / "bad.json"
    bad.write_text('{"n_nodes": 4}')
    r = run(["--graph", str(bad), "--outdir", str(tmp_path / "o")])
    assert r.returncode == 101 and "failed to parse graph JSON: missing edges" in r.stderr
    good = tmp_path / "ring.json"
    good.write_text(pkg.GraphDef(4, [(0, 1), (1, 2), (2, 3), (3, 0)]).to_json())
    for model, frag in [("potts", "Error: --model must be ising, xy, or heisenberg")]:
        r = run(["--graph", str(good), "--model", model, "--outdir", str(tmp_path / "o")])
        assert r.returncode == 1 and frag in r.stderr, r.stderr
        assert f"jfit: model={model}, graph=ring, N=4, T=6..6.7, replicas=20, " \
               "exchange_every=10" in r.stderr


# ----------------------------------------------------------------- GPU


def _graphs(pkg):
    G = pkg.GraphDef
    return {"bcc4": G.bcc(4), "fcc4": G.fcc(4), "dil6": G.diluted_cubic(6, 0.3, seed=2),
            "small": G(SMALL_N, SMALL_EDGES), "dil34": G.diluted_cubic(34, 0.1, seed=3)}


@pytest.mark.gpu
@pytest.mark.parametrize("kind,R,warm,chunks,ee,me", [
    ("bcc4", 8, 7, [(23, 3, 2), (16, 3, 2)], 3, 2),
    ("fcc4", 5, 3, [(30, 4, 1)], 4, 1),
    ("dil6", 6, 0, [(9, 2, 3), (14, 2, 3), (1, 2, 3)], 2, 3),
    ("small", 3, 11, [(40, 1, 1)], 1, 1),
    ("dil34", 2, 2, [(5, 2, 1)], 2, 1),
])
def test_graph_bit_exact_vs_oracle(gpu, oracle, kind, R, warm, chunks, ee, me):
    g = _graphs(gpu)[kind]
    temps = [4.0 + 3.0 * t / max(R - 1, 1) for t in range(R)]
    b = gpu.GraphBatch(g.n_nodes, g.edges, R, seed=99)
    pt = oracle.GraphPT(g.n_nodes, g.edges, R, temps, seed=99)
    k, _ = oracle.graph_colouring(g.n_nodes, g.edges)
    assert b.num_colours() == k
    for r in range(R):
        assert np.array_equal(b.get_spins(r), pt.replica_spins(r)), "hot start differs"
    b.set_temperatures(temps)
    b.step(warm)
    pt.warmup(warm)
    b.reset_sampling()
    pt.reset_sampling()
    for n, ee_, me_ in chunks:
        rt, rb, rm = b.pt_run(n, ee_, me_)
        ot, ob, om = pt.sample(n, ee_, me_)
        assert np.array_equal(rt, ot) and np.array_equal(rb, ob) and np.array_equal(rm, om)
    for r in range(R):
        assert np.array_equal(b.get_spins(r), pt.replica_spins(r)), f"replica {r}"
    assert np.array_equal(b.r2t(), pt.r2t)
    assert b.accepted() == int(pt.accepted[0])


@pytest.mark.gpu
def test_graph_matches_reference_algorithm_statistically(gpu, oracle):
    g = gpu.GraphDef.bcc(3)
    temps = [5.0, 6.0, 7.0, 8.0]
    R, warm, samp, ee = len(temps), 500, 40000, 10
    ref = oracle.graph_ref_pt(g.n_nodes, g.edges, temps, 1.0, 5, warm, samp, ee)
    b = gpu.GraphBatch(g.n_nodes, g.edges, R, seed=5)
    b.set_temperatures(temps)
    b.step(warm)
    b.reset_sampling()
    rt, rb, rm = b.pt_run(samp, ee, 1)
    n = g.n_nodes
    for t in range(R):
        sel = rt == t
        assert sel.sum() == samp
        e = (-rb[sel] / n).mean()
        m = (np.abs(rm[sel]) / n).mean()
        assert abs(e - ref[t, 0] / ref[t, 5]) < 0.03
        assert abs(m - ref[t, 2] / ref[t, 5]) < 0.03


@pytest.mark.gpu
def test_jfit_cli_csv_matches_mirror(gpu, tmp_path):
    g = gpu.GraphDef.bcc(4)
    path = tmp_path / "bcc_N4.json"
    path.write_text(g.to_json())
    R, warm, samp, ee, seed = 6, 50, 300, 7, 17
    r = run(["--graph", str(path), "--outdir", str(tmp_path / "out"), "--replicas", str(R),
             "--warmup", str(warm), "--samples", str(samp), "--exchange-every", str(ee),
             "--seed", str(seed), "--tmin", "6", "--tmax", "6.7", "--unknown-flag"])
    assert r.returncode == 0, r.stderr
    text = (tmp_path / "out" / "gpu_jfit_ising_bcc_N4.csv").read_text()
    temps = gpu.linspace_temperatures(6.0, 6.7, R)
    b = gpu.GraphBatch(g.n_nodes, g.edges, R, seed=seed)
    b.set_temperatures(temps)
    b.step(warm)
    b.reset_sampling()
    rt, rb, rm = b.pt_run(samp, ee, 1)
    n = float(g.n_nodes)
    acc = np.zeros((R, 5))
    cnt = np.zeros(R, np.int64)
    for row in range(len(rt)):
        for rr in range(R):
            t = rt[row, rr]
            e_per = -(1.0 * float(rb[row, rr])) / n
            m_per = abs(float(rm[row, rr]) / n)
            acc[t, 0] += e_per
            acc[t, 1] += e_per * e_per
            acc[t, 2] += m_per
            acc[t, 3] += m_per * m_per
            acc[t, 4] += (m_per * m_per) * (m_per * m_per)
            cnt[t] += 1
    lines = ["T,E,E_err,M,M_err,M2,M2_err,M4,M4_err,Cv,Cv_err,chi,chi_err"]
    for t in range(R):
        s = float(cnt[t])
        beta = 1.0 / temps[t]
        ae, ae2, am, am2, am4 = (acc[t, k] / s for k in range(5))
        cv = beta * beta * (ae2 - ae * ae) * n
        chi = beta * (am2 - am * am) * n
        lines.append(f"{temps[t]:.4f},{ae:.6f},0.0,{am:.6f},0.0,{am2:.6f},0.0,{am4:.6f},0.0,"
                     f"{cv:.6f},0.0,{chi:.6f},0.0")
    assert text == "\n".join(lines) + "\n"
    assert f"PT exchanges accepted: {b.accepted()}" in r.stderr
    assert "jfit: model=ising, graph=bcc_N4, N=128, T=6..6.7, replicas=6, " \
           "exchange_every=7" in r.stderr


@pytest.mark.gpu
def test_exchange_barrier_waits_are_bounded(gpu):
    """The grid barrier of the persistent graph runs: released when every block
    arrives, and when a block never arrives (one more expected than launched)
    every wait runs out after its cycle limit and reports it, with the GPU left
    usable (a plain run follows)."""
    import ctypes as C
    L = gpu.lib()
    flag = C.c_int(-1)
    assert L.isg_barrier_selftest(4, 4, 1 << 30, C.byref(flag)) == 0 and flag.value == 0
    assert L.isg_barrier_selftest(4, 5, 1 << 21, C.byref(flag)) == 0 and flag.value == 1
    g = gpu.GraphDef.bcc(2)
    b = gpu.GraphBatch(g.n_nodes, g.edges, 3, seed=1)
    b.set_temperatures([5.0, 6.0, 7.0])
    rt, _, _ = b.pt_run(20, 5, 1)
    assert rt.shape == (20, 3)
