"""Golden vectors of the reference's reweighting functions.

Usage: python make_reweight_golden.py <path of a faulknco/ising-rs checkout>.
Imports analysis/scripts/reweighting.py from that checkout (numpy only) and evaluates single_histogram,
wham_reweight and reweight_binder on seeded synthetic PT-like samples: four
simulations at beta = 0.20..0.23 with overlapping Gaussian total energies and
|m| values.  Writes tests/golden/reweight_golden.npz (inputs and outputs);
tests read only that file.
"""
import importlib.util
import sys
from pathlib import Path

import numpy as np

if len(sys.argv) != 2:
    sys.exit(f"usage: python {Path(__file__).name} <reference checkout>")
REF = Path(sys.argv[1])
OUT = Path(__file__).resolve().parent / "reweight_golden.npz"

spec = importlib.util.spec_from_file_location(
    "ref_reweighting", REF / "analysis" / "scripts" / "reweighting.py")
rw = importlib.util.module_from_spec(spec)
spec.loader.exec_module(rw)

rng = np.random.default_rng(20260308)
betas = np.array([0.20, 0.21, 0.22, 0.23])
counts = [400, 380, 420, 400]
e_lists, m_lists = [], []
for b, n in zip(betas, counts):
    e_lists.append(rng.normal(-600.0 - 4000.0 * (b - 0.2), 40.0, n))
    m_lists.append(np.clip(rng.normal(0.3 + 5.0 * (b - 0.2), 0.05, n), 0.0, 1.0))
single_w = rw.single_histogram(e_lists[1], betas[1], 0.2135)
wham_w, sim_idx = rw.wham_reweight(e_lists, betas, 0.2175)
targets = np.array([0.2025, 0.2075, 0.2125, 0.2175, 0.2225])
T_out, U_out = rw.reweight_binder(e_lists, m_lists, betas, targets)
obs_m = rw.reweight_observable(np.concatenate(m_lists), wham_w)
np.savez_compressed(OUT, betas=betas, counts=np.array(counts),
                    e=np.concatenate(e_lists), m=np.concatenate(m_lists),
                    single_w=single_w, wham_w=wham_w, sim_idx=sim_idx, targets=targets,
                    T_out=T_out, U_out=U_out, obs_m=np.array(obs_m))
print("wrote", OUT, OUT.stat().st_size, "bytes")
