"""Test-side helpers: turn PT records into the reference's per-temperature
summary (gpu_fss.rs:253-262 accumulation order, :294-320 jackknife)."""
from __future__ import annotations

import numpy as np

from conftest import load_oracle


def pt_summary(rec_t, rec_e_total, rec_m, L, temps, dim=3, n_comp_m=False):
    """rec_t/rec_e_total/rec_m: (records, R) arrays for one size, replica order.
    rec_m holds the integer magnetisation (or |M| already, if n_comp_m)."""
    oracle = load_oracle()
    n = float(L ** dim)
    R = rec_t.shape[1]
    ts = [[] for _ in range(R)]
    for row in range(rec_t.shape[0]):
        for r in range(R):
            m = rec_m[row, r] if n_comp_m else abs(float(rec_m[row, r]))
            ts[int(rec_t[row, r])].append((rec_e_total[row, r] / n, m / n))
    keys = ["E", "E_err", "M", "M_err", "M2", "M2_err", "M4", "M4_err", "Cv", "Cv_err", "chi",
            "chi_err"]
    out = {k: np.zeros(R) for k in keys}
    for t in range(R):
        a = np.array(ts[t])
        o = oracle.jackknife(a[:, 0], a[:, 1], 1.0 / temps[t], n, min(20, len(a)))
        for i, k in enumerate(keys):
            out[k][t] = o[i]
    out["T"] = np.array(temps)
    return out
