"""Golden vectors of the reference's integrated-autocorrelation-time estimator.

Usage: python make_tau_golden.py <path of a faulknco/ising-rs checkout>.
analysis/scripts/reproduce_validation.py of that checkout defines `autocorrelation` and `integrated_autocorrelation_time`
(the windowed estimator with the self-consistent 6 tau window) but imports
matplotlib and pandas at module level, which are not installed here.  So this
script parses the file and executes only those two function definitions (numpy
only), evaluates them on seeded synthetic series (AR(1) chains of several
correlation times and a sticky two-level chain), and writes
tests/golden/tau_golden.npz (series and tau values); tests read only that file.
"""
import ast
import sys
from pathlib import Path

import numpy as np

if len(sys.argv) != 2:
    sys.exit(f"usage: python {Path(__file__).name} <reference checkout>")
REF = Path(sys.argv[1])
OUT = Path(__file__).resolve().parent / "tau_golden.npz"
WANT = {"autocorrelation", "integrated_autocorrelation_time"}

src = (REF / "analysis" / "scripts" / "reproduce_validation.py").read_text()
tree = ast.parse(src)
defs = [n for n in tree.body if isinstance(n, ast.FunctionDef) and n.name in WANT]
assert {d.name for d in defs} == WANT
ns = {"np": np}
mod = ast.fix_missing_locations(ast.Module(body=defs, type_ignores=[]))
exec(compile(mod, "reproduce_validation.py", "exec"), ns)

rng = np.random.default_rng(20260311)
n = 4000
series = []
for rho in (0.0, 0.5, 0.9, 0.98):
    e = rng.standard_normal(n) * np.sqrt(1 - rho * rho)
    x = np.empty(n)
    x[0] = rng.standard_normal()
    for i in range(1, n):
        x[i] = rho * x[i - 1] + e[i]
    series.append(x)
# sticky two-level chain: rare switches between 0.7 and 0.4 plus noise
lvl = np.where(np.cumsum(rng.random(n) < 0.003) % 2 == 0, 0.7, 0.4)
series.append(lvl + 0.05 * rng.standard_normal(n))
series = np.array(series)
tau = np.array([ns["integrated_autocorrelation_time"](ns["autocorrelation"](x)) for x in series])
np.savez_compressed(OUT, series=series, tau=tau)
print("wrote", OUT, OUT.stat().st_size, "bytes; tau =", tau)
