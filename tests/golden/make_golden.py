"""Copies the reference's committed result tables into tests/golden/.

Usage: python make_golden.py <path of a faulknco/ising-rs checkout>.  Sources:
  analysis/data/gpu_windows_pipeline/publication/gpu_fss_{ising,heisenberg,xy}_N*_summary.csv
      PT summaries from the reference's own GPU path (scripts/run_gpu_publication.sh:22-50)
  results/published/classical_validation_full_v1/analysis/data/derived/validation/*.csv
      exact-enumeration, Onsager and known-limit tables (analysis/scripts/reproduce_validation.py)
The files are copied byte for byte; tests read only these copies.
"""
import shutil
import sys
from pathlib import Path

if len(sys.argv) != 2:
    sys.exit(f"usage: python {Path(__file__).name} <reference checkout>")
REF = Path(sys.argv[1])
OUT = Path(__file__).resolve().parent

pub = REF / "analysis/data/gpu_windows_pipeline/publication"
for f in sorted(pub.glob("gpu_fss_*_summary.csv")):
    shutil.copyfile(f, OUT / f.name)
val = REF / "results/published/classical_validation_full_v1/analysis/data/derived/validation"
for name in ["exact_enumeration_comparison.csv", "onsager_comparison.csv",
             "known_limits_summary.csv", "validation_metrics.csv"]:
    shutil.copyfile(val / name, OUT / name)
print("copied to", OUT)
