"""Shared fixtures: the product package (loaded from ising-rs_gb300/), the CPU
oracle (oracle/oracle.py, test infrastructure) and golden-table readers."""
from __future__ import annotations

import csv
import importlib.util
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
GOLDEN = Path(__file__).resolve().parent / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libisinggb")


def _load(name: str, path: Path, package: bool = False):
    if name in sys.modules:
        return sys.modules[name]
    spec = importlib.util.spec_from_file_location(
        name, path, submodule_search_locations=[str(path.parent)] if package else None)
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


def load_pkg():
    return _load("ising_gb300", ROOT / "ising-rs_gb300" / "__init__.py", package=True)


def load_oracle():
    return _load("isg_oracle", ROOT / "oracle" / "oracle.py")


@pytest.fixture(scope="session")
def pkg():
    return load_pkg()


@pytest.fixture(scope="session")
def oracle():
    return load_oracle()


_GPU = None


def gpu_available() -> bool:
    global _GPU
    if _GPU is None:
        try:
            import torch
            _GPU = bool(torch.cuda.is_available())
        except Exception:
            _GPU = False
    return _GPU


@pytest.fixture(scope="session")
def gpu(pkg):
    """Skips without a GPU; on a GPU machine the library must load (no fallback)."""
    if not gpu_available():
        pytest.skip("no CUDA device")
    pkg.lib()
    return pkg


def read_csv(name: str) -> list[dict]:
    with open(GOLDEN / name) as f:
        return [{k: float(v) if _isnum(v) else v for k, v in row.items()}
                for row in csv.DictReader(f)]


def _isnum(v: str) -> bool:
    try:
        float(v)
        return True
    except ValueError:
        return False


def golden_summary(model: str, L: int) -> dict[str, np.ndarray]:
    rows = read_csv(f"gpu_fss_{model}_N{L}_summary.csv")
    return {k: np.array([r[k] for r in rows]) for k in rows[0]}
