"""Build recipe for libisinggb (sm_103a) and the drop-in drivers (gpu_fss, fss, kz,
coarsening, gpu_jfit).

Compiles every translation unit in parallel with one -gencode
(arch=compute_103a,code=sm_103a), links lib/libisinggb.so and bin/<driver> in the package
directory.  Host code is compiled with -ffp-contract=off so the
FP64 threshold tables, exchange energies and jackknife sums round the same on
x86_64 and aarch64.

Usage: python ising-rs_gb300/build.py  (or build_all() from Python)
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
INCLUDE = PKG.parent / "include"
BUILD = PKG / "_build"
LIB = PKG / "lib"
BIN = PKG / "bin"

ARCH = "-gencode=arch=compute_103a,code=sm_103a"
NVCC_FLAGS = [
    ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
    "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr",
]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall"]

CU_SOURCES = ["isg_ising.cu", "isg_cont.cu", "isg_noalloc.cu", "isg_learned.cu", "isg_graph.cu",
              "isg_cgraph.cu", "isg_reweight.cu"]
CPP_SOURCES = ["isg_stats.cpp", "isg_anneal.cpp", "isg_quench.cpp", "isg_io.cpp"]
DRIVERS = ["gpu_fss", "fss", "kz", "coarsening", "gpu_jfit"]   # host/<name>.cpp -> bin/<name>


def _cuda_home() -> Path:
    env = os.environ.get("CUDA_HOME") or os.environ.get("CUDA_PATH")
    if env:
        return Path(env)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    return Path("/usr/local/cuda")


def _run_parallel(cmds: list[list[str]]) -> None:
    procs = [(c, subprocess.Popen(c, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)) for c in cmds]
    errors = []
    for c, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            errors.append(" ".join(c) + "\n" + out.decode(errors="replace"))
    if errors:
        raise RuntimeError("build failed:\n" + "\n\n".join(errors))


def build_all(verbose: bool = False) -> Path:
    """Compile the library and the driver; returns the path of the .so."""
    cuda = _cuda_home()
    nvcc = str(cuda / "bin" / "nvcc") if (cuda / "bin" / "nvcc").exists() else "nvcc"
    cxx = os.environ.get("CXX", "g++")
    BUILD.mkdir(exist_ok=True)
    LIB.mkdir(exist_ok=True)
    BIN.mkdir(exist_ok=True)
    inc = ["-I", str(INCLUDE), "-I", str(CSRC)]
    cmds, objs = [], []
    for src in CU_SOURCES:
        if not (CSRC / src).exists():
            continue
        obj = BUILD / (Path(src).stem + ".o")
        cmds.append([nvcc, *NVCC_FLAGS, *inc, "-c", str(CSRC / src), "-o", str(obj)])
        objs.append(obj)
    for src in CPP_SOURCES:
        obj = BUILD / (Path(src).stem + ".o")
        cmds.append([cxx, *CXX_FLAGS, *inc, "-I", str(cuda / "include"), "-c", str(CSRC / src),
                     "-o", str(obj)])
        objs.append(obj)
    if verbose:
        for c in cmds:
            print(" ".join(c), file=sys.stderr)
    _run_parallel(cmds)
    so = LIB / "libisinggb.so"
    _run_parallel([[nvcc, ARCH, "-shared", "-o", str(so), *map(str, objs)]])
    drivers = [[cxx, *CXX_FLAGS, "-I", str(INCLUDE), str(PKG / "host" / f"{name}.cpp"), "-o",
                str(BIN / name), "-L", str(LIB), "-lisinggb", "-Wl,-rpath,$ORIGIN/../lib"]
               for name in DRIVERS]
    _run_parallel(drivers)
    return so


if __name__ == "__main__":
    print(build_all(verbose=True))
