"""Build the GB300 EVoC library (and the CPU oracle used by the tests).

    python evoc-rs_gb300/build.py            # library + oracle
    python evoc-rs_gb300/build.py --lib      # library only

The library is compiled in-tree for sm_103a only, one nvcc process per
translation unit in parallel, and linked into libevoc_gb300.so next to this
file. The CUDA runtime is linked statically so the .so only needs the driver.
"""
from __future__ import annotations

import argparse
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libevoc_gb300.so"
ORACLE_SRCS = [ROOT / "oracle" / "evoc_oracle.cpp", ROOT / "oracle" / "evoc_labels_oracle.cpp"]
ORACLE_LIB = ROOT / "oracle" / "liboracle.so"

SOURCES = ["primitives.cu", "fuzzy_set.cu", "embed.cu", "capi.cu", "noalloc.cu", "measure.cu", "mlp.cu",
           "label_prop.cu", "lp_init.cu", "mst.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
    "-Xcompiler", "-ffp-contract=off",  # host arithmetic as written (no FMA contraction)
    "-Xptxas", "-warn-spills",
]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"command failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    if res.stderr.strip():
        sys.stderr.write(res.stderr)


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build_library(verbose: bool = False, extra: list[str] | None = None) -> Path:
    BUILD.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + [ROOT / "include" / "evoc_gb300.h"]
    cc = nvcc()
    objs = []
    jobs = []
    for src in SOURCES:
        s = CSRC / src
        o = BUILD / (src + ".o")
        objs.append(o)
        if _stale(o, [s] + headers):
            cmd = [cc, *ARCH, *NVCC_FLAGS, *(extra or []), "-c", str(s), "-o", str(o)]
            jobs.append(cmd)
    with ThreadPoolExecutor(max_workers=len(jobs) or 1) as ex:
        for f in [ex.submit(_run, j) for j in jobs]:
            f.result()
    if jobs or _stale(LIB, objs):
        _run([cc, *ARCH, "-shared", "-cudart", "static", "-o", str(LIB), *map(str, objs)])
    if verbose:
        print(f"built {LIB}")
    return LIB


def build_oracle(verbose: bool = False) -> Path:
    """The oracle is test infrastructure: built for the tests and the CPU baseline."""
    if _stale(ORACLE_LIB, ORACLE_SRCS):
        cxx = os.environ.get("CXX", "g++")
        _run([cxx, "-O3", "-std=c++17", "-fPIC", "-shared", "-fopenmp",
              "-ffp-contract=off", "-o", str(ORACLE_LIB), *map(str, ORACLE_SRCS)])
    if verbose:
        print(f"built {ORACLE_LIB}")
    return ORACLE_LIB


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--lib", action="store_true", help="library only")
    ap.add_argument("--oracle", action="store_true", help="oracle only")
    a = ap.parse_args()
    if not a.oracle:
        build_library(verbose=True)
    if not a.lib:
        build_oracle(verbose=True)


if __name__ == "__main__":
    main()
