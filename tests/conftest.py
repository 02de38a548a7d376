import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
PKG = ROOT / "evoc-rs_gb300"
sys.path.insert(0, str(PKG))
sys.path.insert(0, str(ROOT / "oracle"))
sys.path.insert(0, str(ROOT / "tests"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs an sm_103 GPU and the built CUDA library")


def ensure_library() -> Path:
    lib = PKG / "libevoc_gb300.so"
    if not lib.exists():
        subprocess.run([sys.executable, str(PKG / "build.py"), "--lib"], check=True)
    return lib


@pytest.fixture(scope="session")
def oracle():
    import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def ctx():
    ensure_library()
    import evoc_gb300 as E
    c = E.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="session")
def golden():
    g = ROOT / "tests" / "golden"
    return {name: np.load(g / f"{name}.npz") for name in ("smooth_knn", "fuzzy_set", "embedding")}


@pytest.fixture(scope="session")
def blobs_knn():
    """10,000 x 384 blobs on the sphere (20 clusters, sigma 0.15), cosine kNN k = 15."""
    import workloads as W
    x, labels = W.blobs_sphere_np(10_000, 384, 20, 0.15, seed=42)
    idx, dist = W.knn_np(x, 15)
    return idx, dist, labels


@pytest.fixture(scope="session")
def small_knn():
    """2,000 x 64 blobs, k = 15 (fast on CPU)."""
    import workloads as W
    x, labels = W.blobs_sphere_np(2_000, 64, 8, 0.1, seed=5)
    idx, dist = W.knn_np(x, 15)
    return idx, dist, labels
