"""Shared test setup: the `gpu` marker, golden fixtures, library build."""
import ctypes
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


def _gpu_count() -> int:
    for name in ("libcudart.so", "libcudart.so.13", "/usr/local/cuda/lib64/libcudart.so"):
        try:
            rt = ctypes.CDLL(name)
        except OSError:
            continue
        n = ctypes.c_int(0)
        if rt.cudaGetDeviceCount(ctypes.byref(n)) == 0:
            return n.value
        return 0
    return 0


HAS_GPU = _gpu_count() > 0


def pytest_collection_modifyitems(config, items):
    if HAS_GPU:
        return
    skip = pytest.mark.skip(reason="no CUDA GPU in this environment")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def golden():
    with open(os.path.join(GOLDEN, "golden.json")) as f:
        return json.load(f)


def golden_dat(name: str) -> bytes:
    with open(os.path.join(GOLDEN, name + ".dat"), "rb") as f:
        return f.read()


def golden_rows(name: str):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def rel_l2(a, b) -> float:
    a = np.asarray(a)
    b = np.asarray(b)
    m = np.isfinite(a) & np.isfinite(b)
    return float(np.linalg.norm((a - b)[m]) / max(np.linalg.norm(b[m]), 1e-300))


@pytest.fixture(scope="session")
def lib_path():
    from sentinel1_decode_gb300 import build
    return build()
