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
    """Relative L2 error of `a` (the array under test) against `b`.

    Both arrays must be finite everywhere: a NaN or Inf in the output under
    test is a failure, never a masked-out element."""
    a = np.asarray(a)
    b = np.asarray(b)
    assert a.shape == b.shape, (a.shape, b.shape)
    bad = np.count_nonzero(~np.isfinite(a))
    assert bad == 0, "%d non-finite values in the output under test" % bad
    assert np.isfinite(b).all(), "non-finite values in the reference array"
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.fixture(scope="session")
def lib_path():
    from sentinel1_decode_gb300 import build
    return build()


def golden_extras():
    """Reference outputs of eccm(), scale(), spectrogram() and
    sinc_interpolate() (tests/golden/make_extra_golden.py)."""
    return dict(np.load(os.path.join(GOLDEN, "extras.npz")))
