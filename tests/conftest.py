"""Shared test setup: the `gpu` marker, imports of the package (whose
directory name is not an identifier) and of the oracle (test infrastructure),
and the golden fixtures."""
from __future__ import annotations

import glob
import importlib
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def pkg():
    return importlib.import_module("2dfmm_gb300")


def workloads():
    return importlib.import_module("2dfmm_gb300.workloads")


def oracle():
    import oracle as O  # noqa: WPS433
    return O


def golden_names():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))


def load_golden(name):
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    return {k: d[k] for k in d.files}


@pytest.fixture(scope="session")
def lib():
    """The built library (compiled for sm_103a on first use)."""
    P = pkg()
    P.build()
    return P.load()


@pytest.fixture(scope="session")
def gpu_lib(lib):
    P = pkg()
    import ctypes
    try:
        cudart = ctypes.CDLL("libcudart.so")
        n = ctypes.c_int(0)
        ok = cudart.cudaGetDeviceCount(ctypes.byref(n)) == 0 and n.value > 0
    except OSError:
        ok = False
    if not ok:
        pytest.fail("GPU test run without a usable CUDA device")
    return P


def rel_err(a, b):
    """Per-component relative error, with the normwise fallback for
    components far below their target's velocity magnitude."""
    a = np.asarray(a).reshape(-1, 2)
    b = np.asarray(b).reshape(-1, 2)
    mag = np.linalg.norm(b, axis=1, keepdims=True)
    return np.abs(a - b) / np.maximum(np.abs(b), 1e-300), np.abs(a - b) / np.maximum(mag, 1e-300)
