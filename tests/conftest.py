"""Shared test setup: the `gpu` marker, the CPU oracle, golden fixtures."""
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libqsm_gb300.so")


def _ensure_oracle():
    lib = os.path.join(ROOT, "oracle", "liborc.so")
    src = os.path.join(ROOT, "oracle", "qsm_oracle.c")
    if not os.path.exists(lib) or os.path.getmtime(lib) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)


@pytest.fixture(scope="session")
def port():
    _ensure_oracle()
    import port as _port
    return _port


@pytest.fixture(scope="session")
def golden():
    cache = {}

    def load(name):
        if name not in cache:
            cache[name] = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
        return cache[name]
    return load


@pytest.fixture(scope="session")
def qsm():
    import qsm_gb300
    return qsm_gb300


@pytest.fixture(scope="session")
def gpu_ctx(qsm):
    """A library context on device 0; loading the CUDA library is mandatory."""
    import qsm_gb300.build as b
    b.build()
    return qsm.context(0)


def bits_equal(a, b):
    a = np.ascontiguousarray(np.asarray(a))
    b = np.ascontiguousarray(np.asarray(b))
    return a.shape == b.shape and a.dtype == b.dtype and np.array_equal(a.view(np.uint8), b.view(np.uint8))


def first_diff(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    d = np.abs(a - b)
    idx = np.argwhere(~((a == b) | (np.isnan(a) & np.isnan(b))))
    return f"max|diff|={np.nanmax(d) if d.size else 0:.3e} first={idx[:3].tolist()}"
