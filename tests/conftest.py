"""Shared test setup.

* registers the ``gpu`` marker (tests that need a CUDA device);
* puts ``oracle/`` and ``hal-cpp_gb300/`` on sys.path;
* builds the CPU oracle (``oracle/liboracle.so``) once per session, and the
  CUDA library when a GPU test needs it and it is missing.
"""
from __future__ import annotations

import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "hal-cpp_gb300"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


@pytest.fixture(scope="session")
def oracle():
    import pyoracle

    pyoracle.build(ref=False)
    return pyoracle.Oracle


@pytest.fixture(scope="session")
def golden():
    def load(name):
        return np.load(os.path.join(GOLDEN, name + ".npz"))

    return load


@pytest.fixture(scope="session")
def hal():
    """The CUDA library binding; builds libhal_cuda.so if it is missing."""
    import halcuda

    if not os.path.exists(halcuda.LIB_PATH):
        subprocess.run([sys.executable, os.path.join(ROOT, "hal-cpp_gb300", "build.py")], check=True)
    halcuda.lib()
    if halcuda.device_count() < 1:
        pytest.fail("no CUDA device visible to libhal_cuda.so")
    return halcuda


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (den if den > 0 else 1.0))


def max_rel(a, b):
    """max |a-b| / max |b| (scale-aware maximum error)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.abs(b).max() if b.size else 1.0
    return float(np.abs(a - b).max() / (den if den > 0 else 1.0)) if b.size else 0.0
