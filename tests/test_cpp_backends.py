"""The Hal::Cuda C++ backend classes (hal-cpp_gb300/cpp/).

* CPU: the classes and their test driver build with g++; where HAL-CPP's own
  headers are present, the classes also compile against HAL's interface
  declarations (the drop-in check).
* GPU: the driver runs the reference's interface test cases
  (IDiffusionBackend2DTests.cpp, IAgentForceBackend2DTests.cpp,
  AdiKernel2DTests.cpp) through IDiffusionBackend2D& / IAdiDiffusionBackend2D& /
  IAgentForceBackend2D& and exits 0 only if all pass.
"""
from __future__ import annotations

import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CPP = os.path.join(ROOT, "hal-cpp_gb300", "cpp")
sys.path.insert(0, CPP)


@pytest.fixture(scope="module")
def built(oracle, hal_lib_built):
    import build_cpp

    return build_cpp.build_library(), build_cpp.build_tests()


@pytest.fixture(scope="module")
def hal_lib_built():
    import halcuda

    if not os.path.exists(halcuda.LIB_PATH):
        subprocess.run([sys.executable, os.path.join(ROOT, "hal-cpp_gb300", "build.py")], check=True)
    return halcuda.LIB_PATH


def test_cpp_layer_builds(built):
    lib, test_bin = built
    assert os.path.exists(lib) and os.path.exists(test_bin)


def test_classes_compile_against_hal_interfaces():
    import build_cpp
    import pyoracle

    hal_include = os.path.join(pyoracle.REF_TREE, "include")
    if not os.path.isdir(hal_include):
        pytest.skip("HAL-CPP headers not present on this machine")
    build_cpp.check_against_hal(hal_include)


@pytest.mark.gpu
def test_backend_driver_passes(built, hal):
    _, test_bin = built
    res = subprocess.run([test_bin], capture_output=True, text=True, timeout=300)
    print(res.stdout)
    assert res.returncode == 0, res.stdout + res.stderr
    assert "0 failed" in res.stdout
