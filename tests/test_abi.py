"""The C-ABI library builds, loads and exports every declared entry point.

CPU only: nothing here launches GPU work.
"""
from __future__ import annotations

import ctypes
import os
import re
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))
           if f.endswith(".h")]


def declared_functions():
    names = []
    for h in HEADERS:
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"\b(hal_cuda_\w+)\s*\(", text)
    return sorted(set(names))


@pytest.fixture(scope="module")
def libpath():
    import halcuda

    if not os.path.exists(halcuda.LIB_PATH):
        subprocess.run([sys.executable, os.path.join(ROOT, "hal-cpp_gb300", "build.py")], check=True)
    return halcuda.LIB_PATH


def test_header_declares_the_boundary():
    names = declared_functions()
    for required in ("hal_cuda_diffuse", "hal_cuda_diffuse_adi", "hal_cuda_accumulate_forces",
                     "hal_cuda_agents_get_bins", "hal_cuda_last_error"):
        assert required in names


def test_library_exports_every_declared_symbol(libpath):
    lib = ctypes.CDLL(libpath)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"not exported: {missing}"


def test_binding_covers_every_declared_symbol():
    import halcuda

    assert sorted(halcuda.SIGNATURES) == declared_functions()


def test_version_without_gpu(libpath):
    import halcuda

    assert "sm_103a" in halcuda.version()
    assert halcuda.last_error() == ""


def test_build_targets_sm103a_only():
    sys.path.insert(0, os.path.join(ROOT, "hal-cpp_gb300"))
    import build

    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]
