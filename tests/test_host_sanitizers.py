"""Host code under AddressSanitizer and UndefinedBehaviorSanitizer.

The ADI line plan (hal-cpp_gb300/csrc/adi_plan.cpp) is the library's largest
piece of host arithmetic: the FP64 elimination, the coupling vectors, the
banded inverse of the reduced system and the periodic correction, with their
own index arithmetic.  The driver tests/sanitize/plan_driver.cpp builds it with
g++ -fsanitize=address,undefined for every line-length class (one chunk,
partial last chunks, the 4096 maximum), rates from 1e-3 to 100 and every end
condition, and checks sizes and self-checks; the sanitizers abort on any
out-of-bounds access, overflow or other undefined behaviour.  CPU only.
"""
from __future__ import annotations

import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "hal-cpp_gb300", "csrc")
DRIVER = os.path.join(ROOT, "tests", "sanitize", "plan_driver.cpp")


def test_adi_plan_under_asan_ubsan(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not found")
    exe = str(tmp_path / "plan_driver")
    cmd = [cxx, "-std=c++17", "-O1", "-g", "-fno-omit-frame-pointer", "-ffp-contract=off",
           "-fsanitize=address,undefined", "-fno-sanitize-recover=all", "-I", CSRC,
           DRIVER, os.path.join(CSRC, "adi_plan.cpp"), "-o", exe]
    build = subprocess.run(cmd, capture_output=True, text=True)
    if build.returncode != 0 and "asan" in (build.stderr + build.stdout).lower():
        pytest.skip("sanitizer runtime not available: " + build.stderr[-200:])
    assert build.returncode == 0, build.stderr
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:abort_on_error=1",
               UBSAN_OPTIONS="print_stacktrace=1:halt_on_error=1")
    run = subprocess.run([exe], capture_output=True, text=True, env=env, timeout=600)
    assert run.returncode == 0, run.stdout + run.stderr
    assert run.stdout.startswith("ok "), run.stdout
