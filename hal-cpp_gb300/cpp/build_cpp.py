"""Builds the C++ layer above the C ABI.

    python hal-cpp_gb300/cpp/build_cpp.py [--hal-include DIR]

* hal-cpp_gb300/libhal_cuda_cpp.so -- the Hal::Cuda backend classes
  (src/CudaBackends2D.cpp) and the resident grid Hal::Cuda::CudaPDEGrid2D
  (src/CudaPDEGrid2D.cpp) with the stand-in interface declarations of
  compat/ (used when the backend is built outside a HAL-CPP tree), linked
  against libhal_cuda.so;
* hal-cpp_gb300/_build/cpp/backend_tests -- the test driver
  (tests/backend_tests.cpp), which also links the CPU oracle
  (oracle/liboracle.so) as its checker;
* hal-cpp_gb300/_build/cpp/interface_bench -- per-call times of the three
  interfaces against the CPU oracle (tests/interface_bench.cpp, run by
  bench.py);
* with --hal-include DIR (a HAL-CPP include directory): the backend classes
  are also compiled, syntax and types only, against HAL's own interface
  headers, which shows they drop in unchanged.

g++ only (C++20); no CUDA headers are needed above the C ABI.
"""
from __future__ import annotations

import argparse
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
ROOT = os.path.dirname(PKG)
INCLUDE = os.path.join(ROOT, "include")
ORACLE = os.path.join(ROOT, "oracle")
OUT_DIR = os.path.join(PKG, "_build", "cpp")
LIB = os.path.join(PKG, "libhal_cuda_cpp.so")
TEST_BIN = os.path.join(OUT_DIR, "backend_tests")
BENCH_BIN = os.path.join(OUT_DIR, "interface_bench")
CXXFLAGS = ["-std=c++20", "-O2", "-Wall", "-Wextra", "-fPIC"]


def _cxx():
    exe = shutil.which("g++") or shutil.which("c++")
    if not exe:
        raise RuntimeError("g++ not found")
    return exe


def _run(cmd):
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("command failed:\n" + " ".join(cmd) + "\n" + res.stdout + res.stderr)


def build_library():
    os.makedirs(OUT_DIR, exist_ok=True)
    _run([_cxx()] + CXXFLAGS + ["-shared", "-o", LIB,
          os.path.join(HERE, "src", "CudaBackends2D.cpp"), os.path.join(HERE, "src", "CudaPDEGrid2D.cpp"),
          os.path.join(HERE, "compat", "compat.cpp"),
          "-I", os.path.join(HERE, "include"), "-I", os.path.join(HERE, "compat"), "-I", INCLUDE,
          "-L", PKG, "-lhal_cuda", "-Wl,-rpath,$ORIGIN"])
    return LIB


def build_tests():
    oracle_so = os.path.join(ORACLE, "liboracle.so")
    if not os.path.exists(oracle_so):
        raise RuntimeError("oracle/liboracle.so is missing: build the oracle first")
    for src, out in (("backend_tests.cpp", TEST_BIN), ("interface_bench.cpp", BENCH_BIN)):
        _run([_cxx()] + CXXFLAGS + ["-o", out, os.path.join(HERE, "tests", src),
              "-I", os.path.join(HERE, "include"), "-I", os.path.join(HERE, "compat"), "-I", INCLUDE,
              "-I", ORACLE, "-L", PKG, "-lhal_cuda_cpp", "-lhal_cuda", "-L", ORACLE, "-loracle",
              "-Wl,-rpath," + PKG + ":" + ORACLE])
    return TEST_BIN


def check_against_hal(hal_include):
    """Compiles the backend classes against HAL's own headers (no output)."""
    for src in ("CudaBackends2D.cpp", "CudaPDEGrid2D.cpp"):
        _run([_cxx()] + CXXFLAGS + ["-fsyntax-only", os.path.join(HERE, "src", src),
              "-I", os.path.join(HERE, "include"), "-I", hal_include, "-I", INCLUDE])


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--hal-include", default=None)
    ap.add_argument("--no-tests", action="store_true")
    args = ap.parse_args(argv)
    print(build_library())
    if not args.no_tests:
        print(build_tests())
    if args.hal_include:
        check_against_hal(args.hal_include)
        print(f"backend classes compile against {args.hal_include}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
