"""Builds libhal_cuda.so in place (sm_103a only).

    python hal-cpp_gb300/build.py            # incremental
    python hal-cpp_gb300/build.py --force    # rebuild everything

Each translation unit of csrc/ is compiled by nvcc in parallel, then linked
into hal-cpp_gb300/libhal_cuda.so (CUDA runtime linked statically).  No
cmake; a few seconds per unit.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OBJ = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libhal_cuda.so")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Host code is compiled without floating-point contraction: the FP64 host
# precomputations that must round as the reference's CPU code does (the
# PDEGrid2D ADI plan) stay unfused on every host architecture.
NVFLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
                  "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr", "-I", INCLUDE, "-I", CSRC]

SOURCES = ["core.cu", "diffusion.cu", "adi.cu", "adi_plan.cpp", "agents.cu", "wells.cu", "adjoint.cu", "pde_io.cpp",
           "tick_blocked.cu", "pdegrid.cu"]


def _nvcc():
    exe = shutil.which("nvcc")
    if exe is None:
        cand = "/usr/local/cuda/bin/nvcc"
        if os.path.exists(cand):
            return cand
        raise RuntimeError("nvcc not found")
    return exe


def _newer(src, dst, deps):
    if not os.path.exists(dst):
        return True
    t = os.path.getmtime(dst)
    return any(os.path.getmtime(p) > t for p in [src] + deps)


def _compile(src, force, extra):
    nvcc = _nvcc()
    path = os.path.join(CSRC, src)
    obj = os.path.join(OBJ, os.path.splitext(src)[0] + ".o")
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    deps += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    if not force and not _newer(path, obj, deps):
        return obj, ""
    cmd = [nvcc] + NVFLAGS + extra + ["-c", path, "-o", obj]
    if src.endswith(".cpp"):
        cmd = [nvcc, "-x", "cu"] + NVFLAGS + extra + ["-c", path, "-o", obj]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{res.stdout}\n{res.stderr}")
    return obj, res.stderr


def build(force: bool = False, verbose: bool = False, extra=None) -> str:
    """Compiles every unit and links the library; returns its path."""
    os.makedirs(OBJ, exist_ok=True)
    extra = list(extra or [])
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(lambda s: _compile(s, force, extra), SOURCES))
    objs = [r[0] for r in results]
    if verbose:
        for _, log in results:
            if log:
                print(log, file=sys.stderr)
    if force or not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [_nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart_static", "-lrt", "-lpthread",
                                                                 "-ldl"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    return LIB


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--verbose", action="store_true")
    ap.add_argument("--ptxas", action="store_true", help="print register/spill usage")
    a = ap.parse_args()
    extra = ["-Xptxas", "-v"] if a.ptxas else []
    print(build(force=a.force or a.ptxas, verbose=a.verbose or a.ptxas, extra=extra))
