"""ctypes binding of libhal_cuda.so (the C ABI in include/hal_cuda.h).

This is the Python host side used by the tests and the benchmark; the C++
host side for HAL-CPP models is hal-cpp_gb300/cpp (Hal::Cuda::*Backend2D).
Errors follow the reference's convention: HAL_CUDA_EINVAL raises ValueError
(std::invalid_argument in C++), every other failure RuntimeError.

There is no CPU fallback: importing works without a GPU, but every call that
needs the CUDA library raises if libhal_cuda.so is missing or no device is
present.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

PKG_DIR = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG_DIR, "libhal_cuda.so")

OK, EINVAL, ENOMEM, EDEVICE, ETIMEOUT, ENOTSUP = 0, 1, 2, 3, 4, 5
ADI_MAX_LINE = 4096
STENCIL_DIFFUSE_VAR, STENCIL_ADVECT, STENCIL_ADVECT_VAR = 0, 1, 2

# Every exported symbol of include/hal_cuda.h, with (restype, argtypes).
_i32, _i64, _f64, _vp = ctypes.c_int32, ctypes.c_int64, ctypes.c_double, ctypes.c_void_p
_I = ctypes.c_int
SIGNATURES = {
    "hal_cuda_version": (ctypes.c_char_p, []),
    "hal_cuda_last_error": (ctypes.c_char_p, []),
    "hal_cuda_device_count": (_I, [_vp]),
    "hal_cuda_set_device": (_I, [_i32]),
    "hal_cuda_launch_count": (_i64, []),
    "hal_cuda_diffusion_create": (_I, [_i32, _i32, _vp]),
    "hal_cuda_diffusion_destroy": (_I, [_vp]),
    "hal_cuda_diffuse": (_I, [_vp, _vp, _i64, _vp, _i64, _f64, _i32, _i32, _i32, _i32]),
    "hal_cuda_diffuse_bc": (_I, [_vp, _vp, _vp, _f64, _i32, _i32, _vp]),
    "hal_cuda_diffuse_var": (_I, [_vp, _vp, _vp, _vp, _vp, _i32, _i32]),
    "hal_cuda_advect": (_I, [_vp, _vp, _vp, _f64, _f64, _i32, _i32]),
    "hal_cuda_advect_var": (_I, [_vp, _vp, _vp, _vp, _vp, _i32, _i32]),
    "hal_cuda_advect_bc": (_I, [_vp, _vp, _vp, _f64, _f64, _i32, _i32, _vp]),
    "hal_cuda_advect_var_bc": (_I, [_vp, _vp, _vp, _vp, _vp, _i32, _i32, _vp, _vp, _vp]),
    "hal_cuda_stencil64_profile": (_I, [_vp, _i32, _i32, _f64, _f64, _i32, _i32, _vp]),
    "hal_cuda_fp64_issue_rate": (_I, [_vp]),
    "hal_cuda_check_plan_division": (_I, [_vp, _i64, _vp, _i32, _vp]),
    "hal_cuda_diffusion_set_field": (_I, [_vp, _vp, _i64]),
    "hal_cuda_diffusion_get_field": (_I, [_vp, _vp, _i64]),
    "hal_cuda_diffusion_set_source": (_I, [_vp, _vp, _i64]),
    "hal_cuda_diffusion_set_point_sources": (_I, [_vp, _i32, _vp, _vp]),
    "hal_cuda_diffusion_set_blocking": (_I, [_vp, _i32]),
    "hal_cuda_diffusion_test_stall": (_I, [_vp, _i32, _f64]),
    "hal_cuda_diffusion_set_velocity": (_I, [_vp, _f64, _f64]),
    "hal_cuda_diffusion_set_dirichlet": (_I, [_vp, _vp]),
    "hal_cuda_diffusion_run_ticks": (_I, [_vp, _i32, _f64, _f64, _i32, _i32]),
    "hal_cuda_diffusion_run_steps": (_I, [_vp, _vp, _i64, _i32, _f64, _i32, _i32]),
    "hal_cuda_diffusion_profile": (_I, [_vp, _i32, _f64, _f64, _i32, _i32, _vp]),
    "hal_cuda_diffusion_sync": (_I, [_vp]),
    "hal_cuda_diffusion_stream": (_vp, [_vp]),
    "hal_cuda_diffusion_set_stream": (_I, [_vp, _vp]),
    "hal_cuda_pdegrid2d_write": (_I, [ctypes.c_char_p, _i32, _i32, _i32, _i32, _i32, _vp, _vp]),
    "hal_cuda_pdegrid2d_read_header": (_I, [ctypes.c_char_p, _vp, _vp, _vp, _vp, _vp]),
    "hal_cuda_pdegrid2d_read": (_I, [ctypes.c_char_p, _i32, _i32, _vp, _vp]),
    "hal_cuda_diffusion_save": (_I, [_vp, ctypes.c_char_p, _i32, _i32, _i32]),
    "hal_cuda_diffusion_load": (_I, [_vp, ctypes.c_char_p, _vp, _vp, _vp]),
    "hal_cuda_adi_save": (_I, [_vp, ctypes.c_char_p, _i32, _i32, _i32]),
    "hal_cuda_adi_load": (_I, [_vp, ctypes.c_char_p, _vp, _vp, _vp]),
    "hal_cuda_adi_create": (_I, [_i32, _i32, _vp]),
    "hal_cuda_adi_destroy": (_I, [_vp]),
    "hal_cuda_diffuse_adi": (_I, [_vp, _vp, _i64, _vp, _i64, _f64, _i32, _i32, _i32, _i32]),
    "hal_cuda_diffuse_adi_bc": (_I, [_vp, _vp, _vp, _f64, _i32, _i32, _vp]),
    "hal_cuda_adi_set_field": (_I, [_vp, _vp, _i64]),
    "hal_cuda_adi_get_field": (_I, [_vp, _vp, _i64]),
    "hal_cuda_adi_set_source": (_I, [_vp, _vp, _i64]),
    "hal_cuda_adi_set_dirichlet": (_I, [_vp, _vp]),
    "hal_cuda_adi_set_uptake": (_I, [_vp, _vp, _f64]),
    "hal_cuda_diffusion_set_uptake": (_I, [_vp, _vp, _f64]),
    "hal_cuda_adi_run_ticks": (_I, [_vp, _i32, _f64, _f64, _i32, _i32]),
    "hal_cuda_adi_run_coupled": (_I, [_vp, _vp, _i32, _f64, _f64, _i32, _i32, _f64, _f64, _f64, _f64]),
    "hal_cuda_adi_run_steps": (_I, [_vp, _vp, _i64, _i32, _f64, _i32, _i32]),
    "hal_cuda_adi_run_ticks_host": (_I, [_vp, _vp, _vp, _i64, _i32, _f64, _f64, _i32, _i32]),
    "hal_cuda_adi_profile_graph": (_I, [_vp, _i32, _f64, _f64, _i32, _i32, _vp]),
    "hal_cuda_adi_profile": (_I, [_vp, _i32, _f64, _f64, _i32, _i32, _vp]),
    "hal_cuda_adi_sync": (_I, [_vp]),
    "hal_cuda_adi_stream": (_vp, [_vp]),
    "hal_cuda_adi_set_exact": (_I, [_vp, _i32]),
    "hal_cuda_adi_set_stream": (_I, [_vp, _vp]),
    "hal_cuda_agents_create": (_I, [_i32, _i32, _i32, _vp]),
    "hal_cuda_agents_destroy": (_I, [_vp]),
    "hal_cuda_accumulate_forces": (_I, [_vp, _vp, _i64, _vp, _i64, _vp, _f64, _f64, _i32, _i32, _i32,
                                        _i32]),
    "hal_cuda_sum_forces": (_I, [_vp, _vp, _vp, _i64, _vp, _vp, _vp, _f64, _vp, _i32, _i32, _i32, _i32, _i32]),
    "hal_cuda_agents_dispatch_law": (_I, [_vp, _f64, _vp, _i32, _i32, _i32]),
    "hal_cuda_agents_step_law": (_I, [_vp, _i32, _f64, _vp, _i32, _i32, _i32, _f64, _f64]),
    "hal_cuda_agents_get_force_sums": (_I, [_vp, _vp, _i32]),
    "hal_cuda_agents_upload": (_I, [_vp, _vp, _vp, _i32]),
    "hal_cuda_pdegrid_create": (_I, [_i32, _i32, _i32, _i32, _vp]),
    "hal_cuda_pdegrid_destroy": (_I, [_vp]),
    "hal_cuda_pdegrid_set_state": (_I, [_vp, _vp, _vp, _i32]),
    "hal_cuda_pdegrid_get_state": (_I, [_vp, _vp, _vp, _vp]),
    "hal_cuda_pdegrid_dims": (_I, [_vp, _vp]),
    "hal_cuda_pdegrid_apply": (_I, [_vp, _vp, _i32, _vp, _vp, _f64, _i64]),
    "hal_cuda_pdegrid_apply_agents": (_I, [_vp, _vp, _i32, _f64, _vp]),
    "hal_cuda_pdegrid_apply_all": (_I, [_vp, _i32, _f64, _vp]),
    "hal_cuda_pdegrid_update": (_I, [_vp]),
    "hal_cuda_pdegrid_set_non_negative": (_I, [_vp]),
    "hal_cuda_pdegrid_get_cells": (_I, [_vp, _vp, _i64, _vp]),
    "hal_cuda_pdegrid_gradient": (_I, [_vp, _vp, _vp, _i64, _i32, _f64, _vp, _vp]),
    "hal_cuda_pdegrid_stats": (_I, [_vp, _f64, _vp]),
    "hal_cuda_pdegrid_diffusion": (_I, [_vp, _f64, _vp]),
    "hal_cuda_pdegrid_diffusion_var": (_I, [_vp, _vp, _vp]),
    "hal_cuda_pdegrid_diffusion_adi": (_I, [_vp, _f64, _vp]),
    "hal_cuda_pdegrid_advection": (_I, [_vp, _f64, _f64, _vp]),
    "hal_cuda_pdegrid_advection_var": (_I, [_vp, _vp, _vp, _vp, _vp, _vp]),
    "hal_cuda_pdegrid_sync": (_I, [_vp]),
    "hal_cuda_pdegrid_stream": (_vp, [_vp]),
    "hal_cuda_pdegrid_set_stream": (_I, [_vp, _vp]),
    "hal_cuda_agents_dispatch": (_I, [_vp, _f64, _f64, _i32, _i32]),
    "hal_cuda_agents_download": (_I, [_vp, _vp, _i32]),
    "hal_cuda_agents_set_velocities": (_I, [_vp, _vp, _i32]),
    "hal_cuda_agents_get_state": (_I, [_vp, _vp, _vp, _i32]),
    "hal_cuda_agents_step": (_I, [_vp, _i32, _f64, _f64, _i32, _i32, _f64, _f64]),
    "hal_cuda_agents_get_bins": (_I, [_vp, _vp, _vp]),
    "hal_cuda_agents_profile": (_I, [_vp, _i32, _f64, _f64, _i32, _i32, _vp]),
    "hal_cuda_agents_sync": (_I, [_vp]),
    "hal_cuda_agents_stream": (_vp, [_vp]),
    "hal_cuda_agents_set_stream": (_I, [_vp, _vp]),
    "hal_cuda_wells_create": (_I, [_vp, _i32, _vp]),
    "hal_cuda_wells_destroy": (_I, [_vp]),
    "hal_cuda_wells_set_field": (_I, [_vp, _i32, _vp, _i64]),
    "hal_cuda_wells_get_field": (_I, [_vp, _i32, _vp, _i64]),
    "hal_cuda_wells_set_source": (_I, [_vp, _i32, _vp, _i64]),
    "hal_cuda_wells_set_agents": (_I, [_vp, _vp, _vp, _vp]),
    "hal_cuda_wells_run_ticks": (_I, [_vp, _i32, _f64, _f64]),
    "hal_cuda_wells_get_forces": (_I, [_vp, _vp, _i64]),
    "hal_cuda_wells_profile": (_I, [_vp, _i32, _f64, _f64, _vp]),
    "hal_cuda_wells_set_motion": (_I, [_vp, _i32, _f64, _f64]),
    "hal_cuda_wells_set_velocities": (_I, [_vp, _vp, _i64]),
    "hal_cuda_wells_get_agents": (_I, [_vp, _vp, _vp, _i64]),
    "hal_cuda_wells_autotune": (_I, [_vp, _vp, _vp, _vp]),
    "hal_cuda_wells_sync": (_I, [_vp]),
    "hal_cuda_wells_stream": (_vp, [_vp]),
    "hal_cuda_wells_set_stream": (_I, [_vp, _vp]),
    "hal_cuda_adjoint_create": (_I, [_i32, _i32, _i32, _i32, _vp]),
    "hal_cuda_adjoint_destroy": (_I, [_vp]),
    "hal_cuda_adjoint_set_problem": (_I, [_vp, _vp, _vp, _i64, _i32, _i32]),
    "hal_cuda_adjoint_forward": (_I, [_vp, _vp, _f64, _vp, _vp, _vp]),
    "hal_cuda_adjoint_gradient": (_I, [_vp, _vp, _f64, _vp, _vp, _vp, _vp, _vp]),
    "hal_cuda_adjoint_times": (_I, [_vp, _vp, _vp]),
    "hal_cuda_agents_forces_noalloc": (_I, [_vp, _vp, _i32, _vp, _f64, _f64, _i32, _i32, _i32, _i32,
                                            _vp]),
}

_lib = None


def lib():
    """The loaded library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with hal-cpp_gb300/build.py")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def last_error() -> str:
    return lib().hal_cuda_last_error().decode()


def _check(rc: int, what: str = ""):
    if rc == OK:
        return
    msg = last_error()
    if rc == EINVAL:
        raise ValueError(msg or what)
    raise RuntimeError(f"{what}: status {rc}: {msg}")


def version() -> str:
    return lib().hal_cuda_version().decode()


def device_count() -> int:
    n = ctypes.c_int32(0)
    rc = lib().hal_cuda_device_count(ctypes.byref(n))
    return n.value if rc == OK else 0


def launch_count() -> int:
    return int(lib().hal_cuda_launch_count())


def _path(path) -> bytes:
    return os.fsencode(path)


def pdegrid2d_write(path, xDim, yDim, wrapX, wrapY, updateCt, field, deltas=None):
    """Writes a grid state in PDEGrid2D's on-disk format (SavePDEGrid2D)."""
    f = _f64(field)
    d = None if deltas is None else _f64(deltas)
    n = xDim * yDim
    if f.size != n or (d is not None and d.size != n):
        raise ValueError(f"field/deltas must hold {n} values")
    _check(lib().hal_cuda_pdegrid2d_write(_path(path), xDim, yDim, int(wrapX), int(wrapY), updateCt, _p(f),
                                          _p(d)), "pdegrid2d_write")


def pdegrid2d_read(path):
    """Reads a PDEGrid2D file: dict of xDim, yDim, wrapX, wrapY, updateCt,
    field, deltas (LoadPDEGrid2D)."""
    v = [ctypes.c_int32() for _ in range(5)]
    _check(lib().hal_cuda_pdegrid2d_read_header(_path(path), *[ctypes.byref(x) for x in v]), "pdegrid2d_read")
    xd, yd, wx, wy, u = (x.value for x in v)
    f = np.empty(xd * yd, dtype=np.float64)
    d = np.empty(xd * yd, dtype=np.float64)
    _check(lib().hal_cuda_pdegrid2d_read(_path(path), xd, yd, _p(f), _p(d)), "pdegrid2d_read")
    return {"xDim": xd, "yDim": yd, "wrapX": bool(wx), "wrapY": bool(wy), "updateCt": u, "field": f, "deltas": d}


def _load_resident(fn, h, path):
    v = [ctypes.c_int32() for _ in range(3)]
    _check(fn(h, _path(path), *[ctypes.byref(x) for x in v]), "load")
    return bool(v[0].value), bool(v[1].value), v[2].value


def fp64_issue_rate() -> float:
    """Measured FP64 add issue rate of the current device (ops/s)."""
    v = ctypes.c_double()
    _check(lib().hal_cuda_fp64_issue_rate(ctypes.byref(v)), "fp64_issue_rate")
    return v.value


def check_plan_division(num, den) -> int:
    """Pairs (num[i], den[j]) whose quotient by the FP64 ADI's division (a
    double-word reciprocal and one Markstein correction) differs in any bit
    from IEEE division on the device; every |den| must lie in [2^-20, 2^20]."""
    n = np.ascontiguousarray(num, np.float64)
    d = np.ascontiguousarray(den, np.float64)
    v = ctypes.c_int64()
    _check(lib().hal_cuda_check_plan_division(n.ctypes.data, n.size, d.ctypes.data, d.size, ctypes.byref(v)),
           "check_plan_division")
    return v.value


def _p(a):
    return None if a is None else a.ctypes.data


def _f32(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float32)


def _f64(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.int32)


class _Handle:
    _prefix = ""

    def __init__(self):
        self._h = None

    def close(self):
        if self._h is not None:
            getattr(lib(), f"hal_cuda_{self._prefix}_destroy")(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def handle(self):
        return self._h

    def sync(self):
        _check(getattr(lib(), f"hal_cuda_{self._prefix}_sync")(self._h), "sync")

    def stream(self) -> int:
        return getattr(lib(), f"hal_cuda_{self._prefix}_stream")(self._h) or 0

    def set_stream(self, stream_ptr: int | None):
        _check(getattr(lib(), f"hal_cuda_{self._prefix}_set_stream")(self._h, stream_ptr or None),
               "set_stream")


class Diffusion(_Handle):
    """hal_cuda_diffusion: IDiffusionBackend2D plus the resident fused tick."""

    _prefix = "diffusion"

    def __init__(self, xDim: int, yDim: int):
        super().__init__()
        h = ctypes.c_void_p()
        _check(lib().hal_cuda_diffusion_create(xDim, yDim, ctypes.byref(h)), "diffusion_create")
        self._h = h
        self.xDim, self.yDim = xDim, yDim

    def diffuse(self, field, deltas, diffRate, xDim, yDim, wrapX, wrapY):
        """IDiffusionBackend2D::Diffuse on float64 host arrays; deltas is
        updated in place and returned."""
        f = _f64(field)
        d = np.ascontiguousarray(deltas, dtype=np.float64)
        _check(lib().hal_cuda_diffuse(self._h, _p(f), f.size, _p(d), d.size, diffRate, xDim, yDim,
                                      int(wrapX), int(wrapY)), "diffuse")
        return d

    def diffuse_bc(self, field, deltas, diffRate, wrapX, wrapY, ghost):
        f = _f64(field)
        d = np.ascontiguousarray(deltas, dtype=np.float64)
        g = _f64(ghost)
        _check(lib().hal_cuda_diffuse_bc(self._h, _p(f), _p(d), diffRate, int(wrapX), int(wrapY),
                                         _p(g)), "diffuse_bc")
        return d

    def _cells(self, *arrays):
        n = self.xDim * self.yDim
        for a in arrays:
            if a.size != n:
                raise ValueError(f"array of {a.size} values for a {self.xDim} x {self.yDim} grid")

    def diffuse_var(self, field, deltas, ratesX, ratesY, wrapX, wrapY):
        """Internal::Diffusion2 with per-cell rates on float64 host arrays;
        deltas is updated in place and returned."""
        f, rx, ry = _f64(field), _f64(ratesX), _f64(ratesY)
        d = np.ascontiguousarray(deltas, dtype=np.float64)
        self._cells(f, d, rx, ry)
        _check(lib().hal_cuda_diffuse_var(self._h, _p(f), _p(d), _p(rx), _p(ry), int(wrapX), int(wrapY)),
               "diffuse_var")
        return d

    def _ghost(self, g):
        if g is None:
            return None
        g = _f64(g)
        if g.size != 2 * (self.xDim + self.yDim):
            raise ValueError(f"ghost table of {g.size} values, expected {2 * (self.xDim + self.yDim)}")
        return g

    def advect(self, field, deltas, xVel, yVel, wrapX, wrapY, ghost=None):
        """Internal::Advection2 at a uniform velocity (upwind); with a ghost
        table, its Dirichlet form."""
        f = _f64(field)
        d = np.ascontiguousarray(deltas, dtype=np.float64)
        self._cells(f, d)
        g = self._ghost(ghost)
        if g is None:
            rc = lib().hal_cuda_advect(self._h, _p(f), _p(d), float(xVel), float(yVel), int(wrapX), int(wrapY))
        else:
            rc = lib().hal_cuda_advect_bc(self._h, _p(f), _p(d), float(xVel), float(yVel), int(wrapX), int(wrapY),
                                          _p(g))
        _check(rc, "advect")
        return d

    def advect_var(self, field, deltas, xVels, yVels, wrapX, wrapY, ghost=None, ghost_vx=None, ghost_vy=None):
        """Internal::Advection2 with per-cell velocities (upwind face fluxes);
        with ghost tables (field, x velocity, y velocity), its Dirichlet form."""
        f, vx, vy = _f64(field), _f64(xVels), _f64(yVels)
        d = np.ascontiguousarray(deltas, dtype=np.float64)
        self._cells(f, d, vx, vy)
        gs = [self._ghost(g) for g in (ghost, ghost_vx, ghost_vy)]
        if all(g is None for g in gs):
            rc = lib().hal_cuda_advect_var(self._h, _p(f), _p(d), _p(vx), _p(vy), int(wrapX), int(wrapY))
        else:
            rc = lib().hal_cuda_advect_var_bc(self._h, _p(f), _p(d), _p(vx), _p(vy), int(wrapX), int(wrapY),
                                              *[None if g is None else _p(g) for g in gs])
        _check(rc, "advect_var")
        return d

    def save(self, path, wrapX=False, wrapY=False, updateCt=0):
        """The resident field in PDEGrid2D's on-disk format."""
        _check(lib().hal_cuda_diffusion_save(self._h, _path(path), int(wrapX), int(wrapY), updateCt), "save")

    def load(self, path):
        """Loads a PDEGrid2D file into the resident field; returns (wrapX,
        wrapY, updateCt)."""
        return _load_resident(lib().hal_cuda_diffusion_load, self._h, path)

    def stencil64_profile(self, kind, iters, xVel=0.0, yVel=0.0, wrapX=False, wrapY=False):
        """Average device ms of one FP64 stencil launch of `kind` (STENCIL_*)
        on the arrays the last call of that kind uploaded."""
        ms = ctypes.c_float()
        _check(lib().hal_cuda_stencil64_profile(self._h, kind, iters, float(xVel), float(yVel), int(wrapX),
                                                int(wrapY), ctypes.byref(ms)), "stencil64_profile")
        return ms.value

    def set_field(self, field):
        f = _f32(field)
        _check(lib().hal_cuda_diffusion_set_field(self._h, _p(f), f.size), "set_field")

    def get_field(self):
        out = np.empty(self.xDim * self.yDim, dtype=np.float32)
        _check(lib().hal_cuda_diffusion_get_field(self._h, _p(out), out.size), "get_field")
        return out

    def set_source(self, dense):
        d = _f32(dense)
        _check(lib().hal_cuda_diffusion_set_source(self._h, _p(d), 0 if d is None else d.size),
               "set_source")

    def set_point_sources(self, cells, values):
        c = _i32(cells)
        v = _f32(values)
        n = 0 if c is None else c.size
        _check(lib().hal_cuda_diffusion_set_point_sources(self._h, n, _p(c), _p(v)),
               "set_point_sources")

    def set_dirichlet(self, ghost):
        g = _f32(ghost)
        _check(lib().hal_cuda_diffusion_set_dirichlet(self._h, _p(g)), "set_dirichlet")

    def set_blocking(self, ticksPerLaunch):
        """Ticks per launch: 1, 2 (temporal blocking) or 0 (by grid size)."""
        _check(lib().hal_cuda_diffusion_set_blocking(self._h, int(ticksPerLaunch)), "set_blocking")

    def test_stall(self, stall, waitSeconds=0.0):
        """Failure-detection test hook: the two-tick kernel's staging waits run
        out (see include/hal_cuda_measure.h)."""
        _check(lib().hal_cuda_diffusion_test_stall(self._h, int(stall), float(waitSeconds)), "test_stall")

    def set_velocity(self, xVel, yVel):
        """Uniform upwind advection of every following tick (PDEGrid2D::Advection)."""
        _check(lib().hal_cuda_diffusion_set_velocity(self._h, float(xVel), float(yVel)), "set_velocity")

    def set_uptake(self, agents, uptake):
        """Each agent of ``agents`` (its last binning) multiplies its cell by
        -uptake every following tick; ``agents`` None removes the coupling."""
        _check(lib().hal_cuda_diffusion_set_uptake(self._h, None if agents is None else agents.handle,
                                                   uptake), "set_uptake")

    def run_ticks(self, ticks, diffRate, decay=0.0, wrapX=False, wrapY=False):
        _check(lib().hal_cuda_diffusion_run_ticks(self._h, ticks, diffRate, decay, int(wrapX),
                                                  int(wrapY)), "run_ticks")

    def profile(self, iters, diffRate, decay=0.0, wrapX=False, wrapY=False):
        """Average ms of one fused-tick launch."""
        ms = np.zeros(1, dtype=np.float32)
        _check(lib().hal_cuda_diffusion_profile(self._h, iters, diffRate, decay, int(wrapX),
                                                int(wrapY), _p(ms)), "profile")
        return float(ms[0])

    def run_steps(self, field, steps, diffRate, wrapX=False, wrapY=False):
        f = np.array(field, dtype=np.float32, copy=True)
        _check(lib().hal_cuda_diffusion_run_steps(self._h, _p(f), f.size, steps, diffRate,
                                                  int(wrapX), int(wrapY)), "run_steps")
        return f


class Adi(_Handle):
    """hal_cuda_adi: IAdiDiffusionBackend2D plus the resident ADI tick."""

    _prefix = "adi"

    def __init__(self, xDim: int, yDim: int):
        super().__init__()
        h = ctypes.c_void_p()
        _check(lib().hal_cuda_adi_create(xDim, yDim, ctypes.byref(h)), "adi_create")
        self._h = h
        self.xDim, self.yDim = xDim, yDim

    def diffuse_adi(self, field, deltas, diffRate, xDim, yDim, wrapX, wrapY):
        f = _f64(field)
        d = np.ascontiguousarray(deltas, dtype=np.float64)
        _check(lib().hal_cuda_diffuse_adi(self._h, _p(f), f.size, _p(d), d.size, diffRate, xDim,
                                          yDim, int(wrapX), int(wrapY)), "diffuse_adi")
        return d

    def set_exact(self, exact=True):
        """Interface calls (diffuse_adi, diffuse_adi_bc) in FP64 at every
        size, bit-exact to the CPU backend (default: FP32 up to
        HAL_CUDA_ADI_MAX_LINE)."""
        _check(lib().hal_cuda_adi_set_exact(self._h, int(bool(exact))), "adi_set_exact")

    def diffuse_adi_bc(self, field, deltas, diffRate, wrapX, wrapY, ghost):
        f = _f64(field)
        d = np.ascontiguousarray(deltas, dtype=np.float64)
        g = _f64(ghost)
        _check(lib().hal_cuda_diffuse_adi_bc(self._h, _p(f), _p(d), diffRate, int(wrapX),
                                             int(wrapY), _p(g)), "diffuse_adi_bc")
        return d

    def set_field(self, field):
        f = _f32(field)
        _check(lib().hal_cuda_adi_set_field(self._h, _p(f), f.size), "set_field")

    def get_field(self, out=None):
        """The resident field in HAL's layout, into `out` (a float32 array of
        xDim*yDim values, e.g. pinned pages) when given."""
        if out is None:
            out = np.empty(self.xDim * self.yDim, dtype=np.float32)
        elif out.dtype != np.float32 or out.size != self.xDim * self.yDim or not out.flags.c_contiguous:
            raise ValueError("out must be a contiguous float32 array of xDim*yDim values")
        _check(lib().hal_cuda_adi_get_field(self._h, _p(out), out.size), "get_field")
        return out

    def save(self, path, wrapX=False, wrapY=False, updateCt=0):
        """The resident field in PDEGrid2D's on-disk format."""
        _check(lib().hal_cuda_adi_save(self._h, _path(path), int(wrapX), int(wrapY), updateCt), "save")

    def load(self, path):
        """Loads a PDEGrid2D file into the resident field; returns (wrapX,
        wrapY, updateCt)."""
        return _load_resident(lib().hal_cuda_adi_load, self._h, path)

    def set_source(self, dense):
        d = _f32(dense)
        _check(lib().hal_cuda_adi_set_source(self._h, _p(d), 0 if d is None else d.size),
               "set_source")

    def set_dirichlet(self, ghost):
        g = _f32(ghost)
        _check(lib().hal_cuda_adi_set_dirichlet(self._h, _p(g)), "set_dirichlet")

    def set_uptake(self, agents, uptake):
        _check(lib().hal_cuda_adi_set_uptake(self._h, None if agents is None else agents.handle,
                                             uptake), "set_uptake")

    def run_ticks(self, ticks, diffRate, decay=0.0, wrapX=False, wrapY=False):
        _check(lib().hal_cuda_adi_run_ticks(self._h, ticks, diffRate, decay, int(wrapX),
                                            int(wrapY)), "run_ticks")

    def run_coupled(self, agents, ticks, diffRate, decay=0.0, wrapX=False, wrapY=False, interactionRad=1.0,
                    springConstant=0.1, friction=1.0, maxVel=-1.0):
        """`ticks` ticks of agents.step(1, ...) then run_ticks(1, ...), as one
        graph on this handle's stream (agents coupled by set_uptake)."""
        _check(lib().hal_cuda_adi_run_coupled(self._h, agents.handle, ticks, diffRate, decay, int(wrapX), int(wrapY),
                                              interactionRad, springConstant, friction, maxVel), "run_coupled")

    def run_steps(self, field, steps, diffRate, wrapX=False, wrapY=False):
        f = np.array(field, dtype=np.float32, copy=True)
        _check(lib().hal_cuda_adi_run_steps(self._h, _p(f), f.size, steps, diffRate, int(wrapX),
                                            int(wrapY)), "run_steps")
        return f

    def profile_graph(self, iters, diffRate, decay=0.0, wrapX=False, wrapY=False):
        """Mean ms of one x- and one y-sweep launch among `iters` back-to-back
        launches replayed from a graph (the field does not change)."""
        ms = np.zeros(2, dtype=np.float32)
        _check(lib().hal_cuda_adi_profile_graph(self._h, iters, diffRate, decay, int(wrapX), int(wrapY), _p(ms)),
               "profile_graph")
        return float(ms[0]), float(ms[1])

    def profile(self, iters, diffRate, decay=0.0, wrapX=False, wrapY=False):
        """Average ms of one launch of (x-sweep, y-sweep)."""
        ms = np.zeros(2, dtype=np.float32)
        _check(lib().hal_cuda_adi_profile(self._h, iters, diffRate, decay, int(wrapX), int(wrapY),
                                          _p(ms)), "profile")
        return float(ms[0]), float(ms[1])

    def run_ticks_host(self, field, src, ticks, diffRate, decay=0.0, wrapX=False, wrapY=False,
                       out=None):
        """Host-to-host ticks: field (and src) uploaded, ticks run, field
        downloaded.  ``field`` must be a float32 array; it is updated in place
        when ``out`` is None."""
        f = field if out is None else out
        if f is not field:
            np.copyto(f, field)
        s = None if src is None else src
        _check(lib().hal_cuda_adi_run_ticks_host(self._h, f.ctypes.data,
                                                 None if s is None else s.ctypes.data, f.size,
                                                 ticks, diffRate, decay, int(wrapX), int(wrapY)),
               "run_ticks_host")
        return f


FORCE_LINEAR, FORCE_LINEAR_CLAMPED, FORCE_POWER = 0, 1, 2
ORDER_BACKEND, ORDER_AGENTGRID = 0, 1


class ForceLaw(ctypes.Structure):
    """hal_cuda_force_law: the overlap force law of SphericalAgent2D::SumForces."""

    _fields_ = [("kind", ctypes.c_int32), ("scale", ctypes.c_double), ("exponent", ctypes.c_double)]


def _law(kind, scale, exponent=1.0):
    return ForceLaw(int(kind), float(scale), float(exponent))


class Agents(_Handle):
    """hal_cuda_agents: IAgentForceBackend2D plus the resident dispatch."""

    _prefix = "agents"

    def __init__(self, xDim: int, yDim: int, maxAgents: int):
        super().__init__()
        h = ctypes.c_void_p()
        _check(lib().hal_cuda_agents_create(xDim, yDim, maxAgents, ctypes.byref(h)),
               "agents_create")
        self._h = h
        self.xDim, self.yDim, self.maxAgents = xDim, yDim, maxAgents
        self.n = 0

    def accumulate_forces(self, positions, radii, interactionRad, springConstant, xDim, yDim,
                          wrapX, wrapY):
        """IAgentForceBackend2D::AccumulateForces; returns velocityDeltas
        (float64, 2n)."""
        p = _f64(positions)
        r = _f64(radii)
        out = np.zeros(p.size, dtype=np.float64)
        _check(lib().hal_cuda_accumulate_forces(self._h, _p(p), p.size, _p(r), r.size, _p(out),
                                                interactionRad, springConstant, xDim, yDim,
                                                int(wrapX), int(wrapY)), "accumulate_forces")
        self.n = r.size
        return out

    def sum_forces(self, positions, radii, interactionRad, law, scale, xDim, yDim, wrapX, wrapY,
                   velocities=None, exponent=1.0, order=ORDER_AGENTGRID, sums=True):
        """SphericalAgent2D::SumForces of every agent (FP64); returns
        (velocities after the call [2n], sums of positive forces [n] or None)."""
        p = _f64(positions)
        r = _f64(radii)
        v = None if velocities is None else _f64(velocities)
        out = np.zeros(p.size, dtype=np.float64)
        fs = np.zeros(max(r.size, 1), dtype=np.float64) if sums else None
        lw = _law(law, scale, exponent)
        _check(lib().hal_cuda_sum_forces(self._h, _p(p), _p(r), r.size, _p(v), _p(out), _p(fs), interactionRad,
                                         ctypes.byref(lw), int(order), xDim, yDim, int(wrapX), int(wrapY)),
               "sum_forces")
        self.n = r.size
        return out, (fs[: r.size] if sums else None)

    def dispatch_law(self, interactionRad, law, scale, exponent=1.0, sums=True, wrapX=False, wrapY=False):
        lw = _law(law, scale, exponent)
        _check(lib().hal_cuda_agents_dispatch_law(self._h, interactionRad, ctypes.byref(lw), int(sums), int(wrapX),
                                                  int(wrapY)), "dispatch_law")

    def step_law(self, ticks, interactionRad, law, scale, exponent=1.0, sums=True, wrapX=False, wrapY=False,
                 friction=1.0, maxVel=-1.0):
        lw = _law(law, scale, exponent)
        _check(lib().hal_cuda_agents_step_law(self._h, ticks, interactionRad, ctypes.byref(lw), int(sums),
                                              int(wrapX), int(wrapY), float(friction), float(maxVel)), "step_law")

    def get_force_sums(self):
        out = np.empty(max(self.n, 1), dtype=np.float32)
        _check(lib().hal_cuda_agents_get_force_sums(self._h, _p(out), self.n), "get_force_sums")
        return out[: self.n]

    def upload(self, positions, radii):
        p = _f32(positions)
        r = _f32(radii)
        _check(lib().hal_cuda_agents_upload(self._h, _p(p), _p(r), r.size), "upload")
        self.n = r.size

    def dispatch(self, interactionRad, springConstant, wrapX=False, wrapY=False):
        _check(lib().hal_cuda_agents_dispatch(self._h, interactionRad, springConstant,
                                              int(wrapX), int(wrapY)), "dispatch")

    def download(self):
        out = np.empty(2 * self.n, dtype=np.float32)
        _check(lib().hal_cuda_agents_download(self._h, _p(out), self.n), "download")
        return out

    def set_velocities(self, velocities=None):
        """Each agent's (xVel, yVel), interleaved; None sets them to zero."""
        v = None if velocities is None else _f32(velocities)
        if v is not None and v.size != 2 * self.n:
            raise ValueError(f"{v.size} velocity values for {self.n} agents")
        _check(lib().hal_cuda_agents_set_velocities(self._h, _p(v), self.n), "set_velocities")

    def get_state(self):
        """(positions, velocities) of the resident agents, float32 interleaved."""
        p = np.empty(2 * self.n, dtype=np.float32)
        v = np.empty(2 * self.n, dtype=np.float32)
        _check(lib().hal_cuda_agents_get_state(self._h, _p(p), _p(v), self.n), "get_state")
        return p, v

    def step(self, ticks, interactionRad, springConstant, wrapX=False, wrapY=False, friction=1.0, maxVel=-1.0):
        """`ticks` resident ticks: forces, then vel += delta, CapVelocity
        (maxVel >= 0), ForceMove, ApplyFriction.  Asynchronous."""
        _check(lib().hal_cuda_agents_step(self._h, ticks, interactionRad, springConstant, int(wrapX), int(wrapY),
                                          float(friction), float(maxVel)), "step")

    def profile(self, iters, interactionRad, springConstant, wrapX=False, wrapY=False):
        """Average ms per launch: count, scan, scatter, stabilize, forces, whole."""
        ms = np.zeros(6, dtype=np.float32)
        _check(lib().hal_cuda_agents_profile(self._h, iters, interactionRad, springConstant,
                                             int(wrapX), int(wrapY), _p(ms)), "profile")
        return [float(v) for v in ms]

    def get_bins(self):
        off = np.empty(self.xDim * self.yDim + 1, dtype=np.int32)
        bucket = np.empty(max(self.n, 1), dtype=np.int32)
        _check(lib().hal_cuda_agents_get_bins(self._h, _p(off), _p(bucket)), "get_bins")
        return off, bucket[: self.n]


CELL_SET, CELL_ADD, CELL_MUL, CELL_SCALE = 0, 1, 2, 3


class PDEGrid(_Handle):
    """hal_cuda_pdegrid: Hal::PDEGrid2D resident on the device (FP64), the
    per-cell operations batched into lists."""

    _prefix = "pdegrid"

    def __init__(self, xDim: int, yDim: int, wrapX=False, wrapY=False):
        super().__init__()
        h = ctypes.c_void_p()
        _check(lib().hal_cuda_pdegrid_create(xDim, yDim, int(wrapX), int(wrapY), ctypes.byref(h)),
               "pdegrid_create")
        self._h = h
        self.xDim, self.yDim, self.wrapX, self.wrapY = xDim, yDim, bool(wrapX), bool(wrapY)

    @property
    def length(self):
        return self.xDim * self.yDim

    def set_state(self, field, deltas=None, update_ct=0):
        f = _f64(field)
        d = _f64(deltas)
        _check(lib().hal_cuda_pdegrid_set_state(self._h, _p(f), _p(d), int(update_ct)), "pdegrid_set_state")

    def get_state(self):
        """(field, deltas, updateCt)."""
        f = np.empty(self.length)
        d = np.empty(self.length)
        uc = ctypes.c_int32(0)
        _check(lib().hal_cuda_pdegrid_get_state(self._h, _p(f), _p(d), ctypes.byref(uc)), "pdegrid_get_state")
        return f, d, uc.value

    def apply(self, cells, values, op=None, ops=None):
        """Operations at cells in list order: one `op` for all, or ops[k]."""
        c = _i32(cells)
        v = _f64(values)
        o = _i32(ops)
        n = 0 if c is None else c.size
        _check(lib().hal_cuda_pdegrid_apply(self._h, _p(o), -1 if op is None else int(op), _p(c), _p(v), 0.0, n),
               "pdegrid_apply")

    def apply_agents(self, agents, op, value=0.0, per_agent=None):
        pa = _f64(per_agent)
        _check(lib().hal_cuda_pdegrid_apply_agents(self._h, agents.handle, int(op), float(value), _p(pa)),
               "pdegrid_apply_agents")

    def apply_all(self, op, value=0.0, per_cell=None):
        pc = _f64(per_cell)
        _check(lib().hal_cuda_pdegrid_apply_all(self._h, int(op), float(value), _p(pc)), "pdegrid_apply_all")

    def update(self):
        _check(lib().hal_cuda_pdegrid_update(self._h), "pdegrid_update")

    def set_non_negative(self):
        _check(lib().hal_cuda_pdegrid_set_non_negative(self._h), "pdegrid_set_non_negative")

    def get_cells(self, cells):
        c = _i32(cells)
        out = np.empty(c.size)
        _check(lib().hal_cuda_pdegrid_get_cells(self._h, _p(c), c.size, _p(out)), "pdegrid_get_cells")
        return out

    def gradient(self, xs, ys, boundary=None):
        x, y = _i32(xs), _i32(ys)
        gx, gy = np.empty(x.size), np.empty(x.size)
        _check(lib().hal_cuda_pdegrid_gradient(self._h, _p(x), _p(y), x.size, int(boundary is not None),
                                               0.0 if boundary is None else float(boundary), _p(gx), _p(gy)),
               "pdegrid_gradient")
        return gx, gy

    def stats(self, denom_offset=float("nan")):
        """[GetMax, GetMin, GetAvg, MaxDelta, MaxDeltaScaled(denom_offset)]."""
        out = np.empty(5)
        _check(lib().hal_cuda_pdegrid_stats(self._h, float(denom_offset), _p(out)), "pdegrid_stats")
        return out

    def diffusion(self, diff_coef, ghost=None):
        g = _f64(ghost)
        _check(lib().hal_cuda_pdegrid_diffusion(self._h, float(diff_coef), _p(g)), "pdegrid_diffusion")

    def diffusion_var(self, rates_x, rates_y):
        a, b = _f64(rates_x), _f64(rates_y)
        _check(lib().hal_cuda_pdegrid_diffusion_var(self._h, _p(a), _p(b)), "pdegrid_diffusion_var")

    def diffusion_adi(self, diff_rate, ghost=None):
        g = _f64(ghost)
        _check(lib().hal_cuda_pdegrid_diffusion_adi(self._h, float(diff_rate), _p(g)), "pdegrid_diffusion_adi")

    def advection(self, x_vel, y_vel, ghost=None):
        g = _f64(ghost)
        _check(lib().hal_cuda_pdegrid_advection(self._h, float(x_vel), float(y_vel), _p(g)), "pdegrid_advection")

    def advection_var(self, x_vels, y_vels, ghost=None, ghost_x_vel=None, ghost_y_vel=None):
        a, b = _f64(x_vels), _f64(y_vels)
        g, gx, gy = _f64(ghost), _f64(ghost_x_vel), _f64(ghost_y_vel)
        _check(lib().hal_cuda_pdegrid_advection_var(self._h, _p(a), _p(b), _p(g), _p(gx), _p(gy)),
               "pdegrid_advection_var")


WELL_EXPLICIT, WELL_ADI = 0, 1
WELLS_MAX_SIDE = 4096


class WellDesc(ctypes.Structure):
    """hal_cuda_well_desc."""

    _fields_ = [("xDim", ctypes.c_int32), ("yDim", ctypes.c_int32), ("kind", ctypes.c_int32),
                ("wrapX", ctypes.c_int32), ("wrapY", ctypes.c_int32), ("maxAgents", ctypes.c_int32),
                ("diffRate", ctypes.c_double), ("decay", ctypes.c_double)]


class Wells(_Handle):
    """hal_cuda_wells: many independent wells (MultiWellExperiment::Step) per
    launch.  `wells` is a sequence of dicts with keys xDim, yDim, kind
    ("explicit" or "adi"), diffRate, decay and optionally wrapX, wrapY,
    maxAgents."""

    _prefix = "wells"

    def __init__(self, wells):
        super().__init__()
        arr = (WellDesc * len(wells))()
        for i, w in enumerate(wells):
            kind = w["kind"]
            arr[i] = WellDesc(int(w["xDim"]), int(w["yDim"]),
                              WELL_ADI if kind in ("adi", WELL_ADI) else WELL_EXPLICIT,
                              int(bool(w.get("wrapX", False))), int(bool(w.get("wrapY", False))),
                              int(w.get("maxAgents", 0)), float(w["diffRate"]), float(w.get("decay", 0.0)))
        h = ctypes.c_void_p()
        _check(lib().hal_cuda_wells_create(ctypes.cast(arr, ctypes.c_void_p), len(wells), ctypes.byref(h)),
               "wells_create")
        self._h = h
        self.wells = [dict(w) for w in wells]
        self.counts = np.zeros(len(wells), dtype=np.int32)

    def _cells(self, well):
        w = self.wells[well]
        return int(w["xDim"]) * int(w["yDim"])

    def set_field(self, well, field):
        f = _f32(field)
        _check(lib().hal_cuda_wells_set_field(self._h, well, _p(f), f.size), "wells_set_field")

    def get_field(self, well):
        out = np.empty(self._cells(well), dtype=np.float32)
        _check(lib().hal_cuda_wells_get_field(self._h, well, _p(out), out.size), "wells_get_field")
        return out

    def set_source(self, well, dense):
        if dense is None:
            _check(lib().hal_cuda_wells_set_source(self._h, well, None, 0), "wells_set_source")
            return
        d = _f32(dense)
        _check(lib().hal_cuda_wells_set_source(self._h, well, _p(d), d.size), "wells_set_source")

    def set_agents(self, counts, positions, radii):
        c = np.ascontiguousarray(counts, dtype=np.int32)
        p = _f32(positions)
        r = _f32(radii)
        _check(lib().hal_cuda_wells_set_agents(self._h, _p(c), _p(p) if p.size else None,
                                               _p(r) if r.size else None), "wells_set_agents")
        self.counts = c.copy()

    def run_ticks(self, ticks, interactionRad=1.0, springConstant=0.1):
        _check(lib().hal_cuda_wells_run_ticks(self._h, ticks, interactionRad, springConstant),
               "wells_run_ticks")

    def set_motion(self, enabled=True, friction=1.0, maxVel=-1.0):
        """Agents move after their forces each tick (SphericalAgent2D update)."""
        _check(lib().hal_cuda_wells_set_motion(self._h, int(enabled), float(friction), float(maxVel)), "set_motion")

    def set_velocities(self, velocities=None):
        n = 2 * int(self.counts.sum())
        v = None if velocities is None else _f32(velocities)
        _check(lib().hal_cuda_wells_set_velocities(self._h, _p(v), n if v is None else v.size), "set_velocities")

    def get_agents(self):
        """(positions, velocities) of every well's agents, well after well."""
        n = 2 * int(self.counts.sum())
        p = np.empty(n, dtype=np.float32)
        v = np.empty(n, dtype=np.float32)
        _check(lib().hal_cuda_wells_get_agents(self._h, _p(p), _p(v), n), "get_agents")
        return p, v

    def autotune(self):
        """Re-runs the sweep-tile autotuner; returns (rCap, ms tuned, ms default)."""
        cap = ctypes.c_int32()
        a, b = ctypes.c_float(), ctypes.c_float()
        _check(lib().hal_cuda_wells_autotune(self._h, ctypes.byref(cap), ctypes.byref(a), ctypes.byref(b)),
               "wells_autotune")
        return cap.value, a.value, b.value

    def get_forces(self):
        out = np.empty(2 * int(self.counts.sum()), dtype=np.float32)
        _check(lib().hal_cuda_wells_get_forces(self._h, _p(out) if out.size else None, out.size),
               "wells_get_forces")
        return out

    def profile(self, iters, interactionRad=1.0, springConstant=0.1):
        """Average ms per tick: explicit tiles, ADI x, ADI y, agents, whole."""
        ms = np.zeros(5, dtype=np.float32)
        _check(lib().hal_cuda_wells_profile(self._h, iters, interactionRad, springConstant, _p(ms)),
               "wells_profile")
        return [float(v) for v in ms]


ADJOINT_MAX_SIDE = 1024


class Adjoint(_Handle):
    """hal_cuda_adjoint: variable-rate ADI steps and the gradient of
    1/2 |f_T - target|^2 with respect to the rate field D, decay and source."""

    _prefix = "adjoint"

    def __init__(self, xDim, yDim, wrapX=False, wrapY=False):
        super().__init__()
        h = ctypes.c_void_p()
        _check(lib().hal_cuda_adjoint_create(xDim, yDim, int(wrapX), int(wrapY), ctypes.byref(h)),
               "adjoint_create")
        self._h = h
        self.xDim, self.yDim = xDim, yDim

    def sync(self):
        pass

    def set_problem(self, f0, target, steps, checkpoint_every=22):
        a = _f32(f0)
        t = _f32(target)
        _check(lib().hal_cuda_adjoint_set_problem(self._h, _p(a), _p(t), a.size, steps, checkpoint_every),
               "adjoint_set_problem")

    def forward(self, D, decay, src=None, want_field=False):
        d = _f32(D)
        sv = _f32(src)
        loss = ctypes.c_double(0.0)
        fT = np.empty(self.xDim * self.yDim, dtype=np.float32) if want_field else None
        _check(lib().hal_cuda_adjoint_forward(self._h, _p(d), decay, _p(sv), ctypes.byref(loss), _p(fT)),
               "adjoint_forward")
        return (loss.value, fT) if want_field else loss.value

    def gradient(self, D, decay, src=None):
        """Returns (loss, dD, dDecay, dSrc)."""
        d = _f32(D)
        sv = _f32(src)
        n = self.xDim * self.yDim
        gD = np.empty(n, dtype=np.float32)
        gS = np.empty(n, dtype=np.float32)
        loss = ctypes.c_double(0.0)
        gK = ctypes.c_double(0.0)
        _check(lib().hal_cuda_adjoint_gradient(self._h, _p(d), decay, _p(sv), ctypes.byref(loss), _p(gD),
                                               ctypes.byref(gK), _p(gS)), "adjoint_gradient")
        return loss.value, gD, gK.value, gS

    def times(self):
        """(ms of the last forward, ms of the last gradient), device time."""
        a, b = ctypes.c_float(0.0), ctypes.c_float(0.0)
        _check(lib().hal_cuda_adjoint_times(self._h, ctypes.byref(a), ctypes.byref(b)), "adjoint_times")
        return a.value, b.value


NOALLOC_MAX_AGENTS = 65536
NOALLOC_MAX_CELLS = 65536


def agents_forces_noalloc(positions_ptr: int, radii_ptr: int, n: int, velocity_ptr: int,
                          interactionRad: float, springConstant: float, xDim: int, yDim: int,
                          wrapX: bool = False, wrapY: bool = False, stream: int = 0) -> None:
    """hal_cuda_agents_forces_noalloc: agent forces for callers that cannot
    allocate device memory.  The pointers are device addresses (FP32; 2n, n
    and 2n values) owned by the caller; the call only enqueues work on
    `stream` (0: the legacy default stream)."""
    _check(lib().hal_cuda_agents_forces_noalloc(
        ctypes.c_void_p(positions_ptr), ctypes.c_void_p(radii_ptr), n, ctypes.c_void_p(velocity_ptr),
        interactionRad, springConstant, xDim, yDim, int(wrapX), int(wrapY),
        ctypes.c_void_p(stream) if stream else None), "agents_forces_noalloc")
