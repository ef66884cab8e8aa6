"""ctypes bindings for the CPU oracle (TEST INFRASTRUCTURE ONLY).

Two libraries are wrapped:

* ``liboracle.so`` -- the plain-C restatement of the reference CPU path
  (``hal_oracle.c``).  It builds anywhere gcc does and is what the GPU tests,
  the smoke check and the benchmark's CPU-baseline leg compare against.
* ``_ref/libhal_ref.so`` -- the reference's own CPU sources plus
  ``ref_shim.cpp``.  It exists only where the reference tree is present and is
  used to pin the restatement and to write the golden vectors.

Only ``tests/``, ``__graft_entry__.smoke`` and ``bench.py``'s CPU-baseline
leg may import this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libhal_ref.so")


def _reference_tree() -> str:
    """Where the reference HAL-CPP tree is: $HAL_REFERENCE_TREE, else the
    default that oracle/Makefile states (its HAL_REFERENCE_TREE line)."""
    env = os.environ.get("HAL_REFERENCE_TREE")
    if env:
        return env
    with open(os.path.join(HERE, "Makefile")) as fh:
        for line in fh:
            parts = line.split("?=")
            if len(parts) == 2 and parts[0].strip() == "HAL_REFERENCE_TREE":
                return parts[1].strip()
    return ""


REF_TREE = _reference_tree()

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int32)


def build(ref: bool = False) -> None:
    """Compile liboracle.so (and, when the reference tree exists and ``ref``,
    the reference library)."""
    subprocess.run(["make", "-s", "liboracle.so"], cwd=HERE, check=True)
    if ref and os.path.isdir(REF_TREE):
        subprocess.run(["make", "-s", "-j8", "ref", f"REF={REF_TREE}"], cwd=HERE, check=True)


def _ptr(a, kind=_dp):
    if a is None:
        return None
    return a.ctypes.data_as(kind)


def _f64(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.int32)


class _Lib:
    _lib = None
    path = ORACLE_SO

    @classmethod
    def lib(cls):
        if cls._lib is None:
            if not os.path.exists(cls.path):
                raise FileNotFoundError(cls.path)
            cls._lib = ctypes.CDLL(cls.path)
            cls._setup(cls._lib)
        return cls._lib


class Oracle(_Lib):
    """The C restatement."""

    path = ORACLE_SO

    @staticmethod
    def _setup(L):
        i32, f64, vp = ctypes.c_int32, ctypes.c_double, ctypes.c_void_p
        L.oracle_diffusion2.argtypes = [vp, vp, f64, i32, i32, ctypes.c_int, ctypes.c_int, vp]
        L.oracle_adi2.argtypes = [vp, vp, vp, f64, i32, i32, ctypes.c_int, ctypes.c_int, vp]
        L.oracle_adi2_mt.argtypes = [vp, vp, vp, f64, i32, i32, ctypes.c_int, ctypes.c_int, vp,
                                     ctypes.c_int]
        L.oracle_tick.argtypes = [ctypes.c_int, vp, vp, vp, i32, i32, f64, ctypes.c_int,
                                  ctypes.c_int, vp, f64, vp, i32, vp, vp, vp, f64, ctypes.c_int]
        L.oracle_tick.restype = ctypes.c_int
        L.oracle_tick_adv.argtypes = [ctypes.c_int, vp, vp, vp, i32, i32, f64, f64, f64, ctypes.c_int,
                                      ctypes.c_int, vp, f64, vp, i32, vp, vp, vp, f64, ctypes.c_int]
        L.oracle_tick_adv.restype = ctypes.c_int
        L.oracle_agent_bins.argtypes = [vp, i32, i32, i32, vp, vp]
        L.oracle_accumulate_forces.argtypes = [vp, vp, i32, vp, f64, f64, i32, i32, ctypes.c_int,
                                               ctypes.c_int, vp, vp, ctypes.c_int]
        L.oracle_accumulate_forces.restype = ctypes.c_int
        ci = ctypes.c_int
        L.oracle_diffusion2_var.argtypes = [vp, vp, vp, vp, i32, i32, ci, ci]
        L.oracle_advection2.argtypes = [vp, vp, f64, f64, i32, i32, ci, ci]
        L.oracle_advection2_var.argtypes = [vp, vp, vp, vp, i32, i32, ci, ci]
        L.oracle_agents_move.argtypes = [vp, vp, vp, i32, i32, i32, ci, ci, f64, f64]
        L.oracle_agents_move_f32.argtypes = [vp, vp, vp, i32, i32, i32, ci, ci, ctypes.c_float, ctypes.c_float]
        L.oracle_advection2_bc.argtypes = [vp, vp, f64, f64, i32, i32, ci, ci, vp]
        L.oracle_advection2_var_bc.argtypes = [vp, vp, vp, vp, i32, i32, ci, ci, vp, vp, vp]
        L.oracle_dadi_step.argtypes = [vp, vp, i32, i32, ctypes.c_int, ctypes.c_int, f64, vp, vp, vp]
        L.oracle_dadi_loss_grad.argtypes = [vp, vp, vp, f64, vp, i32, i32, ctypes.c_int, ctypes.c_int,
                                            i32, vp, vp, vp, vp]
        L.oracle_dadi_loss_grad.restype = f64
        L.oracle_sum_forces.argtypes = [vp, vp, i32, vp, vp, vp, f64, ci, f64, f64, ci, i32, i32, ci, ci]
        L.oracle_pdegrid_script.argtypes = [i32, i32, ci, ci, vp, vp, vp, i32, vp, vp, vp, vp, vp]
        L.oracle_pdegrid_script.restype = ci
        L.oracle_rand_init.argtypes = [vp, ctypes.c_uint64]
        L.oracle_rand_double.argtypes = [vp]
        L.oracle_rand_double.restype = f64
        L.oracle_rand_int.argtypes = [vp, i32]
        L.oracle_rand_int.restype = i32
        L.oracle_rand_gaussian.argtypes = [vp, f64, f64]
        L.oracle_rand_gaussian.restype = f64

    # -- explicit / ADI ----------------------------------------------------
    @classmethod
    def diffuse(cls, field, deltas, r, xDim, yDim, wrapX, wrapY, ghost=None):
        """deltas += r * L(field) (in place on a float64 copy, returned)."""
        f = _f64(field)
        d = _f64(deltas).copy()
        g = _f64(ghost)
        cls.lib().oracle_diffusion2(f.ctypes.data, d.ctypes.data, r, xDim, yDim, int(wrapX),
                                    int(wrapY), None if g is None else g.ctypes.data)
        return d

    @classmethod
    def diffuse_adi(cls, field, deltas, r, xDim, yDim, wrapX, wrapY, ghost=None, threads=1):
        f = _f64(field)
        d = _f64(deltas).copy()
        g = _f64(ghost)
        s = np.zeros_like(f)
        cls.lib().oracle_adi2_mt(f.ctypes.data, s.ctypes.data, d.ctypes.data, r, xDim, yDim,
                                 int(wrapX), int(wrapY), None if g is None else g.ctypes.data,
                                 int(threads))
        return d

    @classmethod
    def run_ticks(cls, mode, field, xDim, yDim, r, wrapX=False, wrapY=False, ghost=None,
                  decay=0.0, src_dense=None, src_idx=None, src_val=None, uptake_count=None,
                  uptake=0.0, ticks=1, threads=1, xVel=0.0, yVel=0.0):
        """Run ``ticks`` PDEGrid2D ticks (mode 0 explicit, 1 ADI); returns the
        final field (float64)."""
        f = _f64(field).copy()
        n = xDim * yDim
        d = np.zeros(n, dtype=np.float64)
        s = np.zeros(n, dtype=np.float64)
        g = _f64(ghost)
        sd = _f64(src_dense)
        si = _i32(src_idx)
        sv = _f64(src_val)
        uc = _i32(uptake_count)
        ns = 0 if si is None else len(si)
        L = cls.lib()
        for _ in range(ticks):
            rc = L.oracle_tick_adv(mode, f.ctypes.data, d.ctypes.data, s.ctypes.data, xDim, yDim, r,
                                   float(xVel), float(yVel), int(wrapX), int(wrapY),
                                   None if g is None else g.ctypes.data,
                                   decay, None if sd is None else sd.ctypes.data, ns,
                                   None if si is None else si.ctypes.data,
                                   None if sv is None else sv.ctypes.data,
                                   None if uc is None else uc.ctypes.data, uptake, int(threads))
            if rc == -1:
                raise ValueError("Diffusion rate above stable maximum value of 0.25")
            if rc != 0:
                raise ValueError("Advection rate component sum above stable maximum value of 0.5")
        return f

    # -- agents ------------------------------------------------------------
    @classmethod
    def accumulate_forces(cls, positions, radii, R, k, xDim, yDim, wrapX, wrapY, threads=1):
        """Returns (velocityDeltas[2n], cellOffsets[C+1], bucketAgents[n])."""
        p = _f64(positions)
        rad = _f64(radii)
        n = len(rad)
        if len(p) != 2 * n:
            raise ValueError("positions must hold two values per radius")
        out = np.zeros(2 * n, dtype=np.float64)
        off = np.zeros(xDim * yDim + 1, dtype=np.int32)
        bucket = np.zeros(max(n, 1), dtype=np.int32)
        cls.lib().oracle_accumulate_forces(p.ctypes.data, rad.ctypes.data, n, out.ctypes.data, R,
                                           k, xDim, yDim, int(wrapX), int(wrapY),
                                           off.ctypes.data, bucket.ctypes.data, int(threads))
        return out, off, bucket[:n]

    @classmethod
    def sum_forces(cls, positions, radii, R, law, scale, xDim, yDim, wrapX, wrapY, vel=None, exponent=1.0,
                   order=1):
        """SphericalAgent2D::SumForces of every agent; returns (velocities
        after the call [2n], sums of positive forces [n]).  law 0 linear, 1
        clamped, 2 power; order 1 the agent grid's, 0 the CPU backend's."""
        p = _f64(positions)
        rad = _f64(radii)
        n = len(rad)
        v = None if vel is None else _f64(vel)
        out = np.zeros(2 * n, dtype=np.float64)
        sums = np.zeros(max(n, 1), dtype=np.float64)
        cls.lib().oracle_sum_forces(p.ctypes.data, rad.ctypes.data, n, None if v is None else v.ctypes.data,
                                    out.ctypes.data, sums.ctypes.data, R, int(law), float(scale), float(exponent),
                                    int(order), xDim, yDim, int(wrapX), int(wrapY))
        return out, sums[:n]

    @classmethod
    def pdegrid_script(cls, script, field, deltas=None, update_ct=0):
        """Runs a PDEScript on a PDEGrid2D in the given state; returns
        (field, deltas, updateCt, records)."""
        f, d, uc, args = script.prepare(field, deltas, update_ct)
        n = cls.lib().oracle_pdegrid_script(script.xDim, script.yDim, int(script.wrapX), int(script.wrapY),
                                            f.ctypes.data, d.ctypes.data, ctypes.addressof(uc), *args)
        if n == -1:
            raise ValueError("Diffusion rate above stable maximum value of 0.25")
        if n == -2:
            raise ValueError("Advection rate component sum above stable maximum value of 0.5")
        return f, d, uc.value, script.records[:n].copy()

    @classmethod
    def agent_bins(cls, positions, xDim, yDim):
        p = _f64(positions)
        n = len(p) // 2
        off = np.zeros(xDim * yDim + 1, dtype=np.int32)
        bucket = np.zeros(max(n, 1), dtype=np.int32)
        cls.lib().oracle_agent_bins(p.ctypes.data, n, xDim, yDim, off.ctypes.data,
                                    bucket.ctypes.data)
        return off, bucket[:n]

    # -- Hal::Rand -----------------------------------------------------------
    @classmethod
    def rand_draws(cls, seed, kind, n, bound=1):
        st = (ctypes.c_byte * 128)()
        L = cls.lib()
        L.oracle_rand_init(ctypes.addressof(st), seed)
        out = np.zeros(n, dtype=np.float64)
        for i in range(n):
            if kind == 0:
                out[i] = L.oracle_rand_double(ctypes.addressof(st))
            elif kind == 1:
                out[i] = L.oracle_rand_int(ctypes.addressof(st), bound)
            else:
                out[i] = L.oracle_rand_gaussian(ctypes.addressof(st), 0.0, 1.0)
        return out


    @classmethod
    def diffuse_var(cls, field, deltas, ratesX, ratesY, xDim, yDim, wrapX, wrapY):
        f, rx, ry = _f64(field), _f64(ratesX), _f64(ratesY)
        d = _f64(deltas).copy()
        cls.lib().oracle_diffusion2_var(f.ctypes.data, d.ctypes.data, rx.ctypes.data, ry.ctypes.data, xDim, yDim,
                                        int(wrapX), int(wrapY))
        return d

    @classmethod
    def advect(cls, field, deltas, xVel, yVel, xDim, yDim, wrapX, wrapY, ghost=None):
        f = _f64(field)
        d = _f64(deltas).copy()
        if ghost is None:
            cls.lib().oracle_advection2(f.ctypes.data, d.ctypes.data, xVel, yVel, xDim, yDim, int(wrapX), int(wrapY))
        else:
            g = _f64(ghost)
            cls.lib().oracle_advection2_bc(f.ctypes.data, d.ctypes.data, xVel, yVel, xDim, yDim, int(wrapX),
                                           int(wrapY), g.ctypes.data)
        return d

    @classmethod
    def advect_var(cls, field, deltas, xVels, yVels, xDim, yDim, wrapX, wrapY, ghost=None, ghost_vx=None,
                   ghost_vy=None):
        f, vx, vy = _f64(field), _f64(xVels), _f64(yVels)
        d = _f64(deltas).copy()
        if ghost is None and ghost_vx is None and ghost_vy is None:
            cls.lib().oracle_advection2_var(f.ctypes.data, d.ctypes.data, vx.ctypes.data, vy.ctypes.data, xDim,
                                            yDim, int(wrapX), int(wrapY))
        else:
            gs = [None if g is None else _f64(g) for g in (ghost, ghost_vx, ghost_vy)]
            cls.lib().oracle_advection2_var_bc(f.ctypes.data, d.ctypes.data, vx.ctypes.data, vy.ctypes.data, xDim,
                                               yDim, int(wrapX), int(wrapY),
                                               *[None if g is None else g.ctypes.data for g in gs])
        return d

    @classmethod
    def agents_move(cls, pos, vel, deltas, xDim, yDim, wrapX, wrapY, friction, maxVel, f32=False):
        """SphericalAgent2D's update after its forces; returns (pos, vel).
        f32 runs the same steps in float, the precision of the device step."""
        if f32:
            p = np.array(pos, dtype=np.float32)
            v = np.array(vel, dtype=np.float32)
            d = np.ascontiguousarray(deltas, dtype=np.float32)
            cls.lib().oracle_agents_move_f32(p.ctypes.data, v.ctypes.data, d.ctypes.data, p.size // 2, xDim, yDim,
                                             int(wrapX), int(wrapY), float(friction), float(maxVel))
        else:
            p = np.array(pos, dtype=np.float64)
            v = np.array(vel, dtype=np.float64)
            d = _f64(deltas)
            cls.lib().oracle_agents_move(p.ctypes.data, v.ctypes.data, d.ctypes.data, p.size // 2, xDim, yDim,
                                         int(wrapX), int(wrapY), float(friction), float(maxVel))
        return p, v

    @classmethod
    def dadi_step(cls, field, D, xDim, yDim, wrapX=False, wrapY=False, decay=0.0, src=None):
        """One variable-rate ADI step; returns (f', w)."""
        f = _f64(field)
        d = _f64(D)
        sv = _f64(src)
        w = np.zeros(xDim * yDim)
        out = np.zeros(xDim * yDim)
        cls.lib().oracle_dadi_step(f.ctypes.data, d.ctypes.data, xDim, yDim, int(wrapX), int(wrapY), decay,
                                   None if sv is None else sv.ctypes.data, w.ctypes.data, out.ctypes.data)
        return out, w

    @classmethod
    def dadi_loss_grad(cls, f0, target, D, decay, src, xDim, yDim, steps, wrapX=False, wrapY=False,
                       grad=True):
        """Loss 1/2|f_T - target|^2 of `steps` variable-rate ADI steps and, with
        grad, its gradients: returns (loss, f_T, dD, dDecay, dSrc)."""
        f = _f64(f0)
        t = _f64(target)
        d = _f64(D)
        sv = _f64(src)
        n = xDim * yDim
        fT = np.zeros(n)
        gD = np.zeros(n) if grad else None
        gS = np.zeros(n) if grad else None
        gK = ctypes.c_double(0.0)
        loss = cls.lib().oracle_dadi_loss_grad(
            f.ctypes.data, t.ctypes.data, d.ctypes.data, decay, None if sv is None else sv.ctypes.data, xDim, yDim,
            int(wrapX), int(wrapY), steps, fT.ctypes.data, None if gD is None else gD.ctypes.data,
            ctypes.byref(gK) if grad else None, None if gS is None else gS.ctypes.data)
        return loss, fT, gD, (gK.value if grad else None), gS


def _ok(rc):
    """Status of a reference shim call: 1 invalid_argument, 2 other error."""
    if rc == 1:
        raise ValueError("invalid_argument")
    if rc != 0:
        raise RuntimeError("reference error")


class Reference(_Lib):
    """The reference's own CPU code (only where the reference tree was built)."""

    path = REF_SO

    @classmethod
    def available(cls):
        return os.path.exists(REF_SO)

    @staticmethod
    def _setup(L):
        i32, i64, f64, vp, ci = (ctypes.c_int32, ctypes.c_int64, ctypes.c_double, ctypes.c_void_p,
                                 ctypes.c_int)
        L.ref_diffuse.argtypes = [vp, i64, vp, i64, f64, i32, i32, ci, ci]
        L.ref_diffuse_bc.argtypes = [vp, vp, f64, i32, i32, ci, ci, vp]
        L.ref_diffuse_adi.argtypes = [vp, i64, vp, i64, f64, i32, i32, ci, ci]
        L.ref_diffuse_adi_bc.argtypes = [vp, vp, f64, i32, i32, ci, ci, vp]
        L.ref_pdegrid_run.argtypes = [ci, vp, i32, i32, ci, ci, f64, vp, f64, vp, i32, vp, vp, vp,
                                      f64, i32]
        L.ref_pdegrid_run_adv.argtypes = [ci, vp, i32, i32, ci, ci, f64, f64, f64, vp, f64, vp, i32, vp, vp,
                                          vp, f64, i32]
        L.ref_accumulate_forces.argtypes = [vp, i64, vp, i64, vp, f64, f64, i32, i32, ci, ci, vp,
                                            vp]
        L.ref_rand_draws.argtypes = [ctypes.c_uint64, ci, i32, i32, vp]
        L.ref_diffuse_var.argtypes = [vp, vp, vp, vp, i32, i32, ci, ci]
        L.ref_advect.argtypes = [vp, vp, f64, f64, i32, i32, ci, ci]
        L.ref_advect_var.argtypes = [vp, vp, vp, vp, i32, i32, ci, ci]
        L.ref_agents_move.argtypes = [vp, vp, vp, i32, i32, i32, ci, ci, f64, f64]
        L.ref_pdegrid2d_save.argtypes = [ctypes.c_char_p, i32, i32, ci, ci, i32, vp, vp]
        L.ref_pdegrid2d_load.argtypes = [ctypes.c_char_p, vp, vp, vp, vp, ctypes.c_int64]
        L.ref_advect_bc.argtypes = [vp, vp, f64, f64, i32, i32, ci, ci, vp]
        L.ref_sum_forces.argtypes = [vp, vp, vp, i32, i32, i32, ci, ci, f64, ci, f64, f64, vp, vp]
        L.ref_pdegrid_script.argtypes = [i32, i32, ci, ci, vp, vp, vp, i32, vp, vp, vp, vp, vp, vp]
        L.ref_advect_var_bc.argtypes = [vp, vp, vp, vp, i32, i32, ci, ci, vp, vp, vp]
        for name in ("ref_diffuse", "ref_diffuse_bc", "ref_diffuse_adi", "ref_diffuse_adi_bc",
                     "ref_pdegrid_run", "ref_accumulate_forces"):
            getattr(L, name).restype = ci

    @classmethod
    def diffuse_var(cls, field, deltas, ratesX, ratesY, xDim, yDim, wrapX, wrapY):
        f, rx, ry = _f64(field), _f64(ratesX), _f64(ratesY)
        d = _f64(deltas).copy()
        _ok(cls.lib().ref_diffuse_var(f.ctypes.data, d.ctypes.data, rx.ctypes.data, ry.ctypes.data, xDim, yDim,
                                      int(wrapX), int(wrapY)))
        return d

    @classmethod
    def advect(cls, field, deltas, xVel, yVel, xDim, yDim, wrapX, wrapY, ghost=None):
        f = _f64(field)
        d = _f64(deltas).copy()
        if ghost is None:
            _ok(cls.lib().ref_advect(f.ctypes.data, d.ctypes.data, xVel, yVel, xDim, yDim, int(wrapX), int(wrapY)))
        else:
            g = _f64(ghost)
            _ok(cls.lib().ref_advect_bc(f.ctypes.data, d.ctypes.data, xVel, yVel, xDim, yDim, int(wrapX), int(wrapY),
                                        g.ctypes.data))
        return d

    @classmethod
    def advect_var(cls, field, deltas, xVels, yVels, xDim, yDim, wrapX, wrapY, ghost=None, ghost_vx=None,
                   ghost_vy=None):
        f, vx, vy = _f64(field), _f64(xVels), _f64(yVels)
        d = _f64(deltas).copy()
        if ghost is None:
            _ok(cls.lib().ref_advect_var(f.ctypes.data, d.ctypes.data, vx.ctypes.data, vy.ctypes.data, xDim, yDim,
                                         int(wrapX), int(wrapY)))
        else:
            g, gx, gy = _f64(ghost), _f64(ghost_vx), _f64(ghost_vy)
            _ok(cls.lib().ref_advect_var_bc(f.ctypes.data, d.ctypes.data, vx.ctypes.data, vy.ctypes.data, xDim,
                                            yDim, int(wrapX), int(wrapY), g.ctypes.data, gx.ctypes.data,
                                            gy.ctypes.data))
        return d

    @classmethod
    def pdegrid_script(cls, script, field, deltas=None, update_ct=0):
        """The same script on the reference's own Hal::PDEGrid2D."""
        f, d, uc, args = script.prepare(field, deltas, update_ct)
        nrec = ctypes.c_int32(0)
        _ok(cls.lib().ref_pdegrid_script(script.xDim, script.yDim, int(script.wrapX), int(script.wrapY),
                                         f.ctypes.data, d.ctypes.data, ctypes.addressof(uc), *args,
                                         ctypes.addressof(nrec)))
        return f, d, uc.value, script.records[:nrec.value].copy()

    @classmethod
    def sum_forces(cls, positions, radii, R, law, scale, xDim, yDim, wrapX, wrapY, vel=None, exponent=1.0):
        """SphericalAgent2D::SumForces on the reference's agent grid; returns
        (velocities after the call, sums of positive forces)."""
        p, rad = _f64(positions), _f64(radii)
        n = len(rad)
        v = None if vel is None else _f64(vel)
        out = np.zeros(2 * n, dtype=np.float64)
        sums = np.zeros(max(n, 1), dtype=np.float64)
        _ok(cls.lib().ref_sum_forces(p.ctypes.data, rad.ctypes.data, None if v is None else v.ctypes.data, n, xDim,
                                     yDim, int(wrapX), int(wrapY), R, int(law), float(scale), float(exponent),
                                     out.ctypes.data, sums.ctypes.data))
        return out, sums[:n]

    @classmethod
    def agents_move(cls, pos, vel, deltas, xDim, yDim, wrapX, wrapY, friction, maxVel):
        p = np.array(pos, dtype=np.float64)
        v = np.array(vel, dtype=np.float64)
        d = _f64(deltas)
        _ok(cls.lib().ref_agents_move(p.ctypes.data, v.ctypes.data, d.ctypes.data, p.size // 2, xDim, yDim,
                                      int(wrapX), int(wrapY), float(friction), float(maxVel)))
        return p, v

    @classmethod
    def pdegrid2d_save(cls, path, xDim, yDim, wrapX, wrapY, updateCt, field, deltas):
        f, d = _f64(field), _f64(deltas)
        _ok(cls.lib().ref_pdegrid2d_save(os.fsencode(path), xDim, yDim, int(wrapX), int(wrapY), updateCt,
                                         f.ctypes.data, d.ctypes.data))

    @classmethod
    def pdegrid2d_load(cls, path, cap=1 << 22):
        """LoadPDEGrid2D: (xDim, yDim, wrapX, wrapY, updateCt, field, deltas);
        raises RuntimeError where the reference throws."""
        dims = np.zeros(4, dtype=np.int32)
        u = np.zeros(1, dtype=np.int32)
        f = np.zeros(cap)
        d = np.zeros(cap)
        rc = cls.lib().ref_pdegrid2d_load(os.fsencode(path), dims.ctypes.data, u.ctypes.data, f.ctypes.data,
                                          d.ctypes.data, cap)
        if rc != 0:
            raise RuntimeError(f"LoadPDEGrid2D failed ({rc})")
        n = int(dims[0]) * int(dims[1])
        return int(dims[0]), int(dims[1]), bool(dims[2]), bool(dims[3]), int(u[0]), f[:n].copy(), d[:n].copy()

    @classmethod
    def diffuse(cls, field, deltas, r, xDim, yDim, wrapX, wrapY, ghost=None):
        f = _f64(field)
        d = _f64(deltas).copy()
        L = cls.lib()
        if ghost is None:
            rc = L.ref_diffuse(f.ctypes.data, len(f), d.ctypes.data, len(d), r, xDim, yDim,
                               int(wrapX), int(wrapY))
        else:
            g = _f64(ghost)
            rc = L.ref_diffuse_bc(f.ctypes.data, d.ctypes.data, r, xDim, yDim, int(wrapX),
                                  int(wrapY), g.ctypes.data)
        if rc == 1:
            raise ValueError("invalid_argument")
        if rc != 0:
            raise RuntimeError("reference error")
        return d

    @classmethod
    def diffuse_adi(cls, field, deltas, r, xDim, yDim, wrapX, wrapY, ghost=None):
        f = _f64(field)
        d = _f64(deltas).copy()
        L = cls.lib()
        if ghost is None:
            rc = L.ref_diffuse_adi(f.ctypes.data, len(f), d.ctypes.data, len(d), r, xDim, yDim,
                                   int(wrapX), int(wrapY))
        else:
            g = _f64(ghost)
            rc = L.ref_diffuse_adi_bc(f.ctypes.data, d.ctypes.data, r, xDim, yDim, int(wrapX),
                                      int(wrapY), g.ctypes.data)
        if rc == 1:
            raise ValueError("invalid_argument")
        if rc != 0:
            raise RuntimeError("reference error")
        return d

    @classmethod
    def run_ticks(cls, mode, field, xDim, yDim, r, wrapX=False, wrapY=False, ghost=None,
                  decay=0.0, src_dense=None, src_idx=None, src_val=None, uptake_count=None,
                  uptake=0.0, ticks=1, xVel=0.0, yVel=0.0):
        f = _f64(field).copy()
        g, sd, si, sv, uc = _f64(ghost), _f64(src_dense), _i32(src_idx), _f64(src_val), \
            _i32(uptake_count)
        ns = 0 if si is None else len(si)
        rc = cls.lib().ref_pdegrid_run_adv(mode, f.ctypes.data, xDim, yDim, int(wrapX), int(wrapY),
                                       r, float(xVel), float(yVel), None if g is None else g.ctypes.data, decay,
                                       None if sd is None else sd.ctypes.data, ns,
                                       None if si is None else si.ctypes.data,
                                       None if sv is None else sv.ctypes.data,
                                       None if uc is None else uc.ctypes.data, uptake, ticks)
        if rc == 1:
            raise ValueError("invalid_argument")
        if rc != 0:
            raise RuntimeError("reference error")
        return f

    @classmethod
    def accumulate_forces(cls, positions, radii, R, k, xDim, yDim, wrapX, wrapY):
        p = _f64(positions)
        rad = _f64(radii)
        n = len(rad)
        out = np.zeros(len(p), dtype=np.float64)
        off = np.zeros(xDim * yDim + 1, dtype=np.int32)
        bucket = np.zeros(max(n, 1), dtype=np.int32)
        rc = cls.lib().ref_accumulate_forces(p.ctypes.data, len(p), rad.ctypes.data, n,
                                             out.ctypes.data, R, k, xDim, yDim, int(wrapX),
                                             int(wrapY), off.ctypes.data, bucket.ctypes.data)
        if rc == 1:
            raise ValueError("invalid_argument")
        if rc != 0:
            raise RuntimeError("reference error")
        return out, off, bucket[:n]

    @classmethod
    def rand_draws(cls, seed, kind, n, bound=1):
        out = np.zeros(n, dtype=np.float64)
        cls.lib().ref_rand_draws(seed, kind, bound, n, out.ctypes.data)
        return out


class PDEScript:
    """A sequence of Hal::PDEGrid2D calls on one grid, in the encoding of
    oracle_pdegrid_script (hal_oracle.h): the oracle, the reference library
    and the device handle all run the same script.  Each method appends one
    call; `calls` keeps them as (name, args) for runners that replay them."""

    OPS = {"set": 0, "add": 1, "mul": 2, "scale": 3, "set_all": 10, "add_all": 11, "mul_all": 12,
           "set_all_values": 13, "diffusion": 20, "diffusion_bc": 21, "diffusion_var": 22, "adi": 30,
           "adi_bc": 31, "advection": 40, "advection_bc": 41, "advection_var": 42, "advection_var_bc": 43,
           "update": 50, "set_non_negative": 51, "get": 60, "max": 61, "min": 62, "avg": 63, "max_delta": 64,
           "max_delta_scaled": 65, "gradient_x": 66, "gradient_y": 67, "gradient_x_bc": 68, "gradient_y_bc": 69}

    def __init__(self, xDim, yDim, wrapX=False, wrapY=False):
        self.xDim, self.yDim, self.wrapX, self.wrapY = xDim, yDim, bool(wrapX), bool(wrapY)
        self.calls = []

    def encoded(self):
        """(ops, iargs, dargs, arrays) of the script, for storing it."""
        self.prepare(np.zeros(self.xDim * self.yDim), None, 0)
        return self._keep

    @classmethod
    def from_encoded(cls, xDim, yDim, wrapX, wrapY, ops, iargs, dargs, arrays):
        """The script that `encoded` stored."""
        sc = cls(int(xDim), int(yDim), bool(wrapX), bool(wrapY))
        names = {v: k for k, v in cls.OPS.items()}
        n, g = sc.xDim * sc.yDim, 2 * (sc.xDim + sc.yDim)
        sizes = {13: [n], 21: [g], 31: [g], 41: [g], 22: [n, n], 42: [n, n], 43: [n, n, g, g, g]}
        for k, op in enumerate(ops):
            op = int(op)
            off = int(iargs[3 * k])
            arrs = None
            if op in sizes:
                arrs = []
                for m in sizes[op]:
                    arrs.append(np.array(arrays[off: off + m]))
                    off += m
            i_or_x, y = int(iargs[3 * k + 1]), int(iargs[3 * k + 2])
            grad = names[op].startswith("gradient")
            sc.add(names[op], i=0 if grad else i_or_x, x=i_or_x if grad else 0, y=y, d0=float(dargs[2 * k]),
                   d1=float(dargs[2 * k + 1]), arrays=arrs)
        return sc

    def add(self, name, i=0, x=0, y=0, d0=0.0, d1=0.0, arrays=None):
        self.calls.append((name, dict(i=i, x=x, y=y, d0=d0, d1=d1, arrays=arrays)))
        return self

    def prepare(self, field, deltas, update_ct):
        n = self.xDim * self.yDim
        f = np.array(field, dtype=np.float64).copy()
        d = np.zeros(n) if deltas is None else np.array(deltas, dtype=np.float64).copy()
        ops = np.array([self.OPS[c] for c, _ in self.calls], dtype=np.int32)
        iargs = np.zeros(3 * max(len(self.calls), 1), dtype=np.int32)
        dargs = np.zeros(2 * max(len(self.calls), 1))
        chunks, off = [], 0
        for k, (name, a) in enumerate(self.calls):
            if a["arrays"] is not None:
                arr = np.concatenate([np.asarray(v, dtype=np.float64).ravel() for v in a["arrays"]])
                iargs[3 * k] = off
                chunks.append(arr)
                off += arr.size
            iargs[3 * k + 1] = a["x"] if name.startswith("gradient") else a["i"]
            iargs[3 * k + 2] = a["y"]
            dargs[2 * k], dargs[2 * k + 1] = a["d0"], a["d1"]
        arrays = np.concatenate(chunks) if chunks else np.zeros(1)
        self.records = np.zeros(max(len(self.calls), 1))
        self._keep = (ops, iargs, dargs, arrays)
        uc = ctypes.c_int32(update_ct)
        return f, d, uc, (len(self.calls), ops.ctypes.data, iargs.ctypes.data, dargs.ctypes.data,
                          arrays.ctypes.data, self.records.ctypes.data)
