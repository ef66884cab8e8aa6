"""Writes the golden vectors in this folder from the reference's own CPU code.

Run in a tree where the reference sources exist (it builds
``oracle/_ref/libhal_ref.so`` from them through ``oracle/Makefile``):

    python tests/golden/make_golden.py             # every fixture
    python tests/golden/make_golden.py sumforces   # only the named ones

Every output comes from Hal::CpuDiffusionBackend2D, Hal::CpuAdiDiffusionBackend2D,
Hal::CpuAgentForceBackend2D, Hal::PDEGrid2D (single ticks and whole call
sequences), Hal::SphericalAgent2D on the reference's agent grid or Hal::Rand,
called through
``oracle/ref_shim.cpp``.  The inputs are stored beside the outputs, so the
fixtures need no random generator to be replayed.  Cases restate the
reference's own tests (eigenmode decay, the seed-1234 agent scene, Dirichlet
fixed points) plus random odd-sized and edge-case grids.
"""
from __future__ import annotations

import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import pyoracle  # noqa: E402
from pyoracle import Reference as R  # noqa: E402

SIZES = [(17, 29), (1, 7), (7, 1), (1, 1), (2, 2), (3, 5), (9, 40), (40, 9)]
BIG = [(33, 64, 0, 0, 0), (64, 33, 1, 1, 1), (33, 64, 1, 0, 1)]


def _eigen(nx, ny):
    x = np.arange(nx)[:, None]
    y = np.arange(ny)[None, :]
    return (np.sin(2.0 * math.pi * x / nx) * np.sin(2.0 * math.pi * y / ny)).ravel()


def stencil_cases(rng):
    out = {}
    k = 0
    for (xd, yd) in SIZES:
        for wx in (0, 1):
            for wy in (0, 1):
                for use_bc in (0, 1):
                    f = rng.random(xd * yd)
                    d = rng.random(xd * yd) - 0.5
                    g = rng.random(2 * (xd + yd)) if use_bc else None
                    r_exp = 0.2
                    r_adi = [0.3, 5.0][k % 2]
                    out[f"c{k}_dims"] = np.array([xd, yd, wx, wy, use_bc], dtype=np.int32)
                    out[f"c{k}_rates"] = np.array([r_exp, r_adi])
                    out[f"c{k}_field"] = f
                    out[f"c{k}_deltas"] = d
                    if use_bc:
                        out[f"c{k}_ghost"] = g
                    out[f"c{k}_explicit"] = R.diffuse(f, d, r_exp, xd, yd, wx, wy, g)
                    out[f"c{k}_adi"] = R.diffuse_adi(f, d, r_adi, xd, yd, wx, wy, g)
                    k += 1
    for (xd, yd, wx, wy, use_bc) in BIG:
        f = rng.random(xd * yd)
        d = np.zeros(xd * yd)
        g = rng.random(2 * (xd + yd)) if use_bc else None
        out[f"c{k}_dims"] = np.array([xd, yd, wx, wy, use_bc], dtype=np.int32)
        out[f"c{k}_rates"] = np.array([0.25, 10.0])
        out[f"c{k}_field"] = f
        out[f"c{k}_deltas"] = d
        if use_bc:
            out[f"c{k}_ghost"] = g
        out[f"c{k}_explicit"] = R.diffuse(f, d, 0.25, xd, yd, wx, wy, g)
        out[f"c{k}_adi"] = R.diffuse_adi(f, d, 10.0, xd, yd, wx, wy, g)
        k += 1
    out["count"] = np.array([k])
    # the reference's own interface tests (tests/IDiffusionBackend2DTests.cpp:23-113)
    f = _eigen(16, 20)
    out["eig_explicit_field"] = f
    out["eig_explicit_out"] = R.diffuse(f, np.zeros_like(f), 0.05, 16, 20, 1, 1)
    f = _eigen(12, 18)
    out["eig_adi_field"] = f
    out["eig_adi_out"] = R.diffuse_adi(f, np.zeros_like(f), 0.3, 12, 18, 1, 1)
    return out


def tick_cases(rng):
    out = {}
    # Explicit PDEGrid2D tick with a Dirichlet edge, decay and point sources
    # (the shape of the 256x256 explicit workload, scaled down).
    xd, yd = 32, 40
    f = rng.random(xd * yd)
    ghost = np.zeros(2 * (xd + yd))
    ghost[:yd] = 1.0  # bc(-1, y) = 1, every other edge 0
    sites = rng.choice(xd * yd, 12, replace=False).astype(np.int32)
    vals = np.full(12, 0.05)
    out["exp_field"] = f
    out["exp_ghost"] = ghost
    out["exp_src_idx"] = sites
    out["exp_src_val"] = vals
    out["exp_params"] = np.array([xd, yd, 0.2, 0.001, 150])
    out["exp_out"] = R.run_ticks(0, f, xd, yd, 0.2, False, False, ghost, 0.001, None, sites,
                                 vals, ticks=150)
    # ADI tick with decay and a dense source (the 2048^2 ADI workload, scaled down)
    xd, yd = 40, 48
    f = rng.random(xd * yd)
    src = rng.random(xd * yd) * 0.01
    out["adi_field"] = f
    out["adi_src"] = src
    out["adi_params"] = np.array([xd, yd, 5.0, 0.01, 20])
    out["adi_out"] = R.run_ticks(1, f, xd, yd, 5.0, False, False, None, 0.01, src, ticks=20)
    # ADI tick with periodic x, Dirichlet y ends, and agent uptake counts
    xd, yd = 21, 30
    f = rng.random(xd * yd)
    ghost = rng.random(2 * (xd + yd))
    counts = rng.integers(0, 4, xd * yd).astype(np.int32)
    out["cpl_field"] = f
    out["cpl_ghost"] = ghost
    out["cpl_counts"] = counts
    out["cpl_params"] = np.array([xd, yd, 1.7, 0.005, 0.001, 9])
    out["cpl_out"] = R.run_ticks(1, f, xd, yd, 1.7, True, False, ghost, 0.005, None, None, None,
                                 counts, 0.001, ticks=9)
    # the ADI GPU-vs-CPU case of tests/AdiKernel2DTests.cpp:70-141
    nx, ny = 20, 14
    x = np.arange(nx)[:, None]
    y = np.arange(ny)[None, :]
    f = (1.0 + 0.3 * x - 0.2 * y + 0.5 * np.sin(0.7 * x * y)).ravel()
    out["kat_adi_field"] = f
    out["kat_adi_out"] = R.run_ticks(1, f, nx, ny, 0.6, False, False, ticks=5)
    return out


def agent_cases(rng):
    out = {}
    # The seed-1234 scene of tests/IAgentForceBackend2DTests.cpp:25-37:
    # Rand(1234); x = Double(16), y = Double(16), radius = 0.4 + Double(0.4).
    u = R.rand_draws(1234, 0, 180)
    pos = np.empty(120)
    pos[0::2] = u[0::3] * 16.0
    pos[1::2] = u[1::3] * 16.0
    rad = 0.4 + u[2::3] * 0.4
    v, off, b = R.accumulate_forces(pos, rad, 3.0, 0.4, 16, 16, 1, 1)
    out.update(s1234_pos=pos, s1234_rad=rad, s1234_vel=v, s1234_off=off, s1234_bucket=b)
    # float32 positions, walls, a dense cluster plus stragglers outside the domain
    cases = [
        ("walls", 64, 48, 3000, 0, 0, 1.0, 0.1),
        ("torus", 37, 23, 1500, 1, 1, 1.0, 0.1),
        ("mixed", 30, 50, 2000, 1, 0, 2.3, 0.3),
        ("tiny", 1, 1, 5, 0, 0, 1.0, 0.1),
        ("empty", 8, 8, 0, 0, 0, 2.0, 1.0),
    ]
    for (name, xd, yd, n, wx, wy, R_, k) in cases:
        m = int(n * 0.3)
        uni = rng.random((n - m, 2)) * np.array([xd, yd]) * 1.1 - 0.05 * np.array([xd, yd])
        clu = rng.normal(0.0, 1.0, (m, 2)) * np.array([xd, yd]) * 0.08 + \
            np.array([xd, yd]) * 0.4
        p = np.concatenate([uni, clu]).astype(np.float32).astype(np.float64).ravel()
        if n >= 4:
            p[2:4] = p[0:2]  # two coincident agents
        rad = np.full(n, 0.5)
        v, off, b = R.accumulate_forces(p, rad, R_, k, xd, yd, wx, wy)
        out[f"{name}_pos"] = p
        out[f"{name}_rad"] = rad
        out[f"{name}_params"] = np.array([xd, yd, n, wx, wy, R_, k])
        out[f"{name}_vel"] = v
        out[f"{name}_off"] = off
        out[f"{name}_bucket"] = b
    # coincident-agent no-NaN case (tests/IAgentForceBackend2DTests.cpp:153-165)
    v, off, b = R.accumulate_forces([4.0, 4.0, 4.0, 4.0], [0.5, 0.5], 2.0, 1.0, 8, 8, 0, 0)
    out["coincident_vel"] = v
    return out


def rand_cases():
    out = {}
    for seed in (1, 7, 1234):
        out[f"double_{seed}"] = R.rand_draws(seed, 0, 64)
        out[f"int256_{seed}"] = R.rand_draws(seed, 1, 64, 256)
        out[f"gauss_{seed}"] = R.rand_draws(seed, 2, 64)
    return out


def var_stencil_cases(rng):
    """Internal::Diffusion2 with per-cell rates and both Advection2 forms
    (src/Pde/PDEequations.cpp:199-230, 380-412, 535-575), each advection form
    also with Dirichlet ghost tables (include/Hal/Pde/PDEequations.h:413-447,
    720-778)."""
    out = {}
    k = 0
    grng = np.random.default_rng(8282)  # ghost tables, drawn apart so the other vectors stay as they were
    for (xd, yd) in SIZES:
        n = xd * yd
        for wx, wy in ((0, 0), (1, 1), (1, 0), (0, 1)):
            f = rng.random(n)
            d = rng.random(n) * 0.1
            rx = rng.random(n) * 0.24
            ry = rng.random(n) * 0.24
            vx = rng.random(n) - 0.5
            vy = rng.random(n) - 0.5
            vx[::7] = 0.0  # zero velocity faces take neither branch
            xv, yv = [(0.2, -0.1), (-0.3, 0.15), (0.0, 0.2), (0.1, 0.0)][k % 4]
            pre = f"c{k}_"
            out[pre + "dims"] = np.array([xd, yd, wx, wy], dtype=np.int32)
            out[pre + "vel"] = np.array([xv, yv])
            for key, v in (("f", f), ("d", d), ("rx", rx), ("ry", ry), ("vx", vx), ("vy", vy)):
                out[pre + key] = v
            out[pre + "diffuse_var"] = R.diffuse_var(f, d, rx, ry, xd, yd, wx, wy)
            out[pre + "advect"] = R.advect(f, d, xv, yv, xd, yd, wx, wy)
            out[pre + "advect_var"] = R.advect_var(f, d, vx, vy, xd, yd, wx, wy)
            # Dirichlet forms (Advection2<BCFn> and <BCFn, XVelBCFn, YVelBCFn>)
            g, gvx, gvy = (grng.random(2 * (xd + yd)) - 0.25 for _ in range(3))
            out[pre + "ghost"], out[pre + "ghost_vx"], out[pre + "ghost_vy"] = g, gvx, gvy
            out[pre + "advect_bc"] = R.advect(f, d, xv, yv, xd, yd, wx, wy, ghost=g)
            out[pre + "advect_var_bc"] = R.advect_var(f, d, vx, vy, xd, yd, wx, wy, g, gvx, gvy)
            k += 1
    out["count"] = np.array([k])
    return out


def agent_move_cases(rng):
    """SphericalAgent2D's update after its forces: SetVelocity(vel + delta),
    CapVelocity, ForceMove (MoveSafePT), ApplyFriction
    (include/Hal/Agents/SphericalAgent2D.h:133-162, AgentPT2D.h:157-186), run
    by the reference's own agent grid.  Agents start near the edges as well,
    so moves leave the grid on wrapped and closed axes."""
    out = {}
    cases = [(17, 29, 0, 0, 0.5, -1.0), (40, 9, 1, 1, 1.0, 0.8), (1, 7, 1, 0, 0.0, 2.0), (64, 64, 0, 1, 0.9, 0.0),
             (33, 5, 1, 1, 0.25, 1e9), (5, 33, 0, 0, 1.0, 1.5)]
    for k, (xd, yd, wx, wy, fr, mv) in enumerate(cases):
        n = 400
        pos = np.stack([rng.random(n) * xd, rng.random(n) * yd], 1)
        edge = rng.random(n) < 0.3  # a third start within one cell of an edge
        pos[edge, 0] = np.where(rng.random(edge.sum()) < 0.5, rng.random(edge.sum()),
                                xd - rng.random(edge.sum()))
        pos = np.minimum(pos, np.array([xd, yd]) * (1 - 1e-9)).ravel()
        vel = (rng.random(2 * n) - 0.5) * 2.0
        dv = (rng.random(2 * n) - 0.5) * 2.0
        pre = f"c{k}_"
        out[pre + "dims"] = np.array([xd, yd, wx, wy], dtype=np.int32)
        out[pre + "params"] = np.array([fr, mv])
        out[pre + "pos"], out[pre + "vel"], out[pre + "dv"] = pos, vel, dv
        out[pre + "pos_out"], out[pre + "vel_out"] = R.agents_move(pos, vel, dv, xd, yd, wx, wy, fr, mv)
    out["count"] = np.array([len(cases)])
    return out


def adv_tick_cases(rng):
    """PDEGrid2D ticks with Advection(xVel, yVel[, bc]) after the diffusion
    term (include/Hal/Grids/PDEGrid2D.h:351-375), decay and a dense source,
    run by the reference's own PDEGrid2D."""
    out = {}
    cases = [(40, 33, 0, 0, False, 0.2, 0.15, -0.2), (33, 40, 1, 1, False, 0.24, -0.3, 0.1),
             (48, 20, 0, 1, True, 0.1, 0.25, 0.25), (17, 64, 1, 0, True, 0.2, 0.0, -0.45)]
    for k, (xd, yd, wx, wy, bc, r, xv, yv) in enumerate(cases):
        f = rng.random(xd * yd)
        src = rng.random(xd * yd) * 0.01
        gh = rng.random(2 * (xd + yd)) if bc else None
        pre = f"c{k}_"
        out[pre + "dims"] = np.array([xd, yd, wx, wy, int(bc)], dtype=np.int32)
        out[pre + "params"] = np.array([r, xv, yv, 0.005])
        out[pre + "field"], out[pre + "src"] = f, src
        if bc:
            out[pre + "ghost"] = gh
        out[pre + "out"] = R.run_ticks(0, f, xd, yd, r, wx, wy, gh, decay=0.005, src_dense=src, ticks=6,
                                       xVel=xv, yVel=yv)
    out["count"] = np.array([len(cases)])
    return out


def sum_forces_cases(rng):
    """SphericalAgent2D::SumForces (include/Hal/Agents/SphericalAgent2D.h:
    74-102) on the reference's agent grid, agents created in index order, with
    the linear law, the clamped law of examples/OffLatticeExample.cpp:147-154
    and the power law of examples/Chemotaxis.cpp:128-130; starting velocities
    zero or random; walls, torus and mixed edges; coincident agents."""
    out = {}
    # the seed-1234 scene (tests/IAgentForceBackend2DTests.cpp:25-37), periodic
    u = R.rand_draws(1234, 0, 180)
    pos = np.empty(120)
    pos[0::2] = u[0::3] * 16.0
    pos[1::2] = u[1::3] * 16.0
    rad = 0.4 + u[2::3] * 0.4
    scenes = [("s1234", 16, 16, 1, 1, pos, rad)]
    for (name, xd, yd, n, wx, wy) in [("walls", 40, 30, 800, 0, 0), ("torus", 23, 31, 500, 1, 1),
                                      ("mixed", 30, 12, 400, 0, 1), ("dense", 6, 5, 250, 1, 0)]:
        m = int(n * 0.4)
        uni = rng.random((n - m, 2)) * np.array([xd, yd])
        clu = np.array([xd, yd]) * 0.5 + rng.normal(0.0, 1.5, (m, 2))
        p = np.concatenate([uni, clu])
        hi = np.array([np.nextafter(xd, 0), np.nextafter(yd, 0)])
        p = np.clip(p, 0.0, hi).ravel()
        p[2:4] = p[0:2]  # coincident agents: no direction, skipped
        scenes.append((name, xd, yd, wx, wy, p, 0.25 + 0.35 * rng.random(n)))
    laws = [(0, 0.4, 1.0), (1, 0.25, 1.0), (2, 0.7, 2.0)]
    k = 0
    for (name, xd, yd, wx, wy, p, r) in scenes:
        out[f"{name}_pos"] = p
        out[f"{name}_rad"] = r
        for (law, scale, expo) in laws:
            for R_ in (1.0, 2.2):
                with_vel = (k % 2 == 1)
                vel = (rng.random(p.size) - 0.5) * 0.4 if with_vel else None
                v, sums = R.sum_forces(p, r, R_, law, scale, xd, yd, wx, wy, vel=vel, exponent=expo)
                out[f"c{k}_scene"] = np.array([name.encode()])
                out[f"c{k}_params"] = np.array([xd, yd, wx, wy, R_, law, scale, expo])
                if vel is not None:
                    out[f"c{k}_velin"] = vel
                out[f"c{k}_vel"] = v
                out[f"c{k}_sums"] = sums
                k += 1
    out["count"] = np.array([k])
    return out


def pdegrid_script(rng, xd, yd, wx, wy, cells_per_tick=6):
    """A model-shaped call sequence on one PDEGrid2D: per-cell Set/Add/Mul/
    Scale (repeated cells included) between explicit, Dirichlet, per-cell
    rate and ADI diffusion and both advection forms, Update, the whole-grid
    operations, SetNonNegative and every query."""
    from pyoracle import PDEScript

    n, g = xd * yd, 2 * (xd + yd)
    sc = PDEScript(xd, yd, wx, wy)
    cells = lambda k: rng.integers(0, n, k)
    for tick in range(4):
        for c in cells(cells_per_tick):
            sc.add(["set", "add", "mul", "scale"][int(rng.integers(0, 4))], i=int(c), d0=float(rng.random() - 0.3))
        hot = int(cells(1)[0])
        for _ in range(3):  # one cell hit repeatedly: order matters
            sc.add("mul", i=hot, d0=-0.001).add("add", i=hot, d0=0.02)
        kind = tick % 4
        if kind == 0:
            sc.add("diffusion", d0=0.2).add("advection", d0=0.15, d1=-0.2)
        elif kind == 1:
            sc.add("adi", d0=float(0.5 + 4.5 * rng.random())).add("diffusion_bc", d0=0.1, arrays=[rng.random(g)])
        elif kind == 2:
            sc.add("adi_bc", d0=3.0, arrays=[rng.random(g)])
            sc.add("diffusion_var", arrays=[rng.random(n) * 0.2, rng.random(n) * 0.2])
            sc.add("advection_bc", d0=-0.1, d1=0.25, arrays=[rng.random(g)])
        else:
            sc.add("advection_var", arrays=[rng.random(n) - 0.5, rng.random(n) - 0.5])
            sc.add("advection_var_bc", arrays=[rng.random(n) - 0.5, rng.random(n) - 0.5, rng.random(g),
                                               rng.random(g) - 0.5, rng.random(g) - 0.5])
            sc.add("mul_all", d0=-0.01)
        sc.add("max_delta").add("max_delta_scaled", d0=1e-3)
        if tick == 2:
            sc.add("set_non_negative")
        sc.add("update")
        for c in cells(3):
            sc.add("get", i=int(c))
        sc.add("max").add("min").add("avg")
        x, y = int(rng.integers(0, xd)), int(rng.integers(0, yd))
        sc.add("gradient_x", x=x, y=y).add("gradient_y", x=x, y=y).add("gradient_x_bc", x=0, y=y, d0=1.0)
        sc.add("gradient_y_bc", x=x, y=yd - 1, d0=-0.5)
    sc.add("add_all", d0=0.01).add("set_all_values", arrays=[rng.random(n)]).add("set", i=0, d0=2.0)
    sc.add("set_all", d0=0.25).add("update").add("max").add("min")
    return sc


def pdegrid_script_cases(rng):
    """Hal::PDEGrid2D call sequences (include/Hal/Grids/PDEGrid2D.h) run on the
    reference's own grid: the final field, deltas and update count and every
    query result."""
    out = {}
    k = 0
    for (xd, yd, wx, wy) in [(23, 17, 0, 0), (16, 24, 1, 1), (31, 9, 1, 0), (9, 31, 0, 1), (1, 6, 0, 0),
                             (5, 1, 1, 0)]:
        sc = pdegrid_script(rng, xd, yd, wx, wy)
        f0 = rng.random(xd * yd)
        d0 = (rng.random(xd * yd) - 0.5) * 1e-3
        f, d, uc, rec = R.pdegrid_script(sc, f0, d0, 7)
        ops, iargs, dargs, arrays = sc.encoded()
        out[f"c{k}_dims"] = np.array([xd, yd, wx, wy], dtype=np.int32)
        out.update({f"c{k}_ops": ops, f"c{k}_iargs": iargs, f"c{k}_dargs": dargs, f"c{k}_arrays": arrays,
                    f"c{k}_f0": f0, f"c{k}_d0": d0, f"c{k}_field": f, f"c{k}_deltas": d,
                    f"c{k}_uc": np.array([uc], dtype=np.int32), f"c{k}_records": rec})
        k += 1
    out["count"] = np.array([k])
    return out


def pdegrid_file():
    """A PDEGrid2D file written by the reference's SavePDEGrid2D
    (src/Grids/PDEGridSerialization.cpp:34-45): 13 x 7, wrapX only, update
    count 42, a random field and pending deltas."""
    rng = np.random.default_rng(7171)
    f = rng.random(13 * 7)
    d = (rng.random(13 * 7) - 0.5) * 1e-3
    path = os.path.join(HERE, "pdegrid2d_13x7.bin")
    R.pdegrid2d_save(path, 13, 7, 1, 0, 42, f, d)
    return path


def main():
    pyoracle.build(ref=True)
    if not R.available():
        raise SystemExit("the reference library could not be built (no reference tree?)")
    only = sys.argv[1:]
    if only:
        # write only the named fixtures (each has its own seed)
        makers = {"sumforces": lambda: sum_forces_cases(np.random.default_rng(5353)),
                  "pdegrid": lambda: pdegrid_script_cases(np.random.default_rng(4242))}
        for name in only:
            np.savez_compressed(os.path.join(HERE, name + ".npz"), **makers[name]())
            print(os.path.join(HERE, name + ".npz"))
        return
    rng = np.random.default_rng(20261203)
    np.savez_compressed(os.path.join(HERE, "stencil.npz"), **stencil_cases(rng))
    np.savez_compressed(os.path.join(HERE, "ticks.npz"), **tick_cases(rng))
    np.savez_compressed(os.path.join(HERE, "agents.npz"), **agent_cases(rng))
    np.savez_compressed(os.path.join(HERE, "rand.npz"), **rand_cases())
    np.savez_compressed(os.path.join(HERE, "varstencil.npz"), **var_stencil_cases(np.random.default_rng(8181)))
    np.savez_compressed(os.path.join(HERE, "agentmove.npz"), **agent_move_cases(np.random.default_rng(9191)))
    np.savez_compressed(os.path.join(HERE, "advtick.npz"), **adv_tick_cases(np.random.default_rng(6262)))
    np.savez_compressed(os.path.join(HERE, "sumforces.npz"), **sum_forces_cases(np.random.default_rng(5353)))
    np.savez_compressed(os.path.join(HERE, "pdegrid.npz"), **pdegrid_script_cases(np.random.default_rng(4242)))
    print(pdegrid_file())
    for name in ("stencil", "ticks", "agents", "rand", "varstencil", "agentmove", "advtick", "sumforces",
                 "pdegrid"):
        p = os.path.join(HERE, name + ".npz")
        print(f"{p}: {os.path.getsize(p)} bytes")


if __name__ == "__main__":
    main()
