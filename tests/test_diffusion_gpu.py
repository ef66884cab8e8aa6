"""Explicit diffusion on the GPU against the oracle and the golden vectors.

Tolerances:
* the FP64 interface call (hal_cuda_diffuse) must be bit-identical to the
  reference CPU backend (same IEEE operations in the same order);
* the FP32 fused tick must stay within max|err| <= 1e-5 * max|f| of the FP64
  oracle, and rel-L2 <= 1e-6 on full-size runs.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

from conftest import max_rel, rel_l2

pytestmark = pytest.mark.gpu


def _eigen(nx, ny):
    x = np.arange(nx)[:, None]
    y = np.arange(ny)[None, :]
    return (np.sin(2.0 * math.pi * x / nx) * np.sin(2.0 * math.pi * y / ny)).ravel()


def test_diffuse_fp64_bit_exact_golden(hal, golden):
    g = golden("stencil")
    for k in range(int(g["count"][0])):
        xd, yd, wx, wy, use_bc = (int(v) for v in g[f"c{k}_dims"])
        r = float(g[f"c{k}_rates"][0])
        with hal.Diffusion(xd, yd) as d:
            if use_bc:
                out = d.diffuse_bc(g[f"c{k}_field"], g[f"c{k}_deltas"].copy(), r, wx, wy,
                                   g[f"c{k}_ghost"])
            else:
                out = d.diffuse(g[f"c{k}_field"], g[f"c{k}_deltas"].copy(), r, xd, yd, wx, wy)
        assert np.array_equal(out, g[f"c{k}_explicit"]), f"case {k}: {xd}x{yd} wrap {wx}{wy}"


def test_var_stencil_fp64_bit_exact_golden(hal, golden):
    """Per-cell rate diffusion and both upwind advection forms against the
    reference's vectors, bit for bit."""
    g = golden("varstencil")
    for k in range(int(g["count"][0])):
        xd, yd, wx, wy = (int(v) for v in g[f"c{k}_dims"])
        xv, yv = (float(v) for v in g[f"c{k}_vel"])
        f, d = g[f"c{k}_f"], g[f"c{k}_d"]
        tag = f"case {k}: {xd}x{yd} wrap {wx}{wy}"
        with hal.Diffusion(xd, yd) as h:
            assert np.array_equal(h.diffuse_var(f, d.copy(), g[f"c{k}_rx"], g[f"c{k}_ry"], wx, wy),
                                  g[f"c{k}_diffuse_var"]), tag
            assert np.array_equal(h.advect(f, d.copy(), xv, yv, wx, wy), g[f"c{k}_advect"]), tag
            assert np.array_equal(h.advect_var(f, d.copy(), g[f"c{k}_vx"], g[f"c{k}_vy"], wx, wy),
                                  g[f"c{k}_advect_var"]), tag
            gh = g[f"c{k}_ghost"]
            assert np.array_equal(h.advect(f, d.copy(), xv, yv, wx, wy, ghost=gh), g[f"c{k}_advect_bc"]), tag
            assert np.array_equal(h.advect_var(f, d.copy(), g[f"c{k}_vx"], g[f"c{k}_vy"], wx, wy, gh,
                                               g[f"c{k}_ghost_vx"], g[f"c{k}_ghost_vy"]),
                                  g[f"c{k}_advect_var_bc"]), tag


@pytest.mark.parametrize("xd,yd", [(300, 257), (1024, 1024), (1, 4099)])
def test_var_stencil_matches_oracle_large(hal, oracle, xd, yd):
    rng = np.random.default_rng(xd * 7 + yd)
    n = xd * yd
    f, d = rng.random(n), rng.random(n) * 0.1
    rx, ry = rng.random(n) * 0.24, rng.random(n) * 0.24
    vx, vy = rng.random(n) - 0.5, rng.random(n) - 0.5
    vy[::5] = 0.0
    for wx, wy in ((0, 0), (1, 1), (0, 1)):
        with hal.Diffusion(xd, yd) as h:
            assert np.array_equal(h.diffuse_var(f, d.copy(), rx, ry, wx, wy),
                                  oracle.diffuse_var(f, d, rx, ry, xd, yd, wx, wy))
            for xv, yv in ((0.2, -0.35), (-0.1, 0.0)):
                assert np.array_equal(h.advect(f, d.copy(), xv, yv, wx, wy),
                                      oracle.advect(f, d, xv, yv, xd, yd, wx, wy))
            assert np.array_equal(h.advect_var(f, d.copy(), vx, vy, wx, wy),
                                  oracle.advect_var(f, d, vx, vy, xd, yd, wx, wy))
            gh, gvx, gvy = (rng.random(2 * (xd + yd)) - 0.3 for _ in range(3))
            assert np.array_equal(h.advect(f, d.copy(), -0.15, 0.25, wx, wy, ghost=gh),
                                  oracle.advect(f, d, -0.15, 0.25, xd, yd, wx, wy, ghost=gh))
            assert np.array_equal(h.advect_var(f, d.copy(), vx, vy, wx, wy, gh, gvx, gvy),
                                  oracle.advect_var(f, d, vx, vy, xd, yd, wx, wy, gh, gvx, gvy))


def test_stencil64_profile_reuses_uploaded_arrays(hal, oracle):
    """The profiling launches run on the arrays of the last call and keep
    accumulating into its deltas."""
    n = 64
    rng = np.random.default_rng(3)
    f, vx, vy = rng.random(n * n), rng.random(n * n) - 0.5, rng.random(n * n) - 0.5
    with hal.Diffusion(n, n) as h:
        with pytest.raises(ValueError):
            h.stencil64_profile(hal.STENCIL_ADVECT_VAR, 2)
        h.advect_var(f, np.zeros(n * n), vx, vy, 0, 0)
        assert h.stencil64_profile(hal.STENCIL_ADVECT_VAR, 3) > 0.0
        with pytest.raises(ValueError):
            h.stencil64_profile(7, 1)


def test_var_stencil_rejects_bad_input(hal):
    with hal.Diffusion(8, 8) as h:
        z = np.zeros(64)
        with pytest.raises(ValueError):
            h.diffuse_var(z, z.copy(), np.zeros(63), z, 0, 0)
        with pytest.raises(ValueError):
            h.advect_var(z, z.copy(), z, np.zeros(65), 0, 0)
        with pytest.raises(ValueError):
            h.advect(z, z.copy(), 0.1, 0.1, 0, 0, ghost=np.zeros(31))


def test_advection_special_velocities(hal, oracle):
    """Zero of either sign and NaN velocities add no term; infinite ones
    propagate as in the reference (Advection2 validates nothing)."""
    xd, yd = 19, 23
    n = xd * yd
    rng = np.random.default_rng(17)
    f, d = rng.random(n), rng.random(n)
    vx, vy = rng.random(n) - 0.5, rng.random(n) - 0.5
    vx[::3], vy[::4], vx[1::5], vy[2::7] = 0.0, -0.0, np.nan, np.inf
    with hal.Diffusion(xd, yd) as h:
        for xv, yv in ((0.0, -0.0), (np.nan, 0.3), (-np.inf, -0.2), (1e-310, -1e-310)):
            a = h.advect(f, d.copy(), xv, yv, 1, 0)
            b = oracle.advect(f, d, xv, yv, xd, yd, 1, 0)
            assert np.array_equal(a, b, equal_nan=True), (xv, yv)
        a = h.advect_var(f, d.copy(), vx, vy, 0, 1)
        b = oracle.advect_var(f, d, vx, vy, xd, yd, 0, 1)
        assert np.array_equal(a.view(np.int64), b.view(np.int64))


def test_advection_tick_golden(hal, golden):
    """Resident FP32 ticks with uniform advection against PDEGrid2D ticks
    (Diffusion, Advection, MulAll, Add, Update) written by the reference."""
    g = golden("advtick")
    for k in range(int(g["count"][0])):
        xd, yd, wx, wy, bc = (int(v) for v in g[f"c{k}_dims"])
        r, xv, yv, decay = (float(v) for v in g[f"c{k}_params"])
        f32 = g[f"c{k}_field"].astype(np.float32)
        with hal.Diffusion(xd, yd) as d:
            d.set_field(f32)
            d.set_source(g[f"c{k}_src"].astype(np.float32))
            if bc:
                d.set_dirichlet(g[f"c{k}_ghost"].astype(np.float32))
            d.set_velocity(xv, yv)
            d.run_ticks(6, r, decay, wx, wy)
            out = d.get_field()
        # the golden run starts from the float64 field: allow its rounding
        assert max_rel(out, g[f"c{k}_out"]) <= 2e-6, k


def test_advection_tick_matches_oracle(hal, oracle):
    """500 ticks of diffusion plus advection at 256^2 (Dirichlet edges, 64
    point sources, decay) against the FP64 oracle from the same float32
    start; zero velocity reproduces the plain tick bit for bit."""
    from halcuda import workloads

    w = workloads.explicit_inputs(256, seed=5)
    f32 = w["field"].astype(np.float32)
    g32 = w["ghost"].astype(np.float32)
    for xv, yv in ((0.2, -0.15), (-0.3, 0.2), (0.0, 0.45)):
        # r = 0.1 keeps the centre weight 1 - 4r - |xVel| - |yVel| positive
        ref = oracle.run_ticks(0, f32.astype(np.float64), 256, 256, 0.1, ghost=g32.astype(np.float64), decay=0.001,
                               src_idx=w["src_idx"], src_val=w["src_val"], ticks=500, xVel=xv, yVel=yv)
        with hal.Diffusion(256, 256) as d:
            d.set_field(f32)
            d.set_dirichlet(g32)
            d.set_point_sources(w["src_idx"], w["src_val"])
            d.set_velocity(xv, yv)
            d.run_ticks(500, 0.1, 0.001)
            out = d.get_field()
        assert rel_l2(out, ref) <= 1e-5, (xv, yv)
    outs = []
    for vel in (None, (0.0, 0.0)):
        with hal.Diffusion(64, 48) as d:
            d.set_field(f32[:64 * 48])
            if vel is not None:
                d.set_velocity(*vel)
            d.run_ticks(20, 0.2, 0.01, True, False)
            outs.append(d.get_field())
    assert np.array_equal(outs[0], outs[1])
    with hal.Diffusion(8, 8) as d:
        with pytest.raises(ValueError):
            d.set_velocity(0.3, -0.3)


@pytest.mark.parametrize("xd,yd,wx,wy,bc,vel,ticks", [
    (256, 256, 0, 0, False, (0.0, 0.0), 40),
    (100, 60, 1, 0, True, (0.0, 0.0), 41),
    (37, 44, 0, 1, True, (0.15, -0.1), 20),
    (300, 516, 1, 1, False, (-0.2, 0.2), 33),
    (1, 128, 1, 0, False, (0.0, 0.0), 12),
    (70, 4, 0, 0, True, (0.1, 0.1), 18),
])
def test_two_tick_blocking_matches_oracle(hal, oracle, xd, yd, wx, wy, bc, vel, ticks):
    """Temporal blocking (two ticks per launch, TMA-staged halo tiles) on
    edge, wrapped, Dirichlet, ragged-tile and tiny grids, with a dense source,
    point sources (one cell twice), decay and advection, against the FP64
    oracle and the one-tick launches."""
    rng = np.random.default_rng(xd * 31 + yd)
    n = xd * yd
    f32 = rng.random(n).astype(np.float32)
    src = (rng.random(n) * 0.01).astype(np.float32)
    pts = rng.choice(n, min(n, 12), replace=False).astype(np.int32)
    pts = np.concatenate([pts, pts[:1]])
    pv = (0.02 + 0.03 * rng.random(len(pts))).astype(np.float32)
    ghost = rng.random(2 * (xd + yd)).astype(np.float32) if bc else None
    r = 0.1
    ref = oracle.run_ticks(0, f32.astype(np.float64), xd, yd, r, wx, wy,
                           None if ghost is None else ghost.astype(np.float64), decay=0.002,
                           src_dense=src.astype(np.float64), src_idx=pts, src_val=pv.astype(np.float64),
                           ticks=ticks, xVel=vel[0], yVel=vel[1])
    outs = []
    for mode in (2, 1):
        with hal.Diffusion(xd, yd) as d:
            d.set_blocking(mode)
            d.set_field(f32)
            d.set_source(src)
            d.set_point_sources(pts, pv)
            if ghost is not None:
                d.set_dirichlet(ghost)
            d.set_velocity(*vel)
            d.run_ticks(ticks, r, 0.002, wx, wy)
            outs.append(d.get_field())
    assert rel_l2(outs[0], ref) <= 1e-5 and max_rel(outs[0], ref) <= 1e-5
    assert max_rel(outs[0], outs[1]) <= 1e-5


def test_blocking_modes(hal):
    with hal.Diffusion(16, 30) as d:  # yDim % 4 != 0: no two-tick launches
        with pytest.raises(RuntimeError):
            d.set_blocking(2)
        d.set_blocking(1)
        with pytest.raises(ValueError):
            d.set_blocking(3)
    rng = np.random.default_rng(3)
    f = rng.random(64 * 64).astype(np.float32)
    outs = []
    for mode in (0, 1):  # automatic is one tick per launch
        with hal.Diffusion(64, 64) as d:
            d.set_blocking(mode)
            d.set_field(f)
            d.run_ticks(9, 0.2, 0.01)
            outs.append(d.get_field())
    assert np.array_equal(outs[0], outs[1])


def test_eigenmode_decay_through_interface(hal):
    """tests/IDiffusionBackend2DTests.cpp:23-72 (GPU epsilon 1e-4 there)."""
    nx, ny, r = 16, 20, 0.05
    f = _eigen(nx, ny)
    with hal.Diffusion(nx, ny) as d:
        out = d.diffuse(f, np.zeros_like(f), r, nx, ny, True, True)
    lam = 1.0 - 4.0 * r * (math.sin(math.pi / nx) ** 2 + math.sin(math.pi / ny) ** 2)
    np.testing.assert_allclose(f + out, lam * f, rtol=1e-12, atol=1e-12)


def test_size_mismatch_rejected(hal):
    """tests/IDiffusionBackend2DTests.cpp:146-177."""
    with hal.Diffusion(3, 4) as d:
        with pytest.raises(ValueError):
            d.diffuse(np.zeros(12), np.zeros(11), 0.1, 3, 4, False, False)
        with pytest.raises(ValueError):
            d.diffuse(np.zeros(12), np.zeros(12), 0.1, 4, 3, False, False)
        with pytest.raises(ValueError):
            d.run_steps(np.zeros(15, np.float32), 1, 0.1)
        with pytest.raises(ValueError):
            d.run_ticks(1, 0.26)


def test_run_steps_eigenmode_nth_power(hal):
    """DiffusionKernel2DTests.cpp:220-265: lambda^N after N steps, then 2N."""
    nx, ny, r, steps = 16, 20, 0.05, 50
    f = _eigen(nx, ny)
    lam = 1.0 - 4.0 * r * (math.sin(math.pi / nx) ** 2 + math.sin(math.pi / ny) ** 2)
    with hal.Diffusion(nx, ny) as d:
        out = d.run_steps(f, steps, r, True, True)
        np.testing.assert_allclose(out, lam ** steps * f, rtol=0, atol=1e-5)
        out2 = d.run_steps(out, steps, r, True, True)
        np.testing.assert_allclose(out2, lam ** (2 * steps) * f, rtol=0, atol=1e-5)


def test_fused_tick_golden(hal, golden):
    """PDEGrid2D tick (Dirichlet edge, decay, point sources), 150 ticks."""
    g = golden("ticks")
    xd, yd, r, decay, ticks = g["exp_params"]
    xd, yd, ticks = int(xd), int(yd), int(ticks)
    with hal.Diffusion(xd, yd) as d:
        d.set_field(g["exp_field"])
        d.set_dirichlet(g["exp_ghost"])
        d.set_point_sources(g["exp_src_idx"], g["exp_src_val"])
        d.run_ticks(ticks, r, decay)
        out = d.get_field()
    assert max_rel(out, g["exp_out"]) <= 1e-5


SIZES = [(1, 1), (1, 9), (9, 1), (2, 2), (5, 7), (8, 12), (33, 64), (64, 33), (70, 130),
         (129, 257)]


@pytest.mark.parametrize("xd,yd", SIZES)
def test_fused_tick_matches_oracle_all_boundaries(hal, oracle, xd, yd):
    rng = np.random.default_rng(xd * 1000 + yd)
    f = rng.random(xd * yd)
    src = rng.random(xd * yd) * 0.01
    pts = rng.choice(xd * yd, min(5, xd * yd), replace=False).astype(np.int32)
    vals = rng.random(pts.size) * 0.1
    ghost = rng.random(2 * (xd + yd))
    for wx in (False, True):
        for wy in (False, True):
            for gh in (None, ghost):
                exp = oracle.run_ticks(0, f, xd, yd, 0.21, wx, wy, gh, 0.003, src, pts, vals, ticks=6)
                with hal.Diffusion(xd, yd) as d:
                    d.set_field(f)
                    d.set_source(src)
                    d.set_point_sources(pts, vals)
                    d.set_dirichlet(gh)
                    d.run_ticks(6, 0.21, 0.003, wx, wy)
                    out = d.get_field()
                assert max_rel(out, exp) <= 1e-5, (wx, wy, gh is None)


def test_graph_replay_and_parity_of_buffers(hal, oracle):
    """Odd and even tick counts, repeated calls (graph cache per buffer parity)."""
    rng = np.random.default_rng(3)
    f = rng.random(40 * 52)
    exp = oracle.run_ticks(0, f, 40, 52, 0.2, ticks=3 + 4 + 3 + 3)
    with hal.Diffusion(40, 52) as d:
        d.set_field(f)
        for t in (3, 4, 3, 3):
            d.run_ticks(t, 0.2)
        out = d.get_field()
    assert max_rel(out, exp) <= 1e-5


def test_explicit_256_config_1000_ticks(hal, oracle):
    """The 256x256 FP64 workload shape: Dirichlet 1.0 on the left edge, decay
    0.001, 64 point sources of 0.05, 1000 ticks -- FP32 on the GPU vs FP64."""
    from halcuda import workloads

    w = workloads.explicit_inputs(256, seed=1)
    exp = oracle.run_ticks(0, w["field"], 256, 256, w["diffRate"], ghost=w["ghost"],
                           decay=w["decay"], src_idx=w["src_idx"], src_val=w["src_val"],
                           ticks=1000, threads=8)
    with hal.Diffusion(256, 256) as d:
        d.set_field(w["field"])
        d.set_dirichlet(w["ghost"])
        d.set_point_sources(w["src_idx"], w["src_val"])
        d.run_ticks(1000, w["diffRate"], w["decay"])
        out = d.get_field()
    assert rel_l2(out, exp) <= 1e-5
    assert max_rel(out, exp) <= 2e-5


def test_explicit_2048_full_size(hal, oracle):
    from halcuda import workloads

    w = workloads.explicit_inputs(2048, seed=1)
    exp = oracle.run_ticks(0, w["field"], 2048, 2048, 0.2, decay=0.001, src_idx=w["src_idx"],
                           src_val=w["src_val"], ticks=10, threads=16)
    with hal.Diffusion(2048, 2048) as d:
        d.set_field(w["field"])
        d.set_point_sources(w["src_idx"], w["src_val"])
        d.run_ticks(10, 0.2, 0.001)
        out = d.get_field()
    assert rel_l2(out, exp) <= 1e-6
    assert max_rel(out, exp) <= 1e-5


@pytest.mark.parametrize("xd,yd,wrapX,wrapY,dirichlet,vel", [
    (300, 256, False, False, False, None),   # float4 strips, interior fast path
    (257, 130, True, False, True, None),     # scalar strips, wrapped x, Dirichlet
    (128, 200, False, True, False, (0.1, -0.2)),  # advective tick
])
def test_explicit_tick_uptake_against_oracle(hal, oracle, xd, yd, wrapX, wrapY, dirichlet, vel):
    """Agent uptake on the explicit tick: every agent of the agent handle's
    last binning multiplies its cell by -uptake each tick (a model's
    PDEGrid2D::Mul(cell, -uptake) per agent), with decay, a dense source,
    point sources and every boundary kind, against the FP64 oracle tick with
    the same per-cell counts.  Removing the coupling gives the plain tick."""
    rng = np.random.default_rng(xd * 7 + yd)
    n = xd * yd
    f0 = rng.random(n).astype(np.float32)
    src = (rng.random(n) * 1e-3).astype(np.float32)
    ghost = rng.random(2 * (xd + yd)).astype(np.float32) if dirichlet else None
    pidx = rng.choice(n, 40, replace=False).astype(np.int32)
    pval = (rng.random(40) * 0.05).astype(np.float32)
    r, decay, uptake, ticks = 0.2, 1e-3, 4e-3, 25
    nAgents = 3 * n // 2
    pos = np.empty(2 * nAgents, np.float32)
    pos[0::2] = rng.random(nAgents) * xd
    pos[1::2] = np.clip(yd * 0.5 + rng.normal(0.0, yd * 0.15, nAgents), 0, yd - 1e-3)
    with hal.Agents(xd, yd, nAgents) as ag, hal.Diffusion(xd, yd) as d:
        ag.upload(pos, np.full(nAgents, 0.5, np.float32))
        ag.dispatch(1.0, 0.1)
        ag.sync()
        off, _ = ag.get_bins()
        counts = np.diff(off).astype(np.int32)
        assert counts.sum() == nAgents and counts.max() >= 3
        d.set_field(f0)
        d.set_source(src)
        d.set_point_sources(pidx, pval)
        if ghost is not None:
            d.set_dirichlet(ghost)
        if vel is not None:
            d.set_velocity(*vel)
        d.set_uptake(ag, uptake)
        d.run_ticks(ticks, r, decay, wrapX, wrapY)
        out = d.get_field()
        d.set_uptake(None, 0.0)
        d.set_field(f0)
        d.run_ticks(ticks, r, decay, wrapX, wrapY)
        plain = d.get_field()
    g64 = None if ghost is None else ghost.astype(np.float64)
    vx, vy = vel if vel is not None else (0.0, 0.0)
    exp = oracle.run_ticks(0, f0.astype(np.float64), xd, yd, r, wrapX, wrapY, g64, decay,
                           src_dense=src.astype(np.float64), src_idx=pidx, src_val=pval.astype(np.float64),
                           uptake_count=counts, uptake=uptake, ticks=ticks, xVel=vx, yVel=vy)
    exp_plain = oracle.run_ticks(0, f0.astype(np.float64), xd, yd, r, wrapX, wrapY, g64, decay,
                                 src_dense=src.astype(np.float64), src_idx=pidx, src_val=pval.astype(np.float64),
                                 ticks=ticks, xVel=vx, yVel=vy)
    assert max_rel(exp, exp_plain) > 1e-3  # the coupling changes the field
    assert max_rel(out, exp) <= 1e-5, max_rel(out, exp)
    assert max_rel(plain, exp_plain) <= 1e-5, max_rel(plain, exp_plain)


def test_explicit_uptake_rejects_other_grid(hal):
    with hal.Agents(32, 16, 10) as ag, hal.Diffusion(16, 32) as d:
        with pytest.raises(ValueError, match="differs"):
            d.set_uptake(ag, 1e-3)
