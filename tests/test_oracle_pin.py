"""Pins the CPU oracle (oracle/hal_oracle.c) to the reference.

CPU only.  Every golden vector in tests/golden/ was written from the
reference's own CPU code (tests/golden/make_golden.py); the restatement must
reproduce each FP64 result bit for bit.  The reference's known-answer tests
(tests/IDiffusionBackend2DTests.cpp, PDEADITests.cpp,
IAgentForceBackend2DTests.cpp) are restated against the oracle as well.  When
the reference tree is present, the restatement is also compared with the
freshly built reference library on new random cases.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

import pyoracle


def _eigen(nx, ny):
    x = np.arange(nx)[:, None]
    y = np.arange(ny)[None, :]
    return (np.sin(2.0 * math.pi * x / nx) * np.sin(2.0 * math.pi * y / ny)).ravel()


def test_stencil_and_adi_golden_bit_exact(oracle, golden):
    g = golden("stencil")
    count = int(g["count"][0])
    assert count >= 60
    for k in range(count):
        xd, yd, wx, wy, use_bc = (int(v) for v in g[f"c{k}_dims"])
        r_exp, r_adi = (float(v) for v in g[f"c{k}_rates"])
        f = g[f"c{k}_field"]
        d = g[f"c{k}_deltas"]
        gh = g[f"c{k}_ghost"] if use_bc else None
        out = oracle.diffuse(f, d, r_exp, xd, yd, wx, wy, gh)
        assert np.array_equal(out, g[f"c{k}_explicit"]), f"explicit case {k} {xd}x{yd}"
        out = oracle.diffuse_adi(f, d, r_adi, xd, yd, wx, wy, gh)
        assert np.array_equal(out, g[f"c{k}_adi"]), f"ADI case {k} {xd}x{yd} wrap {wx}{wy} bc {use_bc}"


def test_var_stencil_golden_bit_exact(oracle, golden):
    """Per-cell rate diffusion and both upwind advection forms
    (Internal::Diffusion2 / Advection2, src/Pde/PDEequations.cpp:199-230,
    380-412, 535-575), and the advection forms' Dirichlet variants
    (include/Hal/Pde/PDEequations.h:413-447, 720-778), against vectors
    written by the reference."""
    g = golden("varstencil")
    count = int(g["count"][0])
    assert count == 32
    for k in range(count):
        xd, yd, wx, wy = (int(v) for v in g[f"c{k}_dims"])
        xv, yv = (float(v) for v in g[f"c{k}_vel"])
        f, d = g[f"c{k}_f"], g[f"c{k}_d"]
        tag = f"case {k} {xd}x{yd} wrap {wx}{wy}"
        assert np.array_equal(oracle.diffuse_var(f, d, g[f"c{k}_rx"], g[f"c{k}_ry"], xd, yd, wx, wy),
                              g[f"c{k}_diffuse_var"]), tag
        assert np.array_equal(oracle.advect(f, d, xv, yv, xd, yd, wx, wy), g[f"c{k}_advect"]), tag
        assert np.array_equal(oracle.advect_var(f, d, g[f"c{k}_vx"], g[f"c{k}_vy"], xd, yd, wx, wy),
                              g[f"c{k}_advect_var"]), tag
        gh = g[f"c{k}_ghost"]
        assert np.array_equal(oracle.advect(f, d, xv, yv, xd, yd, wx, wy, ghost=gh), g[f"c{k}_advect_bc"]), tag
        assert np.array_equal(oracle.advect_var(f, d, g[f"c{k}_vx"], g[f"c{k}_vy"], xd, yd, wx, wy, gh,
                                                g[f"c{k}_ghost_vx"], g[f"c{k}_ghost_vy"]),
                              g[f"c{k}_advect_var_bc"]), tag


def test_var_stencil_conservation_kat(oracle):
    """Known answers: with both axes wrapped, every face flux leaves one cell
    and enters its neighbour, so the sums of the per-cell rate diffusion and
    of both advection forms vanish; a uniform field does not diffuse."""
    rng = np.random.default_rng(5)
    xd, yd = 24, 17
    n = xd * yd
    f = rng.random(n)
    z = np.zeros(n)
    rx, ry = rng.random(n) * 0.2, rng.random(n) * 0.2
    vx, vy = rng.random(n) - 0.5, rng.random(n) - 0.5
    for out in (oracle.diffuse_var(f, z, rx, ry, xd, yd, 1, 1), oracle.advect(f, z, 0.3, -0.2, xd, yd, 1, 1),
                oracle.advect_var(f, z, vx, vy, xd, yd, 1, 1)):
        assert abs(out.sum()) <= 1e-12 * n
    assert not oracle.diffuse_var(np.full(n, 2.5), z, rx, ry, xd, yd, 0, 0).any()


def test_advection_tick_golden_bit_exact(oracle, golden):
    """PDEGrid2D ticks with Advection(xVel, yVel[, bc]) after the diffusion
    term, against the reference's own PDEGrid2D, bit for bit."""
    g = golden("advtick")
    for k in range(int(g["count"][0])):
        xd, yd, wx, wy, bc = (int(v) for v in g[f"c{k}_dims"])
        r, xv, yv, decay = (float(v) for v in g[f"c{k}_params"])
        out = oracle.run_ticks(0, g[f"c{k}_field"], xd, yd, r, wx, wy, g[f"c{k}_ghost"] if bc else None,
                               decay=decay, src_dense=g[f"c{k}_src"], ticks=6, xVel=xv, yVel=yv)
        assert np.array_equal(out, g[f"c{k}_out"]), k
    with pytest.raises(ValueError):  # CheckAdvectionStable
        oracle.run_ticks(0, np.zeros(4), 2, 2, 0.1, xVel=0.3, yVel=-0.3)


def test_agent_move_golden_bit_exact(oracle, golden):
    """SphericalAgent2D's update after its forces (SetVelocity, CapVelocity,
    ForceMove -> MoveSafePT, ApplyFriction) against the reference's agent
    grid, bit for bit."""
    g = golden("agentmove")
    for k in range(int(g["count"][0])):
        xd, yd, wx, wy = (int(v) for v in g[f"c{k}_dims"])
        fr, mv = (float(v) for v in g[f"c{k}_params"])
        p, v = oracle.agents_move(g[f"c{k}_pos"], g[f"c{k}_vel"], g[f"c{k}_dv"], xd, yd, wx, wy, fr, mv)
        assert np.array_equal(p, g[f"c{k}_pos_out"]), k
        assert np.array_equal(v, g[f"c{k}_vel_out"]), k


def test_agent_move_kat(oracle):
    """The reference's own checks (tests/SphericalAgentTests.cpp:88-103):
    ApplyFriction(0.5) halves (3, 4); CapVelocity(2) brings |(3, 4)| to 2.
    And MoveSafePT: leaving a closed edge keeps the coordinate, leaving a
    wrapped edge wraps it."""
    z = np.zeros(2)
    _, v = oracle.agents_move([5.0, 5.0], [3.0, 4.0], z, 100, 100, 0, 0, 0.5, -1.0)
    assert np.allclose(v, [1.5, 2.0])
    _, v = oracle.agents_move([5.0, 5.0], [3.0, 4.0], z, 100, 100, 0, 0, 1.0, 2.0)
    assert abs(math.hypot(*v) - 2.0) < 1e-12
    p, _ = oracle.agents_move([9.5, 5.0], [1.0, 0.25], z, 10, 10, 0, 0, 1.0, -1.0)
    assert np.array_equal(p, [9.5, 5.25])
    p, _ = oracle.agents_move([9.5, 5.0], [1.0, 0.25], z, 10, 10, 1, 0, 1.0, -1.0)
    assert np.array_equal(p, [0.5, 5.25])
    p, _ = oracle.agents_move([0.25, 0.5], [-0.5, -1.0], z, 10, 10, 1, 1, 1.0, -1.0)
    assert np.array_equal(p, [9.75, 9.5])
    for f32 in (False, True):
        p, v = oracle.agents_move([2.0, 3.0], [0.5, -0.5], [0.25, 0.25], 10, 10, 0, 0, 0.0, -1.0, f32=f32)
        assert np.array_equal(p, [2.75, 2.75]) and not v.any()


def test_agent_move_f32_tracks_f64(oracle):
    """The FP32 form takes the same branches as the FP64 one away from the
    edges and agrees to float rounding."""
    rng = np.random.default_rng(2)
    n, xd, yd = 5000, 128, 96
    pos = np.stack([4 + rng.random(n) * (xd - 8), 4 + rng.random(n) * (yd - 8)], 1).ravel()
    pos = pos.astype(np.float32).astype(np.float64)
    vel = ((rng.random(2 * n) - 0.5) * 2).astype(np.float32).astype(np.float64)
    dv = ((rng.random(2 * n) - 0.5) * 2).astype(np.float32).astype(np.float64)
    p64, v64 = oracle.agents_move(pos, vel, dv, xd, yd, 1, 0, 0.8, 1.2)
    p32, v32 = oracle.agents_move(pos, vel, dv, xd, yd, 1, 0, 0.8, 1.2, f32=True)
    assert np.max(np.abs(p32 - p64)) <= 2e-5
    assert np.max(np.abs(v32 - v64)) <= 2e-6


def test_tick_golden_bit_exact(oracle, golden):
    g = golden("ticks")
    xd, yd, r, decay, ticks = g["exp_params"]
    out = oracle.run_ticks(0, g["exp_field"], int(xd), int(yd), r, ghost=g["exp_ghost"],
                           decay=decay, src_idx=g["exp_src_idx"], src_val=g["exp_src_val"],
                           ticks=int(ticks))
    assert np.array_equal(out, g["exp_out"])
    xd, yd, r, decay, ticks = g["adi_params"]
    out = oracle.run_ticks(1, g["adi_field"], int(xd), int(yd), r, decay=decay,
                           src_dense=g["adi_src"], ticks=int(ticks))
    assert np.array_equal(out, g["adi_out"])
    xd, yd, r, decay, uptake, ticks = g["cpl_params"]
    out = oracle.run_ticks(1, g["cpl_field"], int(xd), int(yd), r, wrapX=True,
                           ghost=g["cpl_ghost"], decay=decay, uptake_count=g["cpl_counts"],
                           uptake=uptake, ticks=int(ticks))
    assert np.array_equal(out, g["cpl_out"])
    out = oracle.run_ticks(1, g["kat_adi_field"], 20, 14, 0.6, ticks=5)
    assert np.array_equal(out, g["kat_adi_out"])


def test_agents_golden_bit_exact(oracle, golden):
    g = golden("agents")
    v, off, b = oracle.accumulate_forces(g["s1234_pos"], g["s1234_rad"], 3.0, 0.4, 16, 16, 1, 1)
    assert np.array_equal(v, g["s1234_vel"])
    assert np.array_equal(off, g["s1234_off"])
    assert np.array_equal(b, g["s1234_bucket"])
    for name in ("walls", "torus", "mixed", "tiny", "empty"):
        xd, yd, n, wx, wy, R, k = g[f"{name}_params"]
        v, off, b = oracle.accumulate_forces(g[f"{name}_pos"], g[f"{name}_rad"], R, k, int(xd),
                                             int(yd), int(wx), int(wy))
        assert np.array_equal(v, g[f"{name}_vel"]), name
        assert np.array_equal(off, g[f"{name}_off"]), name
        assert np.array_equal(b, g[f"{name}_bucket"]), name
    v, _, _ = oracle.accumulate_forces([4.0, 4.0, 4.0, 4.0], [0.5, 0.5], 2.0, 1.0, 8, 8, 0, 0)
    assert np.array_equal(v, g["coincident_vel"])
    assert np.all(v == 0.0)


def test_rand_golden_bit_exact(oracle, golden):
    g = golden("rand")
    for seed in (1, 7, 1234):
        assert np.array_equal(oracle.rand_draws(seed, 0, 64), g[f"double_{seed}"])
        assert np.array_equal(oracle.rand_draws(seed, 1, 64, 256), g[f"int256_{seed}"])
        # log() may differ by an ulp between C libraries
        assert np.allclose(oracle.rand_draws(seed, 2, 64), g[f"gauss_{seed}"], rtol=1e-14,
                           atol=0)


# --- the reference's known-answer tests, restated against the oracle ------

def test_eigenmode_explicit_kat(oracle):
    """tests/IDiffusionBackend2DTests.cpp:23-54 (epsilon 1e-4 there)."""
    nx, ny, r = 16, 20, 0.05
    f = _eigen(nx, ny)
    d = oracle.diffuse(f, np.zeros_like(f), r, nx, ny, True, True)
    lam = 1.0 - 4.0 * r * (math.sin(math.pi / nx) ** 2 + math.sin(math.pi / ny) ** 2)
    np.testing.assert_allclose(f + d, lam * f, rtol=1e-12, atol=1e-12)


def _lambda_cn(r, n, k=1):
    s = math.sin(math.pi * k / n) ** 2
    return (1.0 - 2.0 * r * s) / (1.0 + 2.0 * r * s)


def test_eigenmode_adi_kat(oracle):
    """tests/IDiffusionBackend2DTests.cpp:76-113 (CPU epsilon 1e-7)."""
    nx, ny, r = 12, 18, 0.3
    f = _eigen(nx, ny)
    d = oracle.diffuse_adi(f, np.zeros_like(f), r, nx, ny, True, True)
    lam = _lambda_cn(r, nx) * _lambda_cn(r, ny)
    np.testing.assert_allclose(f + d, lam * f, rtol=1e-7, atol=1e-12)


def test_adi_dirichlet_fixed_point_kat(oracle):
    """PDEADITests.cpp:219-235: a flat field equal to the Dirichlet value stays put."""
    xd, yd = 7, 5
    f = np.full(xd * yd, 4.0)
    ghost = np.full(2 * (xd + yd), 4.0)
    out = oracle.run_ticks(1, f, xd, yd, 0.9, ghost=ghost)
    np.testing.assert_allclose(out, 4.0, rtol=1e-12)


def test_adi_dirichlet_relaxes_kat(oracle):
    """PDEADITests.cpp:255-268: periodic x, Dirichlet 2.0, 400 steps -> 2.0."""
    xd, yd = 8, 6
    ghost = np.full(2 * (xd + yd), 2.0)
    out = oracle.run_ticks(1, np.zeros(xd * yd), xd, yd, 1.5, wrapX=True, ghost=ghost, ticks=400)
    np.testing.assert_allclose(out, 2.0, rtol=1e-6)


def test_adi_dirichlet_ramp_kat(oracle):
    """PDEADITests.cpp:287-352: the linear steady state between 1 and 3 holds."""
    xd, yd = 6, 4

    def ramp(x):
        return 1.0 if x < 0 else (3.0 if x >= xd else 1.0 + 2.0 * (x + 0.5) / xd)

    f = np.array([ramp(i // yd) for i in range(xd * yd)])
    ghost = np.concatenate([np.full(yd, 1.0), np.full(yd, 3.0),
                            np.array([ramp(x) for x in range(xd)]),
                            np.array([ramp(x) for x in range(xd)])])
    out = oracle.run_ticks(1, f, xd, yd, 0.9, ghost=ghost)
    np.testing.assert_allclose(out, f, rtol=1e-9)


def test_explicit_mass_conservation_kat(oracle):
    """PDEGridTests.cpp:72-104 (2D form): zero-flux and periodic keep the total."""
    rng = np.random.default_rng(5)
    for wrap in (False, True):
        f = rng.random(13 * 11)
        out = oracle.run_ticks(0, f, 13, 11, 0.24, wrapX=wrap, wrapY=wrap, ticks=20)
        assert abs(out.sum() - f.sum()) < 1e-10 * f.sum()


def test_explicit_rate_cap(oracle):
    """PDEGrid2D::CheckDiffusionStable (PDEGrid2D.h:436-442)."""
    with pytest.raises(ValueError):
        oracle.run_ticks(0, np.zeros(25), 5, 5, 0.26)
    oracle.run_ticks(0, np.zeros(25), 5, 5, 0.25)


def test_bruteforce_forces_kat(oracle, golden):
    """tests/IAgentForceBackend2DTests.cpp:55-107: cell buckets equal an
    all-pairs sum (CPU epsilon 1e-12)."""
    g = golden("agents")
    pos, rad = g["s1234_pos"], g["s1234_rad"]
    n = rad.size
    exp = np.zeros(2 * n)
    for i in range(n):
        for j in range(n):
            if i == j:
                continue
            dx = pos[2 * j] - pos[2 * i]
            dy = pos[2 * j + 1] - pos[2 * i + 1]
            if abs(dx) > 8:
                dx = dx + 16 if pos[2 * i] > pos[2 * j] else dx - 16
            if abs(dy) > 8:
                dy = dy + 16 if pos[2 * i + 1] > pos[2 * j + 1] else dy - 16
            dist = math.sqrt(dx * dx + dy * dy)
            if 0 < dist < 3.0:
                force = 0.4 * ((rad[i] + rad[j]) - dist)
                exp[2 * i] -= dx / dist * force
                exp[2 * i + 1] -= dy / dist * force
    v, _, _ = oracle.accumulate_forces(pos, rad, 3.0, 0.4, 16, 16, 1, 1)
    np.testing.assert_allclose(v, exp, rtol=1e-12, atol=1e-12)


def test_forces_size_mismatch(oracle):
    """IAgentForceBackend2DTests.cpp:144-151."""
    with pytest.raises(ValueError):
        oracle.accumulate_forces([1.0, 1.0, 2.0], [0.5, 0.5], 2.0, 1.0, 8, 8, 0, 0)


def test_threaded_oracle_matches_serial(oracle):
    rng = np.random.default_rng(11)
    f = rng.random(70 * 90)
    a = oracle.diffuse_adi(f, np.zeros_like(f), 5.0, 70, 90, False, True, threads=1)
    b = oracle.diffuse_adi(f, np.zeros_like(f), 5.0, 70, 90, False, True, threads=4)
    assert np.array_equal(a, b)
    pos = (rng.random(4000) * 50).astype(np.float32).astype(np.float64)
    rad = np.full(2000, 0.5)
    a = oracle.accumulate_forces(pos, rad, 1.0, 0.1, 50, 50, 0, 0, threads=1)
    b = oracle.accumulate_forces(pos, rad, 1.0, 0.1, 50, 50, 0, 0, threads=3)
    assert all(np.array_equal(x, y) for x, y in zip(a, b))


@pytest.mark.skipif(not pyoracle.Reference.available() and not __import__("os").path.isdir(
    pyoracle.REF_TREE), reason="reference tree not present")
def test_restatement_matches_reference_library_random(oracle):
    """Fresh random cases through the reference's own compiled CPU code."""
    pyoracle.build(ref=True)
    R = pyoracle.Reference
    rng = np.random.default_rng(99)
    for _ in range(6):
        xd, yd = (int(v) for v in rng.integers(1, 40, 2))
        wx, wy = (bool(v) for v in rng.integers(0, 2, 2))
        f = rng.random(xd * yd)
        d = rng.random(xd * yd)
        gh = rng.random(2 * (xd + yd)) if rng.random() < 0.5 else None
        r = float(rng.random() * 8)
        assert np.array_equal(oracle.diffuse(f, d, 0.2, xd, yd, wx, wy, gh),
                              R.diffuse(f, d, 0.2, xd, yd, wx, wy, gh))
        assert np.array_equal(oracle.diffuse_adi(f, d, r, xd, yd, wx, wy, gh),
                              R.diffuse_adi(f, d, r, xd, yd, wx, wy, gh))
        rx, ry = rng.random(xd * yd) * 0.2, rng.random(xd * yd) * 0.2
        vx, vy = rng.random(xd * yd) - 0.5, rng.random(xd * yd) - 0.5
        assert np.array_equal(oracle.diffuse_var(f, d, rx, ry, xd, yd, wx, wy),
                              R.diffuse_var(f, d, rx, ry, xd, yd, wx, wy))
        assert np.array_equal(oracle.advect(f, d, 0.25, -0.125, xd, yd, wx, wy),
                              R.advect(f, d, 0.25, -0.125, xd, yd, wx, wy))
        assert np.array_equal(oracle.advect_var(f, d, vx, vy, xd, yd, wx, wy),
                              R.advect_var(f, d, vx, vy, xd, yd, wx, wy))
        m = 50
        mpos = np.stack([rng.random(m) * xd, rng.random(m) * yd], 1).ravel() * (1 - 1e-9)
        mvel, mdv = rng.random(2 * m) - 0.5, (rng.random(2 * m) - 0.5) * 3
        a = oracle.agents_move(mpos, mvel, mdv, xd, yd, wx, wy, 0.7, 1.1)
        b = R.agents_move(mpos, mvel, mdv, xd, yd, wx, wy, 0.7, 1.1)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
        n = int(rng.integers(0, 300))
        pos = (rng.random(2 * n) * max(xd, yd)).astype(np.float32).astype(np.float64)
        rad = 0.3 + rng.random(n) * 0.5
        a = oracle.accumulate_forces(pos, rad, 1.7, 0.2, xd, yd, wx, wy)
        b = R.accumulate_forces(pos, rad, 1.7, 0.2, xd, yd, wx, wy)
        assert all(np.array_equal(x, y) for x, y in zip(a, b))


def _sumforces_case(g, k):
    """Inputs and outputs of golden SumForces case k."""
    xd, yd, wx, wy, R_, law, scale, expo = (float(v) for v in g[f"c{k}_params"])
    scene = g[f"c{k}_scene"][0].decode()
    vin = g[f"c{k}_velin"] if f"c{k}_velin" in g.files else None
    return dict(pos=g[f"{scene}_pos"], rad=g[f"{scene}_rad"], xd=int(xd), yd=int(yd), wx=int(wx), wy=int(wy),
                R=R_, law=int(law), scale=scale, expo=expo, vin=vin, vel=g[f"c{k}_vel"], sums=g[f"c{k}_sums"],
                tag=f"case {k} {scene} law {int(law)} R {R_}")


def test_sum_forces_golden_bit_exact(oracle, golden):
    """SphericalAgent2D::SumForces (include/Hal/Agents/SphericalAgent2D.h:
    74-102) on the reference's agent grid, for the linear, clamped and power
    laws, with and without starting velocities: the restatement's agent-grid
    order reproduces the velocities and the returned sums bit for bit."""
    g = golden("sumforces")
    count = int(g["count"][0])
    assert count == 30
    laws = set()
    for k in range(count):
        c = _sumforces_case(g, k)
        v, sums = oracle.sum_forces(c["pos"], c["rad"], c["R"], c["law"], c["scale"], c["xd"], c["yd"], c["wx"],
                                    c["wy"], vel=c["vin"], exponent=c["expo"], order=1)
        assert np.array_equal(v, c["vel"]), c["tag"]
        assert np.array_equal(sums, c["sums"]), c["tag"]
        laws.add(c["law"])
        # the clamped law never counts a separated pair, so its sums differ
        # from the linear law's only through overlapping pairs
        assert (c["sums"] >= 0).all()
    assert laws == {0, 1, 2}


def test_sum_forces_backend_order_is_accumulate_forces(oracle):
    """With the backend's order and the linear law from zero velocity,
    SumForces is exactly AccumulateForces (the interface's own definition,
    IAgentForceBackend2D.h:14)."""
    rng = np.random.default_rng(31)
    for (xd, yd, wx, wy) in [(20, 14, 0, 0), (13, 17, 1, 1)]:
        n = 500
        pos = np.stack([rng.random(n) * xd, rng.random(n) * yd], 1).ravel()
        rad = 0.3 + 0.4 * rng.random(n)
        v, _ = oracle.sum_forces(pos, rad, 2.0, 0, 0.3, xd, yd, wx, wy, order=0)
        exp, _, _ = oracle.accumulate_forces(pos, rad, 2.0, 0.3, xd, yd, wx, wy)
        assert np.array_equal(v, exp)


@pytest.mark.skipif(not pyoracle.Reference.available() and not __import__("os").path.isdir(
    pyoracle.REF_TREE), reason="reference tree not present")
def test_sum_forces_matches_reference_library_random(oracle):
    pyoracle.build(ref=True)
    R = pyoracle.Reference
    rng = np.random.default_rng(77)
    for _ in range(6):
        xd, yd = (int(v) for v in rng.integers(1, 30, 2))
        wx, wy = (int(v) for v in rng.integers(0, 2, 2))
        n = int(rng.integers(0, 400))
        pos = np.stack([rng.random(n) * xd, rng.random(n) * yd], 1).ravel() * (1 - 1e-12)
        rad = 0.2 + rng.random(n) * 0.6
        vel = rng.random(2 * n) - 0.5
        for law, scale, expo in [(0, 0.3, 1.0), (1, 0.5, 1.0), (2, 0.6, 2.0)]:
            R_ = float(0.5 + rng.random() * 2.5)
            a = oracle.sum_forces(pos, rad, R_, law, scale, xd, yd, wx, wy, vel=vel, exponent=expo, order=1)
            b = R.sum_forces(pos, rad, R_, law, scale, xd, yd, wx, wy, vel=vel, exponent=expo)
            assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def _script_case(g, k):
    from pyoracle import PDEScript

    xd, yd, wx, wy = (int(v) for v in g[f"c{k}_dims"])
    sc = PDEScript.from_encoded(xd, yd, wx, wy, g[f"c{k}_ops"], g[f"c{k}_iargs"], g[f"c{k}_dargs"],
                                g[f"c{k}_arrays"])
    return sc, g[f"c{k}_f0"], g[f"c{k}_d0"]


def test_pdegrid_script_golden_bit_exact(oracle, golden):
    """Whole Hal::PDEGrid2D call sequences (per-cell Set/Add/Mul/Scale,
    explicit, Dirichlet, per-cell rate and ADI diffusion, both advection
    forms, the whole-grid operations, SetNonNegative, Update and every query;
    include/Hal/Grids/PDEGrid2D.h) written by the reference's own grid: the
    restatement reproduces the final field and deltas, the update count and
    every query result bit for bit."""
    g = golden("pdegrid")
    count = int(g["count"][0])
    assert count == 6
    for k in range(count):
        sc, f0, d0 = _script_case(g, k)
        f, d, uc, rec = oracle.pdegrid_script(sc, f0, d0, 7)
        assert np.array_equal(f, g[f"c{k}_field"]), k
        assert np.array_equal(d, g[f"c{k}_deltas"]), k
        assert uc == int(g[f"c{k}_uc"][0]) == 12
        assert np.array_equal(rec, g[f"c{k}_records"]), k


def test_pdegrid_script_rate_checks(oracle):
    from pyoracle import PDEScript

    f0 = np.zeros(12)
    with pytest.raises(ValueError, match="Diffusion rate above stable maximum value of 0.25"):
        oracle.pdegrid_script(PDEScript(3, 4).add("diffusion", d0=0.3), f0)
    with pytest.raises(ValueError, match="Advection rate component sum above stable maximum value of 0.5"):
        oracle.pdegrid_script(PDEScript(3, 4).add("advection", d0=0.3, d1=-0.25), f0)


@pytest.mark.skipif(not pyoracle.Reference.available() and not __import__("os").path.isdir(
    pyoracle.REF_TREE), reason="reference tree not present")
def test_pdegrid_script_matches_reference_library_random(oracle):
    pyoracle.build(ref=True)
    import importlib.util
    import os

    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(os.path.dirname(__file__), "golden",
                                                                             "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    rng = np.random.default_rng(515)
    for _ in range(4):
        xd, yd = (int(v) for v in rng.integers(1, 30, 2))
        wx, wy = (bool(v) for v in rng.integers(0, 2, 2))
        sc = mg.pdegrid_script(rng, xd, yd, wx, wy)
        f0 = rng.random(xd * yd)
        a = oracle.pdegrid_script(sc, f0)
        b = pyoracle.Reference.pdegrid_script(sc, f0)
        assert all(np.array_equal(x, y) for x, y in zip(a[:2], b[:2])) and a[2] == b[2]
        assert np.array_equal(a[3], b[3])
