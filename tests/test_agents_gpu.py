"""Agent forces on the GPU against the oracle and the golden vectors.

* bins (cell offsets and bucket order) are integer results: bit-exact;
* the FP64 interface call (hal_cuda_accumulate_forces) keeps positions in
  FP64 and sums with IEEE operations in the CPU's order: bit-exact for any
  double positions;
* the FP32 resident dispatch: max|err| <= 1e-4 * max|v| (float32 sums of
  up to a few dozen pair terms).
"""
from __future__ import annotations

import math

import numpy as np
import pytest

from conftest import max_rel

pytestmark = pytest.mark.gpu

SCENES = ("walls", "torus", "mixed", "tiny", "empty")


def test_seed1234_scene_bit_exact(hal, golden):
    """tests/IAgentForceBackend2DTests.cpp:109-121 (GPU epsilon 1e-3 there)."""
    g = golden("agents")
    pos, rad = g["s1234_pos"], g["s1234_rad"]
    # the device rounds positions to float32; the golden run used doubles,
    # so compare the FP64 interface with the oracle fed the rounded values
    with hal.Agents(16, 16, 60) as ag:
        v = ag.accumulate_forces(pos, rad, 3.0, 0.4, 16, 16, True, True)
        off, bucket = ag.get_bins()
    np.testing.assert_allclose(v, g["s1234_vel"], rtol=0, atol=1e-5)
    assert np.array_equal(off, g["s1234_off"])
    assert np.array_equal(bucket, g["s1234_bucket"])


def test_seed1234_scene_matches_oracle_on_float_positions(hal, oracle, golden):
    g = golden("agents")
    pos = g["s1234_pos"].astype(np.float32).astype(np.float64)
    rad = g["s1234_rad"]
    exp, eoff, eb = oracle.accumulate_forces(pos, rad, 3.0, 0.4, 16, 16, 1, 1)
    with hal.Agents(16, 16, 60) as ag:
        v = ag.accumulate_forces(pos, rad, 3.0, 0.4, 16, 16, True, True)
        off, bucket = ag.get_bins()
    assert np.array_equal(v, exp)
    assert np.array_equal(off, eoff) and np.array_equal(bucket, eb)


@pytest.mark.parametrize("name", SCENES)
def test_golden_scenes(hal, golden, name):
    g = golden("agents")
    xd, yd, n, wx, wy, R, k = g[f"{name}_params"]
    xd, yd, n, wx, wy = int(xd), int(yd), int(n), bool(wx), bool(wy)
    pos, rad = g[f"{name}_pos"], g[f"{name}_rad"]
    with hal.Agents(xd, yd, max(n, 1)) as ag:
        v = ag.accumulate_forces(pos, rad, R, k, xd, yd, wx, wy)
        off, bucket = ag.get_bins()
        assert np.array_equal(v, g[f"{name}_vel"]), name  # FP64 path, float32 positions
        assert np.array_equal(off, g[f"{name}_off"]), name
        assert np.array_equal(bucket, g[f"{name}_bucket"]), name
        ag.upload(pos.astype(np.float32), rad.astype(np.float32))
        ag.dispatch(R, k, wx, wy)
        v32 = ag.download()
        off2, bucket2 = ag.get_bins()
    assert np.array_equal(off2, g[f"{name}_off"]) and np.array_equal(bucket2, g[f"{name}_bucket"])
    if n:
        assert max_rel(v32, g[f"{name}_vel"]) <= 1e-4, name


def test_bruteforce_ground_truth(hal, golden):
    """IAgentForceBackend2DTests.cpp:55-100: an all-pairs sum without buckets."""
    g = golden("agents")
    pos = g["s1234_pos"].astype(np.float32).astype(np.float64)
    rad = g["s1234_rad"]
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
    with hal.Agents(16, 16, n) as ag:
        v = ag.accumulate_forces(pos, rad, 3.0, 0.4, 16, 16, True, True)
    np.testing.assert_allclose(v, exp, rtol=1e-12, atol=1e-12)


def test_coincident_zero_and_errors(hal):
    """IAgentForceBackend2DTests.cpp:123-165, AgentForceKernel2DTests.cpp:125-143."""
    with hal.Agents(8, 8, 4) as ag:
        v = ag.accumulate_forces([4.0, 4.0, 4.0, 4.0], [0.5, 0.5], 2.0, 1.0, 8, 8, False, False)
        assert v.shape == (4,) and np.all(v == 0.0)
        v = ag.accumulate_forces([], [], 2.0, 1.0, 8, 8, False, False)
        assert v.size == 0
        off, _ = ag.get_bins()
        assert np.all(off == 0)
        with pytest.raises(ValueError):
            ag.accumulate_forces([1.0, 1.0, 2.0], [0.5, 0.5], 2.0, 1.0, 8, 8, False, False)
        with pytest.raises(ValueError):
            ag.accumulate_forces([1.0] * 10, [0.5] * 5, 2.0, 1.0, 8, 8, False, False)
        with pytest.raises(ValueError):
            ag.accumulate_forces([1.0, 1.0], [0.5], 2.0, 1.0, 16, 8, False, False)
        with pytest.raises(ValueError):
            ag.upload(np.ones(10, np.float32), np.ones(5, np.float32))


def test_million_agent_workload(hal, oracle):
    """1,000,000 agents in 2048^2: bins bit-exact, FP64 forces bit-exact,
    FP32 forces within 1e-4."""
    from halcuda import workloads

    w = workloads.agent_inputs(1_000_000, 2048, seed=3)
    pos32, rad32 = w["positions"], w["radii"]
    pos = pos32.astype(np.float64)
    rad = rad32.astype(np.float64)
    exp, eoff, eb = oracle.accumulate_forces(pos, rad, 1.0, 0.1, 2048, 2048, 0, 0, threads=16)
    with hal.Agents(2048, 2048, 1_000_000) as ag:
        v = ag.accumulate_forces(pos, rad, 1.0, 0.1, 2048, 2048, False, False)
        off, bucket = ag.get_bins()
        assert np.array_equal(off, eoff)
        assert np.array_equal(bucket, eb)
        assert np.array_equal(v, exp)
        ag.upload(pos32, rad32)
        ag.dispatch(1.0, 0.1)
        v32 = ag.download()
        off2, bucket2 = ag.get_bins()
    assert np.array_equal(off2, eoff) and np.array_equal(bucket2, eb)
    assert max_rel(v32, exp) <= 1e-4


def test_large_grid_repeated_dispatches(hal, oracle):
    """25M cells (the counts are cleared inside the scan at every size, only
    where a 4-cell group held a count): three dispatches of different agent
    sets on one handle, bins bit-exact against the oracle each time, so a
    count left behind by an earlier dispatch would show."""
    xd, yd = 5000, 5000
    rng = np.random.default_rng(11)
    with hal.Agents(xd, yd, 300_000) as ag:
        for n in (300_000, 120_000, 250_000):
            pos32 = np.empty(2 * n, np.float32)
            pos32[0::2] = rng.random(n) * xd
            pos32[1::2] = rng.random(n) * yd
            # a dense cluster, so that some groups hold several counts
            m = n // 5
            pos32[0:2 * m:2] = (xd / 2 + rng.standard_normal(m) * 20).astype(np.float32)
            pos32[1:2 * m:2] = (yd / 2 + rng.standard_normal(m) * 20).astype(np.float32)
            rad32 = (0.3 + rng.random(n) * 0.2).astype(np.float32)
            _, eoff, eb = oracle.accumulate_forces(pos32.astype(np.float64), rad32.astype(np.float64), 1.0, 0.1,
                                                    xd, yd, 0, 0, threads=16)
            ag.upload(pos32, rad32)
            ag.dispatch(1.0, 0.1)
            ag.sync()
            off, bucket = ag.get_bins()
            assert np.array_equal(off, eoff), n
            assert np.array_equal(bucket, eb), n


@pytest.mark.parametrize("wrap", [False, True])
def test_fp64_positions_off_the_float_grid(hal, oracle, wrap):
    """The FP64 interface path keeps positions in FP64: cells are floored in
    FP64 (a position just below an integer stays in the lower cell, as on the
    CPU) and the forces equal the CPU backend's bit for bit."""
    rng = np.random.default_rng(21)
    dim, n = 48, 6000
    pos = rng.random(2 * n) * dim
    # a sixth of the agents sit within 1e-12 of a cell boundary, on either side
    k = n // 6
    edges = rng.integers(1, dim, 2 * k).astype(np.float64)
    pos[: 2 * k] = edges + rng.choice([-1e-12, -3e-15, 0.0, 3e-15, 1e-12], 2 * k)
    rad = 0.3 + 0.4 * rng.random(n)
    v_exp, off_exp, b_exp = oracle.accumulate_forces(pos, rad, 1.7, 0.3, dim, dim, int(wrap), int(wrap))
    with hal.Agents(dim, dim, n) as ag:
        v = ag.accumulate_forces(pos, rad, 1.7, 0.3, dim, dim, wrap, wrap)
        off, b = ag.get_bins()
    assert np.array_equal(off, off_exp)
    assert np.array_equal(b, b_exp)
    assert np.array_equal(v, v_exp)
