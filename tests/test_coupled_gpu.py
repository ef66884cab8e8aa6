"""The agent-field coupled workload at full size, against the oracle.

1,000,000 disc agents (radius 0.5; 70% uniform, 30% in a Gaussian cluster of
sigma 100 cells) move through the resident agent step (hal_cuda_agents_step:
linear repulsion, cutoff 1.0, stiffness 0.1, walls) on a 2048 x 2048 grid.
They share that grid with a resident ADI field (D*dt/dx^2 = 5, decay 0.01,
U[0, 0.01) source, zero-flux; 200 Gaussian blobs), and every tick each agent
removes 0.001 of its cell's field value (hal_cuda_adi_set_uptake: the
PDEGrid2D::Mul(Isq(), -uptake) of examples/CompetitiveRelease.cpp:147, one
per agent in the cell, src/Agents/CpuAgentForceBackend2D.cpp:87-97 bins).
100 ticks.

* Every 10th tick the agents' positions are downloaded before the step; the
  bins that the step builds from them (cell offsets and the bucket order) must
  equal the oracle's binning of the same positions bit for bit.
* Every tick the field is advanced by the FP64 oracle tick with that tick's
  per-cell agent counts; after 100 ticks the device field must be within
  rel-L2 1e-5 of it.
"""
from __future__ import annotations

import os

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

N = 2048
TICKS = 100
R, K, UPTAKE = 1.0, 0.1, 0.001
RATE, DECAY = 5.0, 0.01
FRICTION, MAXVEL = 0.5, -1.0


def test_coupled_agents_and_adi_field_100_ticks(hal, oracle):
    from halcuda import workloads

    ag_in = workloads.agent_inputs(1_000_000, N, seed=3)
    fd_in = workloads.adi_inputs(N, seed=2)
    pos0, rad = ag_in["positions"], ag_in["radii"]
    n = rad.size
    f32 = fd_in["field"].astype(np.float32)
    s32 = fd_in["src"].astype(np.float32)
    f64 = f32.astype(np.float64)
    s64 = s32.astype(np.float64)
    threads = os.cpu_count() or 1
    checked = 0
    moved = False
    with hal.Agents(N, N, n) as ag, hal.Adi(N, N) as a:
        ag.set_stream(a.stream())  # one stream orders the step before the tick
        ag.upload(pos0, rad)
        a.set_field(f32)
        a.set_source(s32)
        a.set_uptake(ag, UPTAKE)
        for t in range(TICKS):
            before = ag.get_state()[0] if t % 10 == 0 else None
            ag.step(1, R, K, False, False, friction=FRICTION, maxVel=MAXVEL)
            off, bucket = ag.get_bins()
            if before is not None:
                e_off, e_bucket = oracle.agent_bins(before.astype(np.float64), N, N)
                assert np.array_equal(off, e_off), f"tick {t}: cell offsets differ"
                assert np.array_equal(bucket, e_bucket), f"tick {t}: bucket order differs"
                moved = moved or not np.array_equal(before, pos0)
                checked += 1
            counts = np.diff(off).astype(np.int32)
            assert counts.sum() == n
            a.run_ticks(1, RATE, DECAY)
            f64 = oracle.run_ticks(1, f64, N, N, RATE, decay=DECAY, src_dense=s64, uptake_count=counts,
                                   uptake=UPTAKE, ticks=1, threads=threads)
        out = a.get_field()
        ag.sync()
        ag.set_stream(None)  # back to its own stream before the ADI handle's is destroyed
    assert checked == TICKS // 10
    assert moved, "the agents never moved"
    err = rel_l2(out, f64)
    assert err <= 1e-5, err


@pytest.mark.parametrize("wrap", [(False, False), (True, False)])
def test_run_coupled_equals_alternating_calls(hal, wrap):
    """hal_cuda_adi_run_coupled (each tick: the agents' resident step, then the
    ADI tick with their uptake, all ticks as one cached graph on the field's
    stream) equals alternating agents.step(1) / run_ticks(1) calls bit for bit:
    the field, the positions and the velocities, over runs of both buffer
    parities and a cached-graph replay, with the agent handle on its own
    stream; a dispatch after the run and a new upload are ordered after it."""
    from halcuda import workloads

    n_side, n_agents = 384, 40000
    ag_in = workloads.agent_inputs(n_agents, n_side, seed=5)
    fd_in = workloads.adi_inputs(n_side, seed=6, blobs=20)
    pos0, rad = ag_in["positions"], ag_in["radii"]
    f32 = fd_in["field"].astype(np.float32)
    s32 = fd_in["src"].astype(np.float32)
    wx, wy = wrap
    runs = (3, 4, 3, 5)

    def fresh(ag, a):
        ag.upload(pos0, rad)
        a.set_field(f32)
        a.set_source(s32)
        a.set_uptake(ag, UPTAKE)

    with hal.Agents(n_side, n_side, n_agents) as ag, hal.Adi(n_side, n_side) as a:
        ag.set_stream(a.stream())
        fresh(ag, a)
        for k in runs:
            for _ in range(k):
                ag.step(1, R, K, wx, wy, friction=FRICTION, maxVel=MAXVEL)
                a.run_ticks(1, RATE, DECAY, wx, wy)
        exp_f = a.get_field()
        exp_p, exp_v = ag.get_state()
        ag.dispatch(R, K, wx, wy)
        exp_d = ag.download()
        ag.set_stream(None)
    with hal.Agents(n_side, n_side, n_agents) as ag, hal.Adi(n_side, n_side) as a:
        fresh(ag, a)  # the agent handle keeps its own stream
        for k in runs:
            a.run_coupled(ag, k, RATE, DECAY, wx, wy, R, K, FRICTION, MAXVEL)
        got_f = a.get_field()
        got_p, got_v = ag.get_state()
        ag.dispatch(R, K, wx, wy)
        got_d = ag.download()
        # an upload resets the agents: the next run bins them afresh
        fresh(ag, a)
        a.run_coupled(ag, 3, RATE, DECAY, wx, wy, R, K, FRICTION, MAXVEL)
        again = a.get_field()
        with pytest.raises(ValueError, match="coupled"):
            with hal.Agents(n_side, n_side, 10) as other:
                a.run_coupled(other, 1, RATE, DECAY, wx, wy, R, K, FRICTION, MAXVEL)
    assert np.array_equal(got_f, exp_f)
    assert np.array_equal(got_p, exp_p) and np.array_equal(got_v, exp_v)
    assert np.array_equal(got_d, exp_d)
    with hal.Agents(n_side, n_side, n_agents) as ag, hal.Adi(n_side, n_side) as a:
        ag.set_stream(a.stream())
        fresh(ag, a)
        for _ in range(3):
            ag.step(1, R, K, wx, wy, friction=FRICTION, maxVel=MAXVEL)
            a.run_ticks(1, RATE, DECAY, wx, wy)
        assert np.array_equal(again, a.get_field())
        ag.set_stream(None)
