"""The device-resident agent step (hal_cuda_agents_step) against the oracle.

One tick is a force dispatch whose kernel then applies SphericalAgent2D's
update (vel += delta, CapVelocity, ForceMove via MoveSafePT, ApplyFriction;
include/Hal/Agents/SphericalAgent2D.h:133-162).  The update is FP32 with each
operation rounded to nearest, so given the tick's own velocity deltas (which
the handle still returns) it matches the oracle's FP32 restatement bit for
bit; the FP32 restatement tracks the FP64 one, which is pinned to the
reference's agent grid.  Over several ticks the resident run equals a host
loop of upload / dispatch / download / oracle update exactly, because the
force pass is deterministic for given positions.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _scene(n, xd, yd, seed, edge_frac=0.3):
    rng = np.random.default_rng(seed)
    pos = np.stack([rng.random(n) * xd, rng.random(n) * yd], 1)
    edge = rng.random(n) < edge_frac
    pos[edge, 0] = np.where(rng.random(edge.sum()) < 0.5, rng.random(edge.sum()) * 0.5,
                            xd - rng.random(edge.sum()) * 0.5)
    pos = np.minimum(pos, np.array([xd, yd]) * (1 - 1e-6)).astype(np.float32).ravel()
    rad = (0.3 + 0.4 * rng.random(n)).astype(np.float32)
    vel = ((rng.random(2 * n) - 0.5) * 0.6).astype(np.float32)
    return pos, rad, vel


@pytest.mark.parametrize("wrap,friction,maxVel", [((False, False), 0.5, -1.0), ((True, True), 0.9, 0.35),
                                                   ((True, False), 0.0, 0.2), ((False, True), 1.0, 0.0)])
def test_one_tick_matches_f32_oracle_bit_exact(hal, oracle, wrap, friction, maxVel):
    n, xd, yd = 5000, 64, 48
    pos, rad, vel = _scene(n, xd, yd, 1)
    with hal.Agents(xd, yd, n) as ag:
        ag.upload(pos, rad)
        ag.set_velocities(vel)
        ag.step(1, 1.5, 0.3, *wrap, friction=friction, maxVel=maxVel)
        p1, v1 = ag.get_state()
        dv = ag.download()
    ep, ev = oracle.agents_move(pos, vel, dv, xd, yd, *wrap, friction, maxVel, f32=True)
    assert np.array_equal(p1, ep)
    assert np.array_equal(v1, ev)
    # the deltas are the dispatch's forces at the starting positions
    with hal.Agents(xd, yd, n) as ag:
        ag.upload(pos, rad)
        ag.dispatch(1.5, 0.3, *wrap)
        assert np.array_equal(ag.download(), dv)


def test_many_ticks_equal_host_loop(hal, oracle):
    n, xd, yd, ticks = 20000, 96, 96, 12
    pos, rad, vel = _scene(n, xd, yd, 2)
    args = (1.2, 0.2, True, False)
    with hal.Agents(xd, yd, n) as ag:
        ag.upload(pos, rad)
        ag.set_velocities(vel)
        ag.step(ticks, *args, friction=0.8, maxVel=0.5)
        got_p, got_v = ag.get_state()
    p, v = pos.copy(), vel.copy()
    with hal.Agents(xd, yd, n) as ag:
        for _ in range(ticks):
            ag.upload(p, rad)
            ag.dispatch(*args)
            p, v = oracle.agents_move(p, v, ag.download(), xd, yd, True, False, 0.8, 0.5, f32=True)
    assert np.array_equal(got_p, p)
    assert np.array_equal(got_v, v)
    assert not np.array_equal(got_p, pos)


def test_tracks_fp64_model(hal, oracle):
    """Five ticks against the FP64 model (oracle forces and update in FP64):
    the FP32 trajectory stays within float rounding.  A pair whose distance
    is within rounding of the interaction radius can be in range in one
    precision and not the other (the spring force does not vanish there), so
    a few agents in a thousand may differ by more."""
    n, xd, yd, ticks = 3000, 40, 40, 5
    pos, rad, vel = _scene(n, xd, yd, 3, edge_frac=0.0)
    with hal.Agents(xd, yd, n) as ag:
        ag.upload(pos, rad)
        ag.set_velocities(vel)
        ag.step(ticks, 1.0, 0.1, True, True, friction=0.5, maxVel=0.4)
        got_p, got_v = ag.get_state()
    p, v = pos.astype(np.float64), vel.astype(np.float64)
    for _ in range(ticks):
        dv = oracle.accumulate_forces(p, rad.astype(np.float64), 1.0, 0.1, xd, yd, True, True)
        dv = dv[0] if isinstance(dv, tuple) else dv
        p, v = oracle.agents_move(p, v, dv, xd, yd, True, True, 0.5, 0.4)
    d = np.abs(got_p - p)
    d = np.minimum(d, np.abs(d - xd))  # a coordinate within rounding of the wrap point
    dv = np.abs(got_v - v)
    assert np.median(d) <= 1e-5 and np.median(dv) <= 1e-5
    assert np.mean(d > 1e-3) <= 5e-3 and np.mean(dv > 1e-3) <= 5e-3


def test_resident_state_and_errors(hal):
    n, xd, yd = 100, 16, 16
    pos, rad, vel = _scene(n, xd, yd, 4)
    with hal.Agents(xd, yd, n) as ag:
        ag.upload(pos, rad)
        p0, v0 = ag.get_state()
        assert np.array_equal(p0, pos) and not v0.any()  # upload resets velocities
        ag.step(0, 1.0, 0.1)
        assert np.array_equal(ag.get_state()[0], pos)
        with pytest.raises(ValueError):
            ag.step(1, -1.0, 0.1)
        with pytest.raises(ValueError):
            ag.step(1, 1.0, 0.1, friction=float("nan"))
        with pytest.raises(ValueError):
            ag.set_velocities(np.zeros(3, np.float32))
        ag.set_velocities(vel)
        ag.set_velocities(None)
        assert not ag.get_state()[1].any()
    with hal.Agents(xd, yd, 10) as ag:  # no agents: a tick is a no-op
        ag.upload(np.zeros(0, np.float32), np.zeros(0, np.float32))
        ag.step(3, 1.0, 0.1, True, True)
        p, v = ag.get_state()
        assert p.size == 0 and v.size == 0
