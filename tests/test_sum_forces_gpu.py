"""Force laws and force sums: SphericalAgent2D::SumForces on the GPU.

SumForces (include/Hal/Agents/SphericalAgent2D.h:74-102) sums an overlap
functor's forces over an agent's neighbours, starting from the agent's own
velocity, and returns the sum of the positive forces, which models use to gate
division (examples/OffLatticeExample.cpp:156-165).  hal_cuda_sum_forces runs
it for every agent at once in FP64:

* against vectors written by the reference's own SumForces on its agent grid
  (tests/golden/sumforces.npz), in the agent grid's visiting order: bit-exact
  for the linear law and the clamped law of OffLatticeExample.cpp:147-154;
  the power law of examples/Chemotaxis.cpp:128-130 goes through the device's
  pow, so it is held to 1e-13 of the largest value instead;
* against the oracle on larger random scenes, in both visiting orders;
* in the CPU backend's order with the linear law from zero velocity it is
  AccumulateForces, bit for bit.

The FP32 resident dispatch and step with a law (hal_cuda_agents_dispatch_law /
_step_law) are checked against the FP64 oracle within the FP32 force
tolerance, max|err| <= 1e-4 * max|v|, for the deltas and the sums; their bins
stay bit-exact.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import max_rel

pytestmark = pytest.mark.gpu

TOL32 = 1e-4
TOL_POW = 1e-13


def _case(g, k):
    xd, yd, wx, wy, R_, law, scale, expo = (float(v) for v in g[f"c{k}_params"])
    scene = g[f"c{k}_scene"][0].decode()
    vin = g[f"c{k}_velin"] if f"c{k}_velin" in g.files else None
    return dict(pos=g[f"{scene}_pos"], rad=g[f"{scene}_rad"], xd=int(xd), yd=int(yd), wx=int(wx), wy=int(wy),
                R=R_, law=int(law), scale=scale, expo=expo, vin=vin, vel=g[f"c{k}_vel"], sums=g[f"c{k}_sums"],
                tag=f"case {k} {scene} law {int(law)} R {R_}")


def test_sum_forces_golden(hal, golden):
    g = golden("sumforces")
    count = int(g["count"][0])
    exact = 0
    for k in range(count):
        c = _case(g, k)
        n = c["rad"].size
        with hal.Agents(c["xd"], c["yd"], n) as ag:
            v, sums = ag.sum_forces(c["pos"], c["rad"], c["R"], c["law"], c["scale"], c["xd"], c["yd"], c["wx"],
                                    c["wy"], velocities=c["vin"], exponent=c["expo"], order=hal.ORDER_AGENTGRID)
        if c["law"] == hal.FORCE_POWER:
            assert max_rel(v, c["vel"]) <= TOL_POW, c["tag"]
            assert max_rel(sums, c["sums"]) <= TOL_POW, c["tag"]
        else:
            assert np.array_equal(v, c["vel"]), c["tag"]
            assert np.array_equal(sums, c["sums"]), c["tag"]
            exact += 1
    assert exact == 20


@pytest.mark.parametrize("xd,yd,wx,wy", [(96, 80, 0, 0), (64, 96, 1, 1), (50, 70, 1, 0)])
@pytest.mark.parametrize("order", [0, 1])
def test_sum_forces_random_against_oracle(hal, oracle, xd, yd, wx, wy, order):
    rng = np.random.default_rng(xd * 7 + yd + 3 * wx + 5 * wy + 11 * order)
    n = 12000
    m = n // 3
    pos = np.concatenate([np.stack([rng.random(n - m) * xd, rng.random(n - m) * yd], 1),
                          np.array([xd, yd]) * 0.5 + rng.normal(0, 4.0, (m, 2))])
    pos = np.clip(pos, 0, np.array([xd, yd]) * (1 - 1e-12)).ravel()
    rad = 0.25 + 0.35 * rng.random(n)
    vel = (rng.random(2 * n) - 0.5) * 0.2
    with hal.Agents(xd, yd, n) as ag:
        for law, scale, expo in [(0, 0.1, 1.0), (1, 0.25, 1.0), (2, 0.7, 2.0)]:
            got, gs = ag.sum_forces(pos, rad, 1.3, law, scale, xd, yd, wx, wy, velocities=vel, exponent=expo,
                                    order=order)
            exp, es = oracle.sum_forces(pos, rad, 1.3, law, scale, xd, yd, wx, wy, vel=vel, exponent=expo,
                                        order=order)
            if law == 2:
                assert max_rel(got, exp) <= TOL_POW and max_rel(gs, es) <= TOL_POW
            else:
                assert np.array_equal(got, exp), (law, order)
                assert np.array_equal(gs, es), (law, order)
        # the bins of the last call are the CPU's
        off, bucket = ag.get_bins()
        e_off, e_bucket = oracle.agent_bins(pos, xd, yd)
        assert np.array_equal(off, e_off) and np.array_equal(bucket, e_bucket)


def test_sum_forces_backend_order_is_accumulate_forces(hal):
    rng = np.random.default_rng(5)
    xd, yd, n = 70, 60, 9000
    pos = np.stack([rng.random(n) * xd, rng.random(n) * yd], 1).ravel()
    rad = np.full(n, 0.5)
    with hal.Agents(xd, yd, n) as ag:
        v, sums = ag.sum_forces(pos, rad, 1.0, hal.FORCE_LINEAR, 0.1, xd, yd, 0, 1, order=hal.ORDER_BACKEND,
                                sums=False)
        assert sums is None
        exp = ag.accumulate_forces(pos, rad, 1.0, 0.1, xd, yd, 0, 1)
    assert np.array_equal(v, exp)


@pytest.mark.parametrize("law,scale,expo", [(0, 0.1, 1.0), (1, 0.25, 1.0), (2, 0.7, 2.0)])
def test_resident_dispatch_and_step_with_law(hal, oracle, law, scale, expo):
    """FP32 resident dispatch and step with a law and force sums against the
    FP64 oracle (backend order) on the same float32 positions."""
    rng = np.random.default_rng(40 + law)
    xd, yd, n = 128, 96, 20000
    pos = np.stack([rng.random(n) * xd, rng.random(n) * yd], 1).astype(np.float32).ravel()
    rad = (0.3 + 0.3 * rng.random(n)).astype(np.float32)
    p64, r64 = pos.astype(np.float64), rad.astype(np.float64)
    exp_v, exp_s = oracle.sum_forces(p64, r64, 1.2, law, scale, xd, yd, 0, 0, exponent=expo, order=0)
    with hal.Agents(xd, yd, n) as ag:
        ag.upload(pos, rad)
        ag.dispatch_law(1.2, law, scale, exponent=expo, sums=True)
        v = ag.download()
        s = ag.get_force_sums()
        off, bucket = ag.get_bins()
        assert max_rel(v, exp_v) <= TOL32
        assert max_rel(s, exp_s) <= TOL32
        assert (s >= 0).all() and s.max() > 0
        e_off, e_bucket = oracle.agent_bins(p64, xd, yd)
        assert np.array_equal(off, e_off) and np.array_equal(bucket, e_bucket)
        # one resident tick: the same deltas and sums at the starting positions,
        # then the move of the FP32 restatement
        ag.set_velocities(None)
        ag.step_law(1, 1.2, law, scale, exponent=expo, sums=True, friction=0.5, maxVel=0.4)
        p1, v1 = ag.get_state()
        dv = ag.download()
        assert np.array_equal(dv, v)
        assert np.array_equal(ag.get_force_sums(), s)
        ep, ev = oracle.agents_move(pos, np.zeros(2 * n, np.float32), dv, xd, yd, False, False, 0.5, 0.4, f32=True)
        assert np.array_equal(p1, ep) and np.array_equal(v1, ev)
        # a plain dispatch computes no sums
        ag.dispatch(1.2, 0.1)
        with pytest.raises(ValueError, match="did not compute force sums"):
            ag.get_force_sums()


def test_clamped_law_sums_gate_division(hal, oracle):
    """The off-lattice example's pattern: a clamped Hooke law, the force sum of
    each cell, and a division gate tanh(bias - sum * weight)
    (examples/OffLatticeExample.cpp:145-165).  The gate computed from the
    device's FP64 sums equals the one from the oracle's."""
    rng = np.random.default_rng(9)
    xd = yd = 30
    n = 2500
    pos = (np.array([xd, yd]) * 0.5 + rng.normal(0, 5.0, (n, 2)))
    pos = np.clip(pos, 0, xd * (1 - 1e-12)).ravel()
    rad = np.full(n, 0.25)
    with hal.Agents(xd, yd, n) as ag:
        _, sums = ag.sum_forces(pos, rad, 0.5, hal.FORCE_LINEAR_CLAMPED, 0.25, xd, yd, 0, 0)
    _, exp = oracle.sum_forces(pos, rad, 0.5, 1, 0.25, xd, yd, 0, 0)
    assert np.array_equal(np.tanh(0.01 - sums * 0.02), np.tanh(0.01 - exp * 0.02))
    assert (sums > 0).sum() > n // 4


def test_force_law_rejections(hal):
    with hal.Agents(8, 8, 4) as ag:
        pos = np.array([1.0, 1.0, 1.5, 1.2])
        rad = np.array([0.5, 0.5])
        with pytest.raises(ValueError, match="unknown force law"):
            ag.sum_forces(pos, rad, 1.0, 7, 0.1, 8, 8, 0, 0)
        with pytest.raises(ValueError, match="unknown order"):
            ag.sum_forces(pos, rad, 1.0, 0, 0.1, 8, 8, 0, 0, order=5)
        with pytest.raises(ValueError, match="scale must be finite"):
            ag.sum_forces(pos, rad, 1.0, 0, float("nan"), 8, 8, 0, 0)
        with pytest.raises(ValueError, match="differing from construction"):
            ag.sum_forces(pos, rad, 1.0, 0, 0.1, 9, 8, 0, 0)
