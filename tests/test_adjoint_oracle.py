"""The FP64 variable-rate ADI oracle and its adjoint (CPU).

No reference implementation exists for either (the reference has no
variable-rate ADI and no gradient code), so the oracle is pinned by:
* its constant-rate limit, which must equal the reference-pinned ADI tick
  (oracle_tick mode 1: Diffusion2DADI + decay + source + Update);
* central finite differences of its own loss, in FP64, for the gradients
  with respect to the rate field D, the decay and the source field.
"""
from __future__ import annotations

import numpy as np
import pytest


@pytest.mark.parametrize("wrap", [(False, False), (True, True), (True, False)])
def test_constant_rate_limit_is_the_adi_tick(oracle, wrap):
    rng = np.random.default_rng(7)
    xd, yd, r, decay = 13, 9, 2.5, 0.01
    f = rng.random(xd * yd)
    s = rng.random(xd * yd) * 0.01
    exp = oracle.run_ticks(1, f, xd, yd, r, wrapX=wrap[0], wrapY=wrap[1], decay=decay, src_dense=s, ticks=1)
    got, _ = oracle.dadi_step(f, np.full(xd * yd, r), xd, yd, wrap[0], wrap[1], decay, s)
    assert np.abs(got - exp).max() <= 1e-13 * np.abs(exp).max()


def test_single_cell_and_single_line_grids(oracle):
    """A wrapped line of one cell has no face; 1-wide grids still conserve."""
    for xd, yd in ((1, 1), (1, 7), (6, 1)):
        f = np.linspace(0.5, 1.5, xd * yd)
        D = np.full(xd * yd, 3.0)
        for wrap in (False, True):
            out, _ = oracle.dadi_step(f, D, xd, yd, wrap, wrap)
            assert abs(out.sum() - f.sum()) <= 1e-12 * f.sum()


@pytest.mark.parametrize("wrap", [(False, False), (True, True), (False, True)])
def test_gradient_matches_central_differences(oracle, wrap):
    rng = np.random.default_rng(11)
    xd, yd, steps = 9, 7, 4
    n = xd * yd
    f0 = rng.random(n)
    target = rng.random(n)
    D = 0.5 + 4.5 * rng.random(n)
    src = rng.random(n) * 0.01
    decay = 0.005
    loss, _, gD, gK, gS = oracle.dadi_loss_grad(f0, target, D, decay, src, xd, yd, steps, *wrap)
    h = 1e-6
    for _ in range(3):
        v = rng.standard_normal(n)
        lp = oracle.dadi_loss_grad(f0, target, D + h * v, decay, src, xd, yd, steps, *wrap, grad=False)[0]
        lm = oracle.dadi_loss_grad(f0, target, D - h * v, decay, src, xd, yd, steps, *wrap, grad=False)[0]
        fd = (lp - lm) / (2 * h)
        assert abs(fd - gD @ v) <= 1e-6 * max(1.0, abs(fd)), (fd, gD @ v)
        lp = oracle.dadi_loss_grad(f0, target, D, decay, src + h * v, xd, yd, steps, *wrap, grad=False)[0]
        lm = oracle.dadi_loss_grad(f0, target, D, decay, src - h * v, xd, yd, steps, *wrap, grad=False)[0]
        fd = (lp - lm) / (2 * h)
        assert abs(fd - gS @ v) <= 1e-6 * max(1.0, abs(fd)), (fd, gS @ v)
    lp = oracle.dadi_loss_grad(f0, target, D, decay + h, src, xd, yd, steps, *wrap, grad=False)[0]
    lm = oracle.dadi_loss_grad(f0, target, D, decay - h, src, xd, yd, steps, *wrap, grad=False)[0]
    fd = (lp - lm) / (2 * h)
    assert abs(fd - gK) <= 1e-6 * max(1.0, abs(fd)), (fd, gK)
    assert loss > 0


def test_step_is_linear_and_its_operators_symmetric(oracle):
    """The reverse pass relies on two facts: a step is linear in f (for zero
    source and fixed D), and (I - L/2) is symmetric, so its transpose solve is
    the same solve.  Checked through <u, S(v)> = <S(u), v> of the symmetric
    half-step map S = (I - L/2)^-1 (I + L/2) along one axis (a 1-wide grid)."""
    rng = np.random.default_rng(3)
    xd, yd = 8, 11
    n = xd * yd
    D = 0.5 + 4.5 * rng.random(n)
    u, v = rng.standard_normal(n), rng.standard_normal(n)
    a, b = 0.7, -1.3
    step = lambda f: oracle.dadi_step(f, D, xd, yd, False, True, 0.01, None)[0]
    assert np.allclose(step(a * u + b * v), a * step(u) + b * step(v), rtol=0, atol=1e-12)
    # a 1 x L grid: the x-sweep is the identity, so a step is the y half-step
    # map, which is symmetric (its factors commute: both are polynomials in L)
    L = 17
    D1 = 0.5 + 4.5 * rng.random(L)
    u1, v1 = rng.standard_normal(L), rng.standard_normal(L)
    for wrap in (False, True):
        s1 = lambda f: oracle.dadi_step(f, D1, 1, L, False, wrap, 0.0, None)[0]
        assert abs(u1 @ s1(v1) - s1(u1) @ v1) <= 1e-12
