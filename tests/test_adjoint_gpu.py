"""Variable-rate ADI and its adjoint on the GPU (hal_cuda_adjoint_*).

Parity is against the FP64 CPU oracle (oracle_dadi_*), which is itself pinned
by its constant-rate limit (the reference-pinned ADI tick) and by finite
differences (tests/test_adjoint_oracle.py):
* forward: FP32 device steps against FP64, max-rel <= 2e-6 (1 + max D) per
  step; for a constant rate it is the ADI tick of hal.Adi;
* gradient: relative L2 error of dL/dD and dL/dsrc <= 1e-4 against the FP64
  adjoint (40 steps and the 500-step workload); dL/ddecay = -sum_t <gbar_t,
  f_t> is a sum with heavy cancellation over every step and cell, so its FP32
  inputs' rounding leaves a larger relative error: 1e-3 over 40 steps, 1e-2
  over 500;
* checkpointing: the gradient does not depend on the checkpoint interval
  (recomputed states are bit-identical);
* finite differences of the device loss (h = 1e-3 along D and the source,
  1e-5 along the decay rate) agree with the directional derivatives within 2%
  plus a fixed bound on the difference's rounding noise: the loss is reduced in FP64 from the FP32 final field, whose error
  eps_f against the FP64 model is measured here, so each loss is within
  |r| eps_f + eps_f^2 / 2 of the exact one (r = f_T - target), and a central
  difference within that over h; the bound allows four times it.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import max_rel, rel_l2

pytestmark = pytest.mark.gpu


def _problem(n, steps, seed, wrap=False):
    from halcuda import workloads

    rng = np.random.default_rng(seed)
    f0 = workloads.gaussian_blobs(n, rng, 8).astype(np.float32)
    D = workloads.rate_field(n, rng).astype(np.float32)
    Dt = workloads.rate_field(n, rng).astype(np.float32)
    src = (rng.random(n * n) * 0.01).astype(np.float32)
    return f0, D, Dt, src


def test_constant_rate_is_the_adi_tick(hal, oracle):
    n, steps, r = 64, 6, 4.0
    rng = np.random.default_rng(1)
    f0 = rng.random(n * n).astype(np.float32)
    src = (rng.random(n * n) * 0.01).astype(np.float32)
    D = np.full(n * n, r, np.float32)
    with hal.Adjoint(n, n) as a:
        a.set_problem(f0, np.zeros_like(f0), steps, 4)
        _, fT = a.forward(D, 0.01, src, want_field=True)
    with hal.Adi(n, n) as adi:
        adi.set_field(f0)
        adi.set_source(src)
        adi.run_ticks(steps, r, 0.01)
        exp32 = adi.get_field()
    ref = oracle.run_ticks(1, f0.astype(np.float64), n, n, r, decay=0.01, src_dense=src.astype(np.float64),
                           ticks=steps)
    tol = 2e-6 * (1 + r) * steps
    assert max_rel(fT, ref) <= tol
    assert max_rel(fT, exp32) <= 2 * tol


@pytest.mark.parametrize("wrap", [(False, False), (True, True), (False, True)])
def test_forward_and_gradient_match_fp64_adjoint(hal, oracle, wrap):
    n, steps = 64, 40
    f0, D, Dt, src = _problem(n, steps, 2)
    decay = 0.005
    # target: the final field of the same model with the second rate field
    _, target, *_ = oracle.dadi_loss_grad(f0, np.zeros(n * n), Dt, decay, src, n, n, steps, *wrap, grad=False)
    loss_ref, fT_ref, gD_ref, gK_ref, gS_ref = oracle.dadi_loss_grad(f0, target, D, decay, src, n, n, steps, *wrap)
    with hal.Adjoint(n, n, *wrap) as a:
        a.set_problem(f0, target.astype(np.float32), steps, 7)
        loss_f, fT = a.forward(D, decay, src, want_field=True)
        loss, gD, gK, gS = a.gradient(D, decay, src)
    assert max_rel(fT, fT_ref) <= 2e-6 * (1 + 5.0) * steps
    assert abs(loss - loss_ref) <= 1e-3 * loss_ref and abs(loss_f - loss) <= 1e-6 * loss
    assert rel_l2(gD, gD_ref) <= 1e-4
    assert rel_l2(gS, gS_ref) <= 1e-4
    assert abs(gK - gK_ref) <= 1e-3 * abs(gK_ref)


def test_gradient_independent_of_checkpoint_interval(hal):
    n, steps = 64, 30
    f0, D, Dt, src = _problem(n, steps, 3)
    target = np.roll(f0, 5)
    out = []
    for every in (1, 7, 30, 100, 0):  # 0: every state kept, nothing recomputed
        with hal.Adjoint(n, n) as a:
            a.set_problem(f0, target, steps, every)
            out.append(a.gradient(D, 0.005, src))
    for loss, gD, gK, gS in out[1:]:
        assert loss == out[0][0]
        assert np.array_equal(gD, out[0][1]) and np.array_equal(gS, out[0][3])
        assert abs(gK - out[0][2]) <= 1e-9 * abs(out[0][2])


def test_finite_differences_on_the_device(hal, oracle):
    """Central differences of the device loss, h = 1e-3, on a 128^2 grid,
    within 2% plus a fixed bound on their rounding noise."""
    n, steps = 128, 100
    f0, D, Dt, src = _problem(n, steps, 4)
    rng = np.random.default_rng(9)
    h = 1e-3
    with hal.Adjoint(n, n) as a:
        a.set_problem(f0, np.zeros_like(f0), steps, 22)
        _, target = a.forward(Dt, 0.005, src, want_field=True)
        a.set_problem(f0, target, steps, 22)
        loss, gD, gK, gS = a.gradient(D, 0.005, src)
        _, fT = a.forward(D, 0.005, src, want_field=True)
        # the FP32 forward's error against the FP64 model at D
        _, fT64, *_ = oracle.dadi_loss_grad(f0, target, D, 0.005, src, n, n, steps, grad=False)
        eps_f = float(np.linalg.norm(fT.astype(np.float64) - fT64))
        assert eps_f <= 1e-6 * np.linalg.norm(fT64)
        def noise(step):
            return 4.0 * (np.sqrt(2.0 * loss) * eps_f + 0.5 * eps_f * eps_f) / step

        def fd(f, step):
            return (f(step) - f(-step)) / (2 * step)

        for _ in range(4):
            v = rng.standard_normal(n * n).astype(np.float32)
            f1 = fd(lambda t: a.forward(D + np.float32(t) * v, 0.005, src), h)
            dd = float(gD.astype(np.float64) @ v.astype(np.float64))
            assert abs(f1 - dd) <= 2e-2 * abs(dd) + noise(h), (f1, dd, noise(h))
        # the decay rate (0.005) compounds over the steps: a step of 1e-3
        # (20% of it) leaves a large third-order truncation error, so the
        # decay direction takes h = 1e-5
        hk = 1e-5
        f1 = fd(lambda t: a.forward(D, 0.005 + t, src), hk)
        assert abs(f1 - gK) <= 2e-2 * abs(gK) + noise(hk), (f1, gK, noise(hk))
        f1 = fd(lambda t: a.forward(D, 0.005, src + np.float32(t) * np.sign(gS)), h)
        ds = float(np.abs(gS.astype(np.float64)).sum())
        assert abs(f1 - ds) <= 2e-2 * abs(ds) + noise(h), (f1, ds, noise(h))


@pytest.mark.parametrize("xd,yd,wrap", [(48, 60, (True, True)), (100, 37, (True, False)),
                                         (64, 45, (False, True)), (3, 96, (True, True))])
def test_wrapped_lines_of_any_length(hal, oracle, xd, yd, wrap):
    """Wrapped axes whose length is not a power of two take the
    Sherman-Morrison split of the cyclic line solve: forward and gradient
    against the FP64 adjoint (Thomas with the same split) on rectangular
    grids, at the bounds of the square-grid test."""
    steps = 24
    rng = np.random.default_rng(xd * 131 + yd)
    X, Y = np.meshgrid(np.arange(xd), np.arange(yd), indexing="ij")
    f0 = (np.exp(-((X - 0.3 * xd) ** 2 + (Y - 0.6 * yd) ** 2) / (0.05 * xd * yd)) +
          0.2 * rng.random((xd, yd))).ravel().astype(np.float32)
    D = (0.5 + 4.5 * rng.random(xd * yd)).astype(np.float32)
    Dt = (0.5 + 4.5 * rng.random(xd * yd)).astype(np.float32)
    src = (rng.random(xd * yd) * 0.01).astype(np.float32)
    decay = 0.005
    _, target, *_ = oracle.dadi_loss_grad(f0, np.zeros(xd * yd), Dt, decay, src, xd, yd, steps, *wrap, grad=False)
    loss_ref, fT_ref, gD_ref, gK_ref, gS_ref = oracle.dadi_loss_grad(f0, target, D, decay, src, xd, yd, steps,
                                                                     *wrap)
    with hal.Adjoint(xd, yd, *wrap) as a:
        a.set_problem(f0, target.astype(np.float32), steps, 5)
        loss_f, fT = a.forward(D, decay, src, want_field=True)
        loss, gD, gK, gS = a.gradient(D, decay, src)
    assert max_rel(fT, fT_ref) <= 2e-6 * (1 + 5.0) * steps
    assert abs(loss - loss_ref) <= 1e-3 * loss_ref and abs(loss_f - loss) <= 1e-6 * loss
    assert rel_l2(gD, gD_ref) <= 1e-4, rel_l2(gD, gD_ref)
    assert rel_l2(gS, gS_ref) <= 1e-4, rel_l2(gS, gS_ref)
    assert abs(gK - gK_ref) <= 1e-3 * abs(gK_ref)


def test_rejects_bad_input(hal):
    with pytest.raises(ValueError):
        hal.Adjoint(hal.ADJOINT_MAX_SIDE + 1, 8)
    with hal.Adjoint(16, 16) as a:
        with pytest.raises(ValueError):
            a.forward(np.ones(256, np.float32), 0.0)
        with pytest.raises(ValueError):
            a.set_problem(np.zeros(255, np.float32), np.zeros(255, np.float32), 3)


def test_parameter_recovery_workload_on_a_64_copy(hal, oracle):
    """The parameter-recovery workload's shape on a 64 x 64 copy (500 steps,
    checkpoints every 22, rates in [0.5, 5], decay 0.005) against the FP64
    CPU adjoint."""
    from halcuda import workloads

    w = workloads.adjoint_inputs(n=64, steps=500)
    n = 64
    _, target, *_ = oracle.dadi_loss_grad(w["f0"], np.zeros(n * n), w["D_true"], w["decay"], w["src"], n, n,
                                          w["steps"], grad=False)
    loss_ref, _, gD_ref, gK_ref, gS_ref = oracle.dadi_loss_grad(w["f0"], target, w["D"], w["decay"], w["src"], n, n,
                                                                w["steps"])
    with hal.Adjoint(n, n) as a:
        a.set_problem(w["f0"], target.astype(np.float32), w["steps"], w["checkpoint_every"])
        loss, gD, gK, gS = a.gradient(w["D"], w["decay"], w["src"])
    # the field gradients to 1e-4 (measured: about 5e-6 for dL/dD and 4e-5
    # for dL/dsrc); dL/ddecay sums 500 steps of <gbar, f> with heavy
    # cancellation, so its FP32 inputs leave about 5e-3
    assert abs(loss - loss_ref) <= 1e-4 * loss_ref
    assert rel_l2(gD, gD_ref) <= 1e-4
    assert rel_l2(gS, gS_ref) <= 1e-4
    assert abs(gK - gK_ref) <= 1e-2 * abs(gK_ref)
