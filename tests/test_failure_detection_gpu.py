"""Failure detection on the GPU without a GPU fault.

Every device-side wait of the library is bounded: a staged tile's mbarrier
wait gives up after its limit, records the failure in the handle's device
error word, waits once more (bounded) so that no copy is still writing into
shared memory, and the CTA returns.  The host reads the word at the next
synchronising call and reports HAL_CUDA_ETIMEOUT; the handle then refuses
every later tick, since its field is undefined.

Here the wait is made to run out on purpose through the two-tick kernel's test
hook (hal_cuda_diffusion_test_stall: each tile's mbarrier expects 16 bytes
more than its tensor copy brings -- a flag that nothing sets).  Nothing faults,
traps or hangs: each CTA waits 2 x 50 ms.  The test checks the status, the
stopped handle, and that the CUDA context stays usable: a new handle in the
same process gives the oracle's field.
"""
from __future__ import annotations

import time

import numpy as np
import pytest

from conftest import max_rel

pytestmark = pytest.mark.gpu


def test_bounded_wait_runs_out_and_the_context_stays_usable(hal, oracle):
    xd, yd = 96, 256
    rng = np.random.default_rng(5)
    f0 = rng.random(xd * yd).astype(np.float32)
    with hal.Diffusion(xd, yd) as d:
        d.set_field(f0)
        d.set_blocking(2)
        d.test_stall(1, 0.05)
        t0 = time.perf_counter()
        d.run_ticks(2, 0.2, 0.0)
        with pytest.raises(RuntimeError, match="gave up waiting"):
            d.get_field()
        waited = time.perf_counter() - t0
        assert waited < 10.0  # bounded: 2 x 50 ms per CTA, not the 2 s default
        # the handle has stopped: its field is undefined
        with pytest.raises(RuntimeError, match="stopped"):
            d.run_ticks(2, 0.2, 0.0)
    # the context is intact: a new handle runs and matches the oracle
    exp = oracle.run_ticks(0, f0.astype(np.float64), xd, yd, 0.2, ticks=4)
    with hal.Diffusion(xd, yd) as d:
        d.set_field(f0)
        d.set_blocking(2)
        d.run_ticks(4, 0.2, 0.0)
        out = d.get_field()
    assert max_rel(out, exp) <= 1e-5
    # and the hook switched off leaves a handle's ticks normal
    with hal.Diffusion(xd, yd) as d:
        d.set_field(f0)
        d.set_blocking(2)
        d.test_stall(1, 0.05)
        d.test_stall(0)
        d.run_ticks(4, 0.2, 0.0)
        assert max_rel(d.get_field(), exp) <= 1e-5


def test_stall_hook_rejects_bad_waits(hal):
    with hal.Diffusion(16, 16) as d:
        with pytest.raises(ValueError):
            d.test_stall(1, 3.0)
        with pytest.raises(ValueError):
            d.test_stall(1, -1.0)
