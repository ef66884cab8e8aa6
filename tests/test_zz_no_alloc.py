"""hal_cuda_agents_forces_noalloc against the handle-based dispatch.

The no-alloc entry point is for callers that cannot allocate device memory
themselves (a framework that owns every byte of device memory in its own pool,
or a plugin handed only input and output pointers).  It runs the same FP32 bin
and force kernels as hal_cuda_agents_upload/dispatch/download, in the same
order, with its scratch in a static device array instead of allocated buffers,
so its velocity deltas must equal the dispatch's bit for bit, on consecutive
calls (the array keeps the previous call's contents), also when two calls are
queued on one stream with no synchronisation between them.  The dispatch's
deltas are in turn within the FP32 force tolerance, max|err| <= 1e-4 * max|v|,
of the FP64 oracle.  Device buffers for the inputs and outputs are allocated
here by torch, as a caller with its own pool would.

This file is collected last so that a run stopping at the first failure has
already run every other test.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import max_rel

pytestmark = pytest.mark.gpu

TOL = 1e-4


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    if not t.cuda.is_available():
        pytest.fail("torch sees no CUDA device")
    return t


def _dispatch(hal, w):
    """Velocity deltas from the handle-based entry points."""
    n = w["radii"].size
    with hal.Agents(w["xDim"], w["yDim"], n) as ag:
        ag.upload(w["positions"], w["radii"])
        ag.dispatch(w["interactionRad"], w["springConstant"], w["wrapX"], w["wrapY"])
        return ag.download()


def _device_inputs(torch, w):
    n = w["radii"].size
    pos = torch.from_numpy(w["positions"]).cuda()
    rad = torch.from_numpy(w["radii"]).cuda()
    vel = torch.full((2 * n,), float("nan"), dtype=torch.float32, device="cuda")
    return pos, rad, vel


def _call(hal, w, pos, rad, vel, stream=0):
    hal.agents_forces_noalloc(pos.data_ptr(), rad.data_ptr(), w["radii"].size, vel.data_ptr(),
                              w["interactionRad"], w["springConstant"], w["xDim"], w["yDim"], w["wrapX"],
                              w["wrapY"], stream)


def _noalloc(hal, torch, w, stream=0):
    pos, rad, vel = _device_inputs(torch, w)
    torch.cuda.synchronize()
    _call(hal, w, pos, rad, vel, stream)
    torch.cuda.synchronize()
    return vel.cpu().numpy()


def _scene(n, xd, yd, seed, R, k, wrapX, wrapY, cluster=0.3):
    rng = np.random.default_rng(seed)
    m = int(n * cluster)
    uni = rng.random((n - m, 2)) * (xd, yd)
    clu = rng.random(2) * (xd, yd) + rng.normal(0.0, 6.0, (m, 2))
    pos = np.concatenate([uni, clu])
    hi = (np.nextafter(np.float32(xd), np.float32(0)), np.nextafter(np.float32(yd), np.float32(0)))
    pos = np.clip(pos, 0.0, np.array(hi, dtype=np.float64)).astype(np.float32)
    radii = (0.3 + 0.4 * rng.random(n)).astype(np.float32)
    return dict(positions=pos.ravel(), radii=radii, xDim=xd, yDim=yd, interactionRad=R,
                springConstant=k, wrapX=wrapX, wrapY=wrapY)


def _oracle_forces(oracle, w):
    v, _, _ = oracle.accumulate_forces(w["positions"].astype(np.float64), w["radii"].astype(np.float64),
                                       w["interactionRad"], w["springConstant"], w["xDim"], w["yDim"],
                                       w["wrapX"], w["wrapY"])
    return v


def test_noalloc_matches_dispatch_on_consecutive_calls(hal, torch, oracle):
    # at both limits: 65536 agents in 256 x 256 = 65536 cells, walls
    a = _scene(hal.NOALLOC_MAX_AGENTS, 256, 256, seed=11, R=1.0, k=0.1, wrapX=False, wrapY=False)
    # then a smaller scene on a wrapped grid, reusing the array's stale contents
    b = _scene(20000, 100, 120, seed=12, R=2.5, k=0.3, wrapX=True, wrapY=True)
    for w in (a, b):
        exp = _dispatch(hal, w)
        got = _noalloc(hal, torch, w)
        assert np.array_equal(got, exp)
        assert np.abs(exp).max() > 0
        assert max_rel(exp, _oracle_forces(oracle, w)) <= TOL


def test_noalloc_two_calls_queued_on_one_stream(hal, torch):
    """Two calls with different scenes back to back on one caller stream, no
    synchronisation between them: the second call's clearing of the shared
    counts is ordered after the first call's last kernel, so both are exact."""
    a = _scene(30000, 200, 150, seed=21, R=1.0, k=0.1, wrapX=False, wrapY=True)
    b = _scene(12000, 90, 70, seed=22, R=1.5, k=0.25, wrapX=True, wrapY=False)
    s = torch.cuda.Stream()
    ins = [_device_inputs(torch, w) for w in (a, b)]
    torch.cuda.synchronize()
    for w, (pos, rad, vel) in zip((a, b), ins):
        _call(hal, w, pos, rad, vel, s.cuda_stream)
    s.synchronize()
    for w, (_, _, vel) in zip((a, b), ins):
        assert np.array_equal(vel.cpu().numpy(), _dispatch(hal, w))


def test_noalloc_on_a_caller_stream_and_rejections(hal, torch):
    w = _scene(5000, 64, 48, seed=13, R=1.5, k=0.2, wrapX=True, wrapY=False)
    exp = _dispatch(hal, w)
    s = torch.cuda.Stream()
    got = _noalloc(hal, torch, w, stream=s.cuda_stream)
    assert np.array_equal(got, exp)

    dev = torch.zeros(2 * 16, dtype=torch.float32, device="cuda")
    p = dev.data_ptr()
    with pytest.raises(ValueError, match="no-alloc limit"):
        hal.agents_forces_noalloc(p, p, hal.NOALLOC_MAX_AGENTS + 1, p, 1.0, 0.1, 8, 8)
    with pytest.raises(ValueError, match="no-alloc limit"):
        hal.agents_forces_noalloc(p, p, 16, p, 1.0, 0.1, 257, 256)
    host = np.zeros(32, dtype=np.float32)
    with pytest.raises(ValueError, match="device memory"):
        hal.agents_forces_noalloc(host.ctypes.data, p, 16, p, 1.0, 0.1, 8, 8)
    with pytest.raises(ValueError, match="interactionRad"):
        hal.agents_forces_noalloc(p, p, 16, p, -1.0, 0.1, 8, 8)
