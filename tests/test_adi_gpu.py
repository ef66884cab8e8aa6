"""ADI on the GPU (FP32) against the FP64 oracle and the golden vectors.

Tolerance: the GPU solves in FP32 what the reference solves in FP64 by
Thomas.  One step is held to max|err| <= TOL(r) * max|f| with
TOL(r) = 2e-6 * (1 + r) (the line systems' condition number grows like
1 + 2r); multi-step runs to rel-L2 <= 1e-5, the 2048^2 workload target.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

from conftest import max_rel, rel_l2

pytestmark = pytest.mark.gpu


def TOL(r):
    return 2e-6 * (1.0 + r)


def _eigen(nx, ny):
    x = np.arange(nx)[:, None]
    y = np.arange(ny)[None, :]
    return (np.sin(2.0 * math.pi * x / nx) * np.sin(2.0 * math.pi * y / ny)).ravel()


def _lambda_cn(r, n, k=1):
    s = math.sin(math.pi * k / n) ** 2
    return (1.0 - 2.0 * r * s) / (1.0 + 2.0 * r * s)


def _step_err(out, exp, f):
    scale = max(np.abs(f).max(), np.abs(exp).max(), 1e-30)
    return float(np.abs(out - exp).max() / scale)


def test_diffuse_adi_golden(hal, golden):
    g = golden("stencil")
    for k in range(int(g["count"][0])):
        xd, yd, wx, wy, use_bc = (int(v) for v in g[f"c{k}_dims"])
        r = float(g[f"c{k}_rates"][1])
        f = g[f"c{k}_field"]
        with hal.Adi(xd, yd) as a:
            if use_bc:
                out = a.diffuse_adi_bc(f, g[f"c{k}_deltas"].copy(), r, wx, wy, g[f"c{k}_ghost"])
            else:
                out = a.diffuse_adi(f, g[f"c{k}_deltas"].copy(), r, xd, yd, wx, wy)
        err = _step_err(out, g[f"c{k}_adi"], f)
        assert err <= TOL(r), f"case {k}: {xd}x{yd} wrap {wx}{wy} bc {use_bc} r {r}: {err}"


def test_adi_eigenmode_through_interface(hal):
    """tests/IDiffusionBackend2DTests.cpp:115-144 (GPU epsilon 1e-4 there)."""
    nx, ny, r = 12, 18, 0.3
    f = _eigen(nx, ny)
    lam = _lambda_cn(r, nx) * _lambda_cn(r, ny)
    with hal.Adi(nx, ny) as a:
        for _ in range(2):  # second call reuses the handle
            out = a.diffuse_adi(f, np.zeros_like(f), r, nx, ny, True, True)
            np.testing.assert_allclose(f + out, lam * f, rtol=0, atol=1e-5)


def test_run_steps_cn_nth_power(hal):
    """tests/AdiKernel2DTests.cpp:18-68: 24x16, r = 0.8, 50 steps (1e-3 there)."""
    nx, ny, r, steps = 24, 16, 0.8, 50
    f = _eigen(nx, ny)
    lam = _lambda_cn(r, nx) * _lambda_cn(r, ny)
    with hal.Adi(nx, ny) as a:
        out = a.run_steps(f, steps, r, True, True)
    np.testing.assert_allclose(out, lam ** steps * f, rtol=0, atol=1e-5)


def test_zero_flux_mass_and_cpu_match(hal, golden):
    """tests/AdiKernel2DTests.cpp:70-141: 20x14, r = 0.6, 5 steps, 1e-4 there."""
    g = golden("ticks")
    f = g["kat_adi_field"]
    with hal.Adi(20, 14) as a:
        out = a.run_steps(f, 5, 0.6, False, False)
    assert abs(out.astype(np.float64).sum() - f.sum()) <= 1e-5 * f.sum()
    assert max_rel(out, g["kat_adi_out"]) <= 1e-5


def test_adi_tick_golden(hal, golden):
    """ADI + decay + dense source, 40x48, r = 5, 20 ticks."""
    g = golden("ticks")
    xd, yd, r, decay, ticks = g["adi_params"]
    with hal.Adi(int(xd), int(yd)) as a:
        a.set_field(g["adi_field"])
        a.set_source(g["adi_src"])
        a.run_ticks(int(ticks), r, decay)
        out = a.get_field()
    assert rel_l2(out, g["adi_out"]) <= 1e-5


def test_adi_tick_dirichlet_periodic_uptake_golden(hal, golden):
    """Periodic x, Dirichlet y ends, per-agent uptake (counts from a binned
    agent set): the coupled tick of the agent workload."""
    g = golden("ticks")
    xd, yd, r, decay, uptake, ticks = g["cpl_params"]
    xd, yd = int(xd), int(yd)
    counts = g["cpl_counts"]
    # agents at the cell centres reproduce the per-cell counts
    cells = np.repeat(np.arange(xd * yd), counts)
    pos = np.empty(2 * cells.size, np.float32)
    pos[0::2] = cells // yd + 0.5
    pos[1::2] = cells % yd + 0.5
    with hal.Agents(xd, yd, cells.size) as ag, hal.Adi(xd, yd) as a:
        ag.upload(pos, np.full(cells.size, 0.5, np.float32))
        ag.dispatch(1.0, 0.1)
        ag.sync()
        off, _ = ag.get_bins()
        assert np.array_equal(np.diff(off), counts)
        a.set_field(g["cpl_field"])
        a.set_dirichlet(g["cpl_ghost"])
        a.set_uptake(ag, uptake)
        a.run_ticks(int(ticks), r, decay, True, False)
        out = a.get_field()
    assert rel_l2(out, g["cpl_out"]) <= 1e-5


@pytest.mark.parametrize("xd,yd", [(512, 256), (256, 512)])
@pytest.mark.parametrize("wrapX,wrapY,dirichlet,uptake", [
    (True, False, True, 2e-3), (False, True, True, 0.0), (True, True, False, 2e-3), (False, False, False, 0.0)])
def test_tensor_staged_tick_against_oracle(hal, oracle, xd, yd, wrapX, wrapY, dirichlet, uptake):
    """Resident ticks whose line lengths are multiples of 256: both sweeps run
    the tensor-staged form (swizzled staged rows, the per-quad permutation of
    the solution rows, 16-byte write-out with the commit, f and src loaded
    ahead) over several CTAs, with every boundary kind, a dense source, decay
    and per-agent uptake, against the FP64 oracle."""
    rng = np.random.default_rng(xd + 3 * yd + 7 * wrapX + 11 * wrapY)
    n = xd * yd
    f0 = rng.random(n).astype(np.float32)
    src = (rng.random(n) * 1e-3).astype(np.float32)
    ghost = rng.random(2 * (xd + yd)).astype(np.float32) if dirichlet else None
    r, decay, ticks = 3.0, 5e-3, 6
    nAgents = 20000
    pos = np.empty(2 * nAgents, np.float32)
    pos[0::2] = rng.random(nAgents) * xd
    pos[1::2] = rng.random(nAgents) * yd
    with hal.Agents(xd, yd, nAgents) as ag, hal.Adi(xd, yd) as a:
        counts = None
        if uptake:
            ag.upload(pos, np.full(nAgents, 0.5, np.float32))
            ag.dispatch(1.0, 0.1)
            ag.sync()
            off, _ = ag.get_bins()
            counts = np.diff(off).astype(np.int32)
            assert counts.sum() == nAgents and counts.max() >= 2
            a.set_uptake(ag, uptake)
        a.set_field(f0)
        a.set_source(src)
        if ghost is not None:
            a.set_dirichlet(ghost)
        a.run_ticks(ticks, r, decay, wrapX, wrapY)
        out = a.get_field()
    exp = oracle.run_ticks(1, f0.astype(np.float64), xd, yd, r, wrapX, wrapY,
                           None if ghost is None else ghost.astype(np.float64), decay,
                           src_dense=src.astype(np.float64), uptake_count=counts, uptake=uptake, ticks=ticks)
    assert rel_l2(out, exp) <= 1e-5, rel_l2(out, exp)


@pytest.mark.parametrize("wrapX,wrapY,dirichlet,uptake", [(True, False, True, 2e-3), (False, True, False, 0.0)])
def test_ragged_last_tile_tick_against_oracle(hal, oracle, wrapX, wrapY, dirichlet, uptake):
    """x-lines of 2048 over 1940 lines: tensor-staged 16-line x-sweep tiles,
    the last one 4 lines wide, with a periodic or Dirichlet x-axis, a dense
    source, decay and uptake, against the FP64 oracle."""
    xd, yd = 2048, 1940
    rng = np.random.default_rng(77 + wrapX)
    n = xd * yd
    f0 = rng.random(n).astype(np.float32)
    src = (rng.random(n) * 1e-3).astype(np.float32)
    ghost = rng.random(2 * (xd + yd)).astype(np.float32) if dirichlet else None
    r, decay, ticks = 5.0, 1e-2, 3
    nAgents = 100000
    pos = np.empty(2 * nAgents, np.float32)
    pos[0::2] = rng.random(nAgents) * xd
    pos[1::2] = rng.random(nAgents) * yd
    with hal.Agents(xd, yd, nAgents) as ag, hal.Adi(xd, yd) as a:
        counts = None
        if uptake:
            ag.upload(pos, np.full(nAgents, 0.5, np.float32))
            ag.dispatch(1.0, 0.1)
            ag.sync()
            off, _ = ag.get_bins()
            counts = np.diff(off).astype(np.int32)
            a.set_uptake(ag, uptake)
        a.set_field(f0)
        a.set_source(src)
        if ghost is not None:
            a.set_dirichlet(ghost)
        a.run_ticks(ticks, r, decay, wrapX, wrapY)
        out = a.get_field()
    exp = oracle.run_ticks(1, f0.astype(np.float64), xd, yd, r, wrapX, wrapY,
                           None if ghost is None else ghost.astype(np.float64), decay,
                           src_dense=src.astype(np.float64), uptake_count=counts, uptake=uptake, ticks=ticks,
                           threads=16)
    assert rel_l2(out, exp) <= 1e-5, rel_l2(out, exp)
    # the last tile's four lines (y = 1936 .. 1939; HAL's layout is x * yDim + y)
    last = out.reshape(xd, yd)[:, 1936:]
    assert rel_l2(last, exp.reshape(xd, yd)[:, 1936:]) <= 1e-5


@pytest.mark.parametrize("xd,yd,wrapX,wrapY,dirichlet", [
    (2048, 2048, False, False, True),   # both sweeps tensor-staged: ghost lines, implicit ends
    (2048, 2048, True, False, False),   # periodic x-lines, wrapped cross lines of the y-sweep
    (2048, 1920, False, True, False),   # wrapped cross lines of the x-sweep, 120 tiles
    (1024, 4096, False, False, True),   # x-lines of 1024 over 4096 lines
    (4096, 1024, True, False, False),   # y-lines of 1024 over 4096 lines, wrapped cross lines
])
def test_large_tensor_staged_grids_against_oracle(hal, oracle, xd, yd, wrapX, wrapY, dirichlet):
    """Full-size grids whose sweeps run the tensor-staged tiles over many
    CTAs: every boundary kind of the cross axis, Dirichlet ends, decay and a
    dense source, against the FP64 oracle."""
    rng = np.random.default_rng(xd + 13 * yd + 7 * wrapX)
    n = xd * yd
    f0 = rng.random(n).astype(np.float32)
    src = (rng.random(n) * 1e-3).astype(np.float32)
    ghost = rng.random(2 * (xd + yd)).astype(np.float32) if dirichlet else None
    r, decay, ticks = 5.0, 1e-2, 3
    with hal.Adi(xd, yd) as a:
        a.set_field(f0)
        a.set_source(src)
        if ghost is not None:
            a.set_dirichlet(ghost)
        a.run_ticks(ticks, r, decay, wrapX, wrapY)
        out = a.get_field()
    exp = oracle.run_ticks(1, f0.astype(np.float64), xd, yd, r, wrapX, wrapY,
                           None if ghost is None else ghost.astype(np.float64), decay,
                           src_dense=src.astype(np.float64), ticks=ticks, threads=16)
    assert rel_l2(out, exp) <= 1e-5, rel_l2(out, exp)
    assert max_rel(out, exp) <= 2e-6 * (1 + r) * ticks, max_rel(out, exp)


LINES = [1, 2, 3, 31, 32, 33, 63, 64, 65, 100, 257, 1000, 2048, 4096]


@pytest.mark.parametrize("L", LINES)
def test_line_lengths_against_oracle(hal, oracle, L):
    """Every chunk layout: one chunk, partial last chunks, full clusters."""
    rng = np.random.default_rng(L)
    other = {1: 7, 2: 5, 3: 64, 4096: 3}.get(L, 37)
    for (xd, yd) in ((L, other), (other, L)):
        f = rng.random(xd * yd)
        ghost = rng.random(2 * (xd + yd))
        for r in (0.3, 5.0, 100.0):
            for wx, wy, gh in ((False, False, None), (True, True, None), (True, False, ghost),
                               (False, True, ghost)):
                exp = oracle.diffuse_adi(f, np.zeros_like(f), r, xd, yd, wx, wy, gh)
                with hal.Adi(xd, yd) as a:
                    if gh is None:
                        out = a.diffuse_adi(f, np.zeros_like(f), r, xd, yd, wx, wy)
                    else:
                        out = a.diffuse_adi_bc(f, np.zeros_like(f), r, wx, wy, gh)
                err = _step_err(out, exp, f)
                assert err <= TOL(r), (xd, yd, r, wx, wy, gh is None, err)


@pytest.mark.parametrize("xd,yd,wx,wy,dirichlet", [(5000, 24, True, False, False), (17, 4100, False, True, True),
                                                   (4097, 9, False, False, True)])
def test_lines_above_max_through_the_interface(hal, oracle, xd, yd, wx, wy, dirichlet):
    """A side above HAL_CUDA_ADI_MAX_LINE: DiffuseADI (and its Dirichlet
    form) solves the step in FP64, Thomas per line in the CPU backend's order,
    so the deltas equal the CPU's bit for bit; the resident FP32 ticks refuse
    such a grid."""
    rng = np.random.default_rng(xd + yd)
    f = rng.random(xd * yd)
    d = (rng.random(xd * yd) - 0.5) * 0.1
    ghost = rng.random(2 * (xd + yd)) if dirichlet else None
    with hal.Adi(xd, yd) as a:
        if dirichlet:
            got = a.diffuse_adi_bc(f, d.copy(), 3.0, wx, wy, ghost)
        else:
            got = a.diffuse_adi(f, d.copy(), 3.0, xd, yd, wx, wy)
        exp = oracle.diffuse_adi(f, d, 3.0, xd, yd, wx, wy, ghost=ghost)
        assert np.array_equal(got, exp)
        assert np.abs(got - d).max() > 0
        with pytest.raises(RuntimeError, match="ADI line length"):
            a.run_ticks(1, 3.0, 0.0)


@pytest.mark.parametrize("xd,yd,wx,wy,dirichlet", [(512, 384, False, False, False), (300, 257, True, True, False),
                                                   (640, 96, False, True, True), (129, 1024, True, False, True),
                                                   (1, 7, False, False, False), (7, 1, True, True, False),
                                                   (2, 3, True, True, False), (3, 2, False, False, True),
                                                   (1, 1, False, False, True), (17, 33, True, False, False)])
def test_exact_mode_interface_bit_exact(hal, oracle, xd, yd, wx, wy, dirichlet):
    """With set_exact, DiffuseADI and its Dirichlet form solve every size in
    FP64, Thomas per line in the CPU backend's order: the deltas equal the
    CPU's bit for bit (without it these sizes take the FP32 solve)."""
    rng = np.random.default_rng(xd * 3 + yd)
    f = rng.random(xd * yd)
    d = (rng.random(xd * yd) - 0.5) * 0.1
    ghost = rng.random(2 * (xd + yd)) if dirichlet else None
    with hal.Adi(xd, yd) as a:
        a.set_exact(True)
        if dirichlet:
            got = a.diffuse_adi_bc(f, d.copy(), 4.0, wx, wy, ghost)
        else:
            got = a.diffuse_adi(f, d.copy(), 4.0, xd, yd, wx, wy)
        exp = oracle.diffuse_adi(f, d, 4.0, xd, yd, wx, wy, ghost=ghost)
        assert np.array_equal(got.view(np.uint64), exp.view(np.uint64))
        if xd * yd < 4096:
            return
        a.set_exact(False)
        if dirichlet:
            fp32 = a.diffuse_adi_bc(f, d.copy(), 4.0, wx, wy, ghost)
        else:
            fp32 = a.diffuse_adi(f, d.copy(), 4.0, xd, yd, wx, wy)
        assert not np.array_equal(fp32, exp)
        assert _step_err(fp32, exp, f) <= TOL(4.0)


def test_rejects_bad_sizes(hal):
    with hal.Adi(4, 4) as a:
        with pytest.raises(ValueError):
            a.run_steps(np.zeros(15, np.float32), 1, 0.1)
        with pytest.raises(ValueError):
            a.diffuse_adi(np.zeros(12), np.zeros(12), 0.1, 3, 4, False, False)
        with pytest.raises(ValueError):
            a.diffuse_adi(np.zeros(16), np.zeros(15), 0.1, 4, 4, False, False)


def test_adi_2048_workload_200_ticks(hal, oracle):
    """The 2048^2 ADI workload end to end: r = 5, decay 0.01, source field,
    zero-flux, 200 ticks; FP32 on the GPU against FP64 Thomas (target
    rel-L2 <= 1e-5)."""
    from halcuda import workloads

    w = workloads.adi_inputs(2048, seed=2)
    exp = oracle.run_ticks(1, w["field"], 2048, 2048, w["diffRate"], decay=w["decay"],
                           src_dense=w["src"], ticks=200, threads=16)
    with hal.Adi(2048, 2048) as a:
        a.set_field(w["field"])
        a.set_source(w["src"])
        a.run_ticks(200, w["diffRate"], w["decay"])
        out = a.get_field()
    e2 = rel_l2(out, exp)
    print(f"2048^2 ADI 200 ticks: rel-L2 {e2:.3e} max-rel {max_rel(out, exp):.3e}")
    assert e2 <= 1e-5


def test_host_ticks_match_resident_ticks(hal):
    from halcuda import workloads

    w = workloads.adi_inputs(256, seed=4, blobs=20)
    f32 = w["field"].astype(np.float32)
    s32 = w["src"].astype(np.float32)
    with hal.Adi(256, 256) as a:
        a.set_field(f32)
        a.set_source(s32)
        a.run_ticks(7, 5.0, 0.01)
        res = a.get_field()
        host = a.run_ticks_host(f32.copy(), s32, 7, 5.0, 0.01)
    assert np.array_equal(res, host)


def test_profile_graph_leaves_the_field(hal):
    """The steady-state sweep profile replays back-to-back launches on the
    same inputs and leaves the resident field as it was; the ticks after it
    equal ticks without it."""
    n = 256
    rng = np.random.default_rng(12)
    f0 = rng.random(n * n).astype(np.float32)
    src = (rng.random(n * n) * 0.01).astype(np.float32)
    outs = []
    for probe in (False, True):
        with hal.Adi(n, n) as a:
            a.set_field(f0)
            a.set_source(src)
            a.run_ticks(3, 5.0, 0.01)
            if probe:
                before = a.get_field()
                msx, msy = a.profile_graph(10, 5.0, 0.01)
                assert msx > 0 and msy > 0
                assert np.array_equal(a.get_field(), before)
            a.run_ticks(3, 5.0, 0.01)
            outs.append(a.get_field())
    assert np.array_equal(outs[0], outs[1])


def test_pinned_host_buffers_take_the_direct_path(hal):
    """Pinned host buffers are read and written by the transposes in place
    (no staging copy): set_field / get_field and the host-to-host ticks give
    the same bits as pageable buffers, for a field and a source."""
    torch = pytest.importorskip("torch")
    xd, yd = 640, 384
    rng = np.random.default_rng(17)
    f0 = rng.random(xd * yd).astype(np.float32)
    src = (rng.random(xd * yd) * 1e-3).astype(np.float32)
    pf = torch.from_numpy(f0.copy()).pin_memory()
    ps = torch.from_numpy(src.copy()).pin_memory()
    pf_np, ps_np = pf.numpy(), ps.numpy()
    with hal.Adi(xd, yd) as a:
        exp = a.run_ticks_host(f0.copy(), src, 5, 3.0, 0.01)
        got = a.run_ticks_host(pf_np, ps_np, 5, 3.0, 0.01)  # in place, through the pinned pages
        assert got is pf_np
        assert np.array_equal(got, exp)
        # set_field from pinned memory, get_field into pinned memory
        a.set_field(ps_np)
        back = torch.empty(xd * yd, dtype=torch.float32).pin_memory()
        a.get_field(out=back.numpy())
        assert np.array_equal(back.numpy(), src)
