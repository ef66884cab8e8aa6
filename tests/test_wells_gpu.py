"""Batched wells (MultiWellExperiment::Step over many wells per launch).

Every well of a batch must equal the same well run alone on the single-grid
handles bit for bit (same kernels, same arithmetic), and through them the
CPU oracle within the usual tolerances:
* explicit and ADI fields: bit-identical to hal.Diffusion / hal.Adi
  run_ticks; against the FP64 oracle ticks max-rel <= 1e-5 (explicit) and
  <= 2e-6 (1 + r) per tick (ADI);
* agent forces: bit-identical to hal.Agents dispatch; bins per well follow
  the CPU's order, so the FP32 forces equal the single-grid ones exactly.
  They are also compared directly with the FP64 oracle's forces (max-rel
  <= 1e-4), as are the fields of a sample of the 512-well workload.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import max_rel

pytestmark = pytest.mark.gpu

R, K = 1.0, 0.1


def _mixed_wells(rng):
    """Sizes that exercise every tile path: float4 and scalar rows, ragged
    line groups, 1-wide grids, periodic and zero-flux, with and without
    agents and sources."""
    specs = [
        (64, 64, "explicit", 0.2, 0.001, False, False, 500),
        (37, 50, "explicit", 0.24, 0.0, True, False, 0),
        (130, 33, "explicit", 0.05, 0.02, False, True, 300),
        (1, 40, "explicit", 0.1, 0.0, False, False, 0),
        (96, 80, "adi", 5.0, 0.01, False, False, 800),
        (257, 31, "adi", 1.5, 0.0, True, True, 0),
        (33, 200, "adi", 10.0, 0.005, False, True, 200),
        (48, 1, "adi", 2.0, 0.0, False, False, 0),
        (256, 256, "adi", 3.0, 0.02, False, False, 2000),
        (200, 128, "explicit", 0.15, 0.01, False, False, 1500),
    ]
    wells, fields, srcs, pos, rad, counts = [], [], [], [], [], []
    for i, (xd, yd, kind, rate, decay, wx, wy, na) in enumerate(specs):
        wells.append(dict(xDim=xd, yDim=yd, kind=kind, diffRate=rate, decay=decay, wrapX=wx, wrapY=wy,
                          maxAgents=na + 7))
        fields.append(rng.random(xd * yd).astype(np.float32))
        srcs.append((rng.random(xd * yd) * 0.01).astype(np.float32) if i % 2 == 0 else None)
        counts.append(na)
        p = rng.random((na, 2)) * (xd, yd)
        hi = np.array([np.nextafter(np.float32(xd), np.float32(0)), np.nextafter(np.float32(yd), np.float32(0))])
        pos.append(np.minimum(p, hi).astype(np.float32).ravel())
        rad.append((0.3 + 0.4 * rng.random(na)).astype(np.float32))
    return wells, fields, srcs, np.array(counts, np.int32), pos, rad


def _alone(hal, w, field, src, ticks):
    with (hal.Adi(w["xDim"], w["yDim"]) if w["kind"] == "adi" else hal.Diffusion(w["xDim"], w["yDim"])) as h:
        h.set_field(field)
        if src is not None:
            h.set_source(src)
        h.run_ticks(ticks, w["diffRate"], w["decay"], w["wrapX"], w["wrapY"])
        return h.get_field()


FORCE_TOL = 1e-4


def _oracle_forces(oracle, w, pos, rad):
    v, _, _ = oracle.accumulate_forces(pos.astype(np.float64), rad.astype(np.float64), R, K, w["xDim"],
                                       w["yDim"], w.get("wrapX", False), w.get("wrapY", False))
    return v


def _alone_forces(hal, w, pos, rad):
    with hal.Agents(w["xDim"], w["yDim"], max(len(rad), 1)) as ag:
        ag.upload(pos, rad)
        ag.dispatch(R, K, w["wrapX"], w["wrapY"])
        return ag.download()


def test_wells_equal_single_grid_handles(hal, oracle):
    rng = np.random.default_rng(40)
    wells, fields, srcs, counts, pos, rad = _mixed_wells(rng)
    ticks = 7
    with hal.Wells(wells) as b:
        for i, f in enumerate(fields):
            b.set_field(i, f)
            if srcs[i] is not None:
                b.set_source(i, srcs[i])
        b.set_agents(counts, np.concatenate(pos), np.concatenate(rad))
        b.run_ticks(3, R, K)
        b.run_ticks(ticks - 3, R, K)  # graphs of both parities
        got = [b.get_field(i) for i in range(len(wells))]
        forces = b.get_forces()
    at = 0
    for i, w in enumerate(wells):
        exp = _alone(hal, w, fields[i], srcs[i], ticks)
        assert np.array_equal(got[i], exp), (i, w)
        # the oracle, FP64 from the same float32 start
        mode = 1 if w["kind"] == "adi" else 0
        ref = oracle.run_ticks(mode, fields[i].astype(np.float64), w["xDim"], w["yDim"], w["diffRate"],
                               decay=w["decay"], src_dense=None if srcs[i] is None else srcs[i].astype(np.float64),
                               ticks=ticks, wrapX=w["wrapX"], wrapY=w["wrapY"])
        # FP32 against FP64: 1e-5 per explicit run; an ADI step's FP32 solve
        # error is up to 2e-6 (1 + r) of the field and accumulates per tick
        tol = 2e-6 * (1 + w["diffRate"]) * ticks if mode == 1 else 1e-5
        assert max_rel(got[i], ref) <= tol, (i, w)
        n = int(counts[i])
        v = forces[2 * at: 2 * (at + n)]
        at += n
        if n:
            assert np.array_equal(v, _alone_forces(hal, w, pos[i], rad[i])), (i, w)
            assert max_rel(v, _oracle_forces(oracle, w, pos[i], rad[i])) <= FORCE_TOL, (i, w)


def test_wells_bin_sizes_equal_single_grid_forces(hal):
    """Each well's bin size follows its agent capacity: one cell per bin for
    dense wells (whose force walk reads each window row as one run of bins),
    up to 8 x 8 cells for sparse ones.  Dense and sparse wells, with every
    wrap combination and clustered agents, give the forces of their own
    single-grid handles bit for bit."""
    rng = np.random.default_rng(41)
    specs = [  # xDim, yDim, kind, wrapX, wrapY, agents
        (40, 50, "explicit", True, False, 3000),    # 1 x 1 bins
        (64, 64, "adi", False, True, 5000),         # 1 x 1, y wraps: the general walk
        (70, 30, "explicit", True, True, 2500),     # 1 x 1
        (33, 47, "adi", False, False, 1200),        # 1 x 1, odd sides
        (300, 300, "adi", False, False, 1000),      # 8 x 8 bins
        (100, 300, "explicit", True, True, 400),    # 8 x 8, both wrap
        (90, 130, "explicit", False, True, 700),    # 4 x 4
    ]
    wells, pos, rad, counts = [], [], [], []
    for xd, yd, kind, wx, wy, na in specs:
        wells.append(dict(xDim=xd, yDim=yd, kind=kind, diffRate=0.2 if kind == "explicit" else 2.0, decay=0.0,
                          wrapX=wx, wrapY=wy, maxAgents=na))
        m = na // 3
        p = np.concatenate([rng.random((na - m, 2)) * (xd, yd),
                            np.array([xd, yd]) * 0.4 + rng.normal(0, 3.0, (m, 2))])
        hi = np.array([np.nextafter(np.float32(xd), np.float32(0)), np.nextafter(np.float32(yd), np.float32(0))])
        pos.append(np.clip(p, 0, hi).astype(np.float32).ravel())
        rad.append((0.3 + 0.4 * rng.random(na)).astype(np.float32))
        counts.append(na)
    with hal.Wells(wells) as b:
        for i, w in enumerate(wells):
            b.set_field(i, np.zeros(w["xDim"] * w["yDim"], np.float32))
        b.set_agents(np.array(counts, np.int32), np.concatenate(pos), np.concatenate(rad))
        b.run_ticks(1, R, K)
        forces = b.get_forces()
    at = 0
    for i, w in enumerate(wells):
        n = counts[i]
        v = forces[2 * at: 2 * (at + n)]
        at += n
        exp = _alone_forces(hal, w, pos[i], rad[i])
        assert np.abs(exp).max() > 0
        assert np.array_equal(v, exp), (i, w)


def test_autotune_keeps_state_and_results(hal):
    """The sweep-tile autotuner times the sweeps on the wells' own data
    without changing it, and whatever cap it picks, the ticks stay equal to
    the single-grid handles."""
    rng = np.random.default_rng(41)
    wells, fields, srcs, counts, pos, rad = _mixed_wells(rng)
    with hal.Wells(wells) as b:
        for i, f in enumerate(fields):
            b.set_field(i, f)
            if srcs[i] is not None:
                b.set_source(i, srcs[i])
        b.set_agents(counts, np.concatenate(pos), np.concatenate(rad))
        cap, ms_tuned, ms_default = b.autotune()
        assert cap in (8, 16, 32, 64, 128)
        assert 0 < ms_tuned <= ms_default
        assert all(np.array_equal(b.get_field(i), fields[i]) for i in range(len(wells)))
        b.run_ticks(4, R, K)
        b.autotune()  # re-tuning mid-run keeps the state too
        b.run_ticks(1, R, K)
        got = [b.get_field(i) for i in range(len(wells))]
    for i, w in enumerate(wells):
        assert np.array_equal(got[i], _alone(hal, w, fields[i], srcs[i], 5)), (i, w)


def test_wells_motion_equals_single_grid_steps(hal, oracle):
    """With motion on, every well's agents move tick after tick exactly as
    that well's agents do under the single-grid resident step."""
    rng = np.random.default_rng(42)
    wells, fields, srcs, counts, pos, rad = _mixed_wells(rng)
    vel = [((rng.random(2 * len(r)) - 0.5) * 0.4).astype(np.float32) for r in rad]
    ticks, fr, mv = 6, 0.7, 0.3
    with hal.Wells(wells) as b:
        for i, f in enumerate(fields):
            b.set_field(i, f)
        b.set_agents(counts, np.concatenate(pos), np.concatenate(rad))
        p0, v0 = b.get_agents()
        assert np.array_equal(p0, np.concatenate(pos)) and not v0.any()
        b.set_velocities(np.concatenate(vel))
        b.set_motion(True, fr, mv)
        b.run_ticks(ticks, R, K)
        got_p, got_v = b.get_agents()
        b.set_motion(False)
        b.run_ticks(1, R, K)  # forces only: the agents stay where they are
        assert np.array_equal(b.get_agents()[0], got_p)
    at = 0
    for i, w in enumerate(wells):
        n = int(counts[i])
        if n == 0:
            continue
        with hal.Agents(w["xDim"], w["yDim"], n) as ag:
            ag.upload(pos[i], rad[i])
            ag.set_velocities(vel[i])
            ag.step(ticks, R, K, w["wrapX"], w["wrapY"], friction=fr, maxVel=mv)
            ep, ev = ag.get_state()
        assert np.array_equal(got_p[2 * at: 2 * (at + n)], ep), (i, w)
        assert np.array_equal(got_v[2 * at: 2 * (at + n)], ev), (i, w)
        at += n


def test_wells_profile_and_source_clear(hal):
    rng = np.random.default_rng(41)
    wells, fields, srcs, counts, pos, rad = _mixed_wells(rng)
    with hal.Wells(wells) as b:
        for i, f in enumerate(fields):
            b.set_field(i, f)
            b.set_source(i, (rng.random(f.size) * 0.01).astype(np.float32))
            b.set_source(i, None)  # cleared again: plain decay and diffusion
        b.set_agents(counts, np.concatenate(pos), np.concatenate(rad))
        ms = b.profile(3, R, K)
        assert len(ms) == 5 and ms[4] > 0.0
        got = [b.get_field(i) for i in range(len(wells))]
    for i, w in enumerate(wells):
        assert np.array_equal(got[i], _alone(hal, w, fields[i], None, 3)), (i, w)


def test_wells_reject_bad_input(hal):
    with pytest.raises(ValueError):
        hal.Wells([dict(xDim=8, yDim=8, kind="explicit", diffRate=0.3, decay=0.0)])
    with pytest.raises(ValueError):
        hal.Wells([dict(xDim=hal.WELLS_MAX_SIDE + 1, yDim=8, kind="adi", diffRate=1.0, decay=0.0)])
    with pytest.raises(ValueError):
        hal.Wells([])
    with hal.Wells([dict(xDim=8, yDim=8, kind="adi", diffRate=1.0, decay=0.0, maxAgents=2)]) as b:
        with pytest.raises(ValueError):
            b.set_field(0, np.zeros(63, np.float32))
        with pytest.raises(ValueError):
            b.set_field(1, np.zeros(64, np.float32))
        with pytest.raises(ValueError):
            b.set_agents([3], np.zeros(6, np.float32), np.zeros(3, np.float32))
        with pytest.raises(ValueError):
            b.run_ticks(1, -1.0, 0.1)


def test_wells_batched_workload_sample(hal, oracle):
    """512 wells of the batched workload (109M cells, 5.2M agents): two
    ticks, and a sample of wells against the single-grid handles and the
    FP64 oracle (fields and forces)."""
    from halcuda import workloads

    w = workloads.wells_inputs()
    rng = np.random.default_rng(5)
    sample = sorted(rng.choice(len(w["wells"]), 8, replace=False).tolist())
    with hal.Wells(w["wells"]) as b:
        for i, f in enumerate(w["fields"]):
            b.set_field(i, f)
        b.set_agents(w["counts"], w["positions"], w["radii"])
        b.run_ticks(2, R, K)
        got = {i: b.get_field(i) for i in sample}
        forces = b.get_forces()
    starts = np.concatenate([[0], np.cumsum(w["counts"])])
    for i in sample:
        wd = w["wells"][i]
        wd = dict(wd, wrapX=False, wrapY=False)
        assert np.array_equal(got[i], _alone(hal, wd, w["fields"][i], None, 2)), i
        mode = 1 if wd["kind"] == "adi" else 0
        ref = oracle.run_ticks(mode, w["fields"][i].astype(np.float64), wd["xDim"], wd["yDim"], wd["diffRate"],
                               decay=wd["decay"], ticks=2, threads=8)
        tol = 2e-6 * (1 + wd["diffRate"]) * 2 if mode == 1 else 1e-5
        assert max_rel(got[i], ref) <= tol, i
        a, e = int(starts[i]), int(starts[i + 1])
        if e > a:
            p, rd = w["positions"][2 * a: 2 * e], w["radii"][a:e]
            exp = _alone_forces(hal, wd, p, rd)
            assert np.array_equal(forces[2 * a: 2 * e], exp), i
            assert max_rel(forces[2 * a: 2 * e], _oracle_forces(oracle, wd, p, rd)) <= FORCE_TOL, i
