"""The device-resident PDEGrid2D (hal_cuda_pdegrid) against the reference.

Hal::PDEGrid2D (include/Hal/Grids/PDEGrid2D.h) is what HAL models call each
tick: per-cell Set/Add/Mul/Scale between the PDE operators, then Update.  The
handle keeps the field and the deltas on the device in FP64 and must reproduce
every call bit for bit:

* whole call sequences written by the reference's own PDEGrid2D
  (tests/golden/pdegrid.npz) replayed through the C ABI, the per-cell
  operations sent one call each and, separately, batched into one list
  between operators: final field, deltas, update count and every query
  result equal (GetAvg within the reference's own summation error bound,
  n * eps relative: a parallel sum);
* random sequences on larger grids against the oracle (which is pinned to the
  reference by tests/test_oracle_pin.py), explicit and ADI diffusion on one
  field, every boundary kind;
* the FP64 ADI step alone at 1024^2 against the oracle;
* per-agent operations from an agent handle's binning (Mul(Isq(), -uptake) of
  examples/CompetitiveRelease.cpp:147) against the same operations as a list
  in agent index order.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CELL_OPS = {"set": 0, "add": 1, "mul": 2, "scale": 3}


def run_on_device(hal, grid, script, batch):
    """Replays a PDEScript through the handle; returns the query records.
    batch sends consecutive per-cell operations as one list."""
    records = []
    pending = []

    def flush():
        if pending:
            ops, cells, vals = zip(*pending)
            grid.apply(np.array(cells), np.array(vals), ops=np.array(ops))
            pending.clear()

    for name, a in script.calls:
        if name in CELL_OPS:
            if batch:
                pending.append((CELL_OPS[name], a["i"], a["d0"]))
            else:
                grid.apply([a["i"]], [a["d0"]], op=CELL_OPS[name])
            continue
        flush()
        arr = a["arrays"]
        if name in ("set_all", "add_all", "mul_all"):
            grid.apply_all({"set_all": 0, "add_all": 1, "mul_all": 2}[name], a["d0"])
        elif name == "set_all_values":
            grid.apply_all(0, per_cell=arr[0])
        elif name == "diffusion":
            grid.diffusion(a["d0"])
        elif name == "diffusion_bc":
            grid.diffusion(a["d0"], ghost=arr[0])
        elif name == "diffusion_var":
            grid.diffusion_var(arr[0], arr[1])
        elif name == "adi":
            grid.diffusion_adi(a["d0"])
        elif name == "adi_bc":
            grid.diffusion_adi(a["d0"], ghost=arr[0])
        elif name == "advection":
            grid.advection(a["d0"], a["d1"])
        elif name == "advection_bc":
            grid.advection(a["d0"], a["d1"], ghost=arr[0])
        elif name == "advection_var":
            grid.advection_var(arr[0], arr[1])
        elif name == "advection_var_bc":
            grid.advection_var(arr[0], arr[1], arr[2], arr[3], arr[4])
        elif name == "update":
            grid.update()
        elif name == "set_non_negative":
            grid.set_non_negative()
        elif name == "get":
            records.append(grid.get_cells([a["i"]])[0])
        elif name in ("max", "min", "avg", "max_delta"):
            records.append(grid.stats()[{"max": 0, "min": 1, "avg": 2, "max_delta": 3}[name]])
        elif name == "max_delta_scaled":
            records.append(grid.stats(a["d0"])[4])
        elif name.startswith("gradient"):
            bc = a["d0"] if name.endswith("_bc") else None
            gx, gy = grid.gradient([a["x"]], [a["y"]], boundary=bc)
            records.append((gx if name.startswith("gradient_x") else gy)[0])
        else:
            raise AssertionError(name)
    flush()
    return np.array(records)


def _avg_positions(script):
    return [k for k, (name, _) in enumerate(c for c in script.calls if c[0] in (
        "get", "max", "min", "avg", "max_delta", "max_delta_scaled", "gradient_x", "gradient_y", "gradient_x_bc",
        "gradient_y_bc")) if name == "avg"]


def _check_records(got, exp, script):
    """Every query bit-exact, except GetAvg: the reference sums the n cells
    one after another, whose rounding error is bounded by n * eps relative
    (the device's blocked sum is more accurate than that)."""
    avg = _avg_positions(script)
    exact = np.ones(exp.size, bool)
    exact[avg] = False
    assert np.array_equal(got[exact], exp[exact])
    if avg:
        n = script.xDim * script.yDim
        assert np.allclose(got[avg], exp[avg], rtol=n * np.finfo(np.float64).eps, atol=0)


@pytest.mark.parametrize("batch", [False, True])
def test_pdegrid_scripts_golden(hal, golden, batch):
    from pyoracle import PDEScript

    g = golden("pdegrid")
    for k in range(int(g["count"][0])):
        xd, yd, wx, wy = (int(v) for v in g[f"c{k}_dims"])
        sc = PDEScript.from_encoded(xd, yd, wx, wy, g[f"c{k}_ops"], g[f"c{k}_iargs"], g[f"c{k}_dargs"],
                                    g[f"c{k}_arrays"])
        with hal.PDEGrid(xd, yd, wx, wy) as grid:
            grid.set_state(g[f"c{k}_f0"], g[f"c{k}_d0"], 7)
            rec = run_on_device(hal, grid, sc, batch)
            f, d, uc = grid.get_state()
        assert np.array_equal(f, g[f"c{k}_field"]), k
        assert np.array_equal(d, g[f"c{k}_deltas"]), k
        assert uc == int(g[f"c{k}_uc"][0])
        _check_records(rec, g[f"c{k}_records"], sc)


@pytest.mark.parametrize("xd,yd,wx,wy", [(200, 150, 0, 0), (128, 257, 1, 1), (300, 64, 1, 0), (96, 512, 0, 1)])
def test_pdegrid_random_scripts_against_oracle(hal, oracle, xd, yd, wx, wy):
    import importlib.util
    import os

    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(os.path.dirname(__file__), "golden",
                                                                             "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    rng = np.random.default_rng(xd + 7 * yd + wx + 2 * wy)
    sc = mg.pdegrid_script(rng, xd, yd, wx, wy, cells_per_tick=200)
    f0 = rng.random(xd * yd)
    ef, ed, euc, erec = oracle.pdegrid_script(sc, f0)
    with hal.PDEGrid(xd, yd, wx, wy) as grid:
        grid.set_state(f0)
        rec = run_on_device(hal, grid, sc, batch=True)
        f, d, uc = grid.get_state()
    assert np.array_equal(f, ef) and np.array_equal(d, ed) and uc == euc
    _check_records(rec, erec, sc)


@pytest.mark.parametrize("wx,wy,dirichlet", [(0, 0, False), (1, 1, False), (0, 1, True), (1, 0, True)])
def test_pdegrid_adi_1024_bit_exact(hal, oracle, wx, wy, dirichlet):
    from pyoracle import PDEScript

    n = 1024
    rng = np.random.default_rng(3 + wx + 2 * wy + 4 * dirichlet)
    f0 = rng.random(n * n)
    ghost = rng.random(4 * n) if dirichlet else None
    sc = PDEScript(n, n, wx, wy)
    sc.add("adi_bc" if dirichlet else "adi", d0=5.0, arrays=[ghost] if dirichlet else None)
    ef, ed, _, _ = oracle.pdegrid_script(sc, f0)
    with hal.PDEGrid(n, n, wx, wy) as grid:
        grid.set_state(f0)
        grid.diffusion_adi(5.0, ghost=ghost)
        f, d, _ = grid.get_state()
    assert np.array_equal(f, ef)
    assert np.array_equal(d, ed)
    assert np.abs(d).max() > 0


@pytest.mark.parametrize("batch", [False, True])
def test_pdegrid_deferred_all_calls(hal, oracle, batch):
    """A value-form SetAll / AddAll / MulAll runs inside the next Update's
    pass, or before any other call: sequences that follow it with another
    *All, a per-cell list, a query of the deltas, an operator, a per-cell
    *All, a stream change or the Update itself equal the reference's calls
    one by one."""
    from pyoracle import PDEScript

    xd, yd = 97, 130
    rng = np.random.default_rng(31)
    f0 = rng.random(xd * yd)
    sc = PDEScript(xd, yd)
    sc.add("mul_all", d0=-0.01).add("update")
    sc.add("mul_all", d0=-0.02).add("add_all", d0=0.003).add("update")
    sc.add("add_all", d0=0.01).add("max_delta").add("max_delta_scaled", d0=0.5).add("update")
    sc.add("set_all", d0=0.25).add("get", i=17).add("set", i=5, d0=0.9).add("update")
    sc.add("mul_all", d0=-0.05).add("diffusion", d0=0.1).add("update")
    sc.add("mul_all", d0=-0.03).add("set_all_values", arrays=[rng.random(xd * yd)]).add("update")
    sc.add("mul_all", d0=-0.04).add("adi", d0=2.0).add("mul_all", d0=0.5).add("update").add("max").add("avg")
    ef, ed, euc, erec = oracle.pdegrid_script(sc, f0)
    with hal.PDEGrid(xd, yd) as grid:
        grid.set_state(f0)
        rec = run_on_device(hal, grid, sc, batch)
        grid.apply_all(2, -0.07)
        grid.set_stream(None)
        f1, d1, _ = grid.get_state()
        f, d, uc = grid.get_state()
    # the trailing MulAll is pending until get_state runs it
    assert np.array_equal(f, ef) and np.array_equal(d1, ed + ef * -0.07) and uc == euc
    _check_records(rec, erec, sc)


def _plan_diagonals(r, n=64, end_adjust=-1.0):
    """TdmaSolver::TDMA's modified diagonal of a line's ADI matrix
    (off-diagonal -r/2, diagonal 1 - w * off, w = 2 + end_adjust at the
    ends), in its operations."""
    off = -r / 2.0
    b = np.empty(n)
    for i in range(n):
        w = 2.0 + (end_adjust if i == 0 else 0.0) + (end_adjust if i == n - 1 else 0.0)
        b[i] = 1 - w * off
        if i > 0:
            b[i] = b[i] - (off / b[i - 1]) * off
    return b


def test_adi_plan_division_matches_ieee(hal):
    """The FP64 ADI's back substitution divides through the diagonal's
    reciprocal (a double-word and one Markstein correction).  Its quotients
    must equal IEEE division bit for bit: for numerators in the sweeps'
    ranges, random bit patterns, signed zeros, subnormals, huge values,
    infinities and NaN (for -0 and nonzero numerators outside [2^-900,
    2^900) the sweeps solve the line again with IEEE divisions), and for
    divisors from the plans' diagonals and across [2^-20, 2^20]."""
    rng = np.random.default_rng(11)
    m = 1 << 17
    special = np.array([0.0, -0.0, 5e-324, -5e-324, 2.2250738585072014e-308, np.inf, -np.inf, np.nan,
                        1.7976931348623157e308, -1.7976931348623157e308, np.ldexp(1.0, -900),
                        np.ldexp(1.0, -900) * (1 - 2.0 ** -53), np.ldexp(1.0, 900), np.ldexp(1.0, 900) * (1 - 2.0 ** -53)])
    num = np.concatenate([
        rng.random(m) - 0.5,
        rng.random(m) * 10.0,
        np.ldexp(rng.random(m) + 0.5, rng.integers(-1000, 1000, m)) * rng.choice([-1.0, 1.0], m),
        rng.integers(0, np.iinfo(np.uint64).max, m, dtype=np.uint64, endpoint=True).view(np.float64),
        special,
    ])
    den = np.concatenate([
        _plan_diagonals(0.1), _plan_diagonals(5.0), _plan_diagonals(5.0, end_adjust=1.0), _plan_diagonals(300.0),
        np.ldexp(rng.random(32) + 1.0, rng.integers(-20, 20, 32)),
        [1.0, 2.0 ** -20, 2.0 ** 20, 3.0, 1.0 + 2.0 ** -52],
    ])
    assert hal.check_plan_division(num, den) == 0
    for bad in (2.0 ** 21, -1.0, 0.0):
        with pytest.raises(ValueError):
            hal.check_plan_division(num[:4], np.array([bad]))


@pytest.mark.parametrize("wx,wy,dirichlet", [(0, 0, False), (1, 0, False), (0, 1, True)])
def test_pdegrid_adi_extreme_values_bit_exact(hal, oracle, wx, wy, dirichlet):
    """DiffusionADI on a field with a zero region, negative zeros, values
    below 2^-900 and above 2^900 (the sweeps' fast division does not cover
    those numerators; their lines are solved again with IEEE divisions)
    equals the CPU's bit for bit, signs of zero included."""
    from pyoracle import PDEScript

    xd, yd = 300, 200
    rng = np.random.default_rng(21 + wx + 2 * wy)
    f0 = rng.random((xd, yd))
    f0[:, :60] = 0.0
    f0[100:140, 60:80] = -0.0
    f0[150:170, :] = rng.random((20, yd)) * 1e-300
    f0[200:205, 100:150] = 1e280
    f0 = f0.ravel()
    ghost = np.where(rng.random(2 * (xd + yd)) < 0.5, 0.0, rng.random(2 * (xd + yd))) if dirichlet else None
    sc = PDEScript(xd, yd, wx, wy)
    sc.add("adi_bc" if dirichlet else "adi", d0=3.0, arrays=[ghost] if dirichlet else None)
    ef, ed, _, _ = oracle.pdegrid_script(sc, f0)
    with hal.PDEGrid(xd, yd, wx, wy) as grid:
        grid.set_state(f0)
        grid.diffusion_adi(3.0, ghost=ghost)
        f, d, _ = grid.get_state()
    assert np.array_equal(f.view(np.uint64), ef.view(np.uint64))
    assert np.array_equal(d.view(np.uint64), ed.view(np.uint64))


def test_pdegrid_agent_operations(hal, oracle):
    """Each agent's Mul(Isq(), -uptake) from the agent handle's binning,
    and per-agent Add values, equal the same operations as a list in agent
    index order (the order a model's loop over its agents would apply)."""
    from pyoracle import PDEScript

    xd, yd, n = 120, 90, 30000
    rng = np.random.default_rng(8)
    pos = np.stack([rng.random(n) * xd, 45 + rng.normal(0, 8, n)], 1)
    pos = np.clip(pos, 0, np.array([xd, yd]) * (1 - 1e-6)).astype(np.float32).ravel()
    rad = np.full(n, 0.5, np.float32)
    per = rng.random(n) * 1e-3
    f0 = rng.random(xd * yd)
    cx = np.minimum(np.floor(pos[0::2]).astype(np.int64), xd - 1)
    cy = np.minimum(np.floor(pos[1::2]).astype(np.int64), yd - 1)
    cells = (cx * yd + cy).astype(np.int32)
    sc = PDEScript(xd, yd)
    for c in cells:
        sc.add("mul", i=int(c), d0=-0.03)
    for c, v in zip(cells, per):
        sc.add("add", i=int(c), d0=float(v))
    sc.add("update")
    ef, ed, _, _ = oracle.pdegrid_script(sc, f0)
    with hal.Agents(xd, yd, n) as ag, hal.PDEGrid(xd, yd) as grid:
        ag.upload(pos, rad)
        ag.dispatch(1.0, 0.1)
        grid.set_state(f0)
        grid.apply_agents(ag, hal.CELL_MUL, -0.03)
        grid.apply_agents(ag, hal.CELL_ADD, per_agent=per)
        grid.update()
        f, d, uc = grid.get_state()
    assert np.array_equal(f, ef) and np.array_equal(d, ed) and uc == 1


def test_pdegrid_rejections(hal):
    with hal.PDEGrid(8, 6) as grid:
        with pytest.raises(ValueError, match="Diffusion rate above stable maximum value of 0.25"):
            grid.diffusion(0.3)
        with pytest.raises(ValueError, match="Advection rate component sum above stable maximum value of 0.5"):
            grid.advection(0.3, 0.3)
        with pytest.raises(ValueError, match="outside the grid"):
            grid.apply([48], [1.0], op=hal.CELL_ADD)
        with pytest.raises(ValueError, match="unknown operation"):
            grid.apply([1], [1.0], op=9)
        with pytest.raises(ValueError, match="outside the grid"):
            grid.gradient([8], [0])
        with hal.Agents(9, 6, 4) as ag:
            with pytest.raises(ValueError, match="differs from the field"):
                grid.apply_agents(ag, hal.CELL_MUL, -0.1)
