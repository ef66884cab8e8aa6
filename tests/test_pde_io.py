"""PDEGrid2D's on-disk format (SavePDEGrid2D / LoadPDEGrid2D).

The write / read calls of the library are host code, so the format checks
run without a GPU: against a file the reference's own SavePDEGrid2D wrote
(tests/golden/pdegrid2d_13x7.bin, made by tests/golden/make_golden.py) and,
where the reference tree is present, both ways through the reference's
loader and writer.  Save / load of the resident handles is marked gpu.
"""
from __future__ import annotations

import os

import numpy as np
import pytest

import pyoracle

GOLDEN_FILE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "pdegrid2d_13x7.bin")


@pytest.fixture(scope="module")
def halio():
    """The library's host-only calls; builds libhal_cuda.so if it is missing."""
    import subprocess
    import sys

    import halcuda

    if not os.path.exists(halcuda.LIB_PATH):
        root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
        subprocess.run([sys.executable, os.path.join(root, "hal-cpp_gb300", "build.py")], check=True)
    halcuda.lib()
    return halcuda


def _golden_state():
    rng = np.random.default_rng(7171)
    f = rng.random(13 * 7)
    d = (rng.random(13 * 7) - 0.5) * 1e-3
    return f, d


def test_reads_a_file_the_reference_wrote(halio):
    g = halio.pdegrid2d_read(GOLDEN_FILE)
    f, d = _golden_state()
    assert (g["xDim"], g["yDim"], g["wrapX"], g["wrapY"], g["updateCt"]) == (13, 7, True, False, 42)
    assert np.array_equal(g["field"], f) and np.array_equal(g["deltas"], d)


def test_writes_the_reference_bytes(halio, tmp_path):
    f, d = _golden_state()
    out = tmp_path / "ours.bin"
    halio.pdegrid2d_write(out, 13, 7, True, False, 42, f, d)
    assert out.read_bytes() == open(GOLDEN_FILE, "rb").read()
    # layout: 14-byte header, then field, then deltas
    raw = out.read_bytes()
    assert len(raw) == 14 + 16 * 91
    assert np.array_equal(np.frombuffer(raw[14:14 + 8 * 91], dtype="<f8"), f)


def test_zero_deltas_and_header_fields(halio, tmp_path):
    out = tmp_path / "z.bin"
    f = np.arange(6, dtype=np.float64)
    halio.pdegrid2d_write(out, 2, 3, False, True, -5, f)
    g = halio.pdegrid2d_read(out)
    assert (g["xDim"], g["yDim"], g["wrapX"], g["wrapY"], g["updateCt"]) == (2, 3, False, True, -5)
    assert np.array_equal(g["field"], f) and not g["deltas"].any()


def test_rejects_bad_files(halio, tmp_path):
    raw = open(GOLDEN_FILE, "rb").read()
    short = tmp_path / "short.bin"
    short.write_bytes(raw[:-8])  # one double missing
    with pytest.raises(ValueError):
        halio.pdegrid2d_read(short)
    header_only = tmp_path / "hdr.bin"
    header_only.write_bytes(raw[:10])  # cut inside the header
    with pytest.raises(ValueError):
        halio.pdegrid2d_read(header_only)
    bad = tmp_path / "bad.bin"
    bad.write_bytes(np.int32(0).tobytes() + raw[4:])  # xDim = 0
    with pytest.raises(ValueError):
        halio.pdegrid2d_read(bad)
    huge = tmp_path / "huge.bin"
    huge.write_bytes(np.int32(1 << 16).tobytes() + np.int32(1 << 16).tobytes() + raw[8:])  # 2^32 cells
    with pytest.raises(ValueError):
        halio.pdegrid2d_read(huge)
    with pytest.raises(ValueError):
        halio.pdegrid2d_read(tmp_path / "missing.bin")
    with pytest.raises(ValueError):
        halio.pdegrid2d_write(tmp_path / "x.bin", 0, 3, False, False, 0, np.zeros(0))


@pytest.mark.skipif(not os.path.isdir(pyoracle.REF_TREE), reason="reference tree not present")
def test_round_trips_through_the_reference(halio, tmp_path):
    pyoracle.build(ref=True)
    R = pyoracle.Reference
    rng = np.random.default_rng(3)
    for xd, yd, wx, wy in ((1, 1, 0, 0), (5, 64, 1, 1), (40, 3, 0, 1)):
        f, d = rng.standard_normal(xd * yd), rng.standard_normal(xd * yd)
        ours = tmp_path / f"o{xd}.bin"
        halio.pdegrid2d_write(ours, xd, yd, wx, wy, 7, f, d)
        got = R.pdegrid2d_load(ours)
        assert got[:5] == (xd, yd, bool(wx), bool(wy), 7)
        assert np.array_equal(got[5], f) and np.array_equal(got[6], d)
        theirs = tmp_path / f"r{xd}.bin"
        R.pdegrid2d_save(theirs, xd, yd, wx, wy, 9, f, d)
        assert theirs.read_bytes()[14:] == ours.read_bytes()[14:]
        g = halio.pdegrid2d_read(theirs)
        assert g["updateCt"] == 9 and np.array_equal(g["field"], f) and np.array_equal(g["deltas"], d)


@pytest.mark.gpu
def test_resident_save_and_resume(hal, oracle, tmp_path):
    """Checkpoint after 20 ticks, resume in a new handle, 20 more: the same
    field as 40 ticks straight through, for the explicit and the ADI tick."""
    n = 96
    rng = np.random.default_rng(5)
    f0 = rng.random(n * n).astype(np.float32)
    for cls, r in ((hal.Diffusion, 0.2), (hal.Adi, 3.0)):
        with cls(n, n) as a:
            a.set_field(f0)
            a.run_ticks(40, r, 0.01, True, False)
            straight = a.get_field()
        path = tmp_path / f"{cls.__name__}.bin"
        with cls(n, n) as a:
            a.set_field(f0)
            a.run_ticks(20, r, 0.01, True, False)
            a.save(path, True, False, 20)
        g = hal.pdegrid2d_read(path)
        assert (g["wrapX"], g["wrapY"], g["updateCt"]) == (True, False, 20) and not g["deltas"].any()
        with cls(n, n) as b:
            assert b.load(path) == (True, False, 20)
            b.run_ticks(20, r, 0.01, True, False)
            assert np.array_equal(b.get_field(), straight)
        with cls(n + 1, n) as c, pytest.raises(ValueError):
            c.load(path)
    pending = tmp_path / "pending.bin"
    hal.pdegrid2d_write(pending, n, n, 0, 0, 3, f0, np.full(n * n, 1e-3))
    with hal.Diffusion(n, n) as a:
        with pytest.raises(RuntimeError):
            a.load(pending)
