"""bench.py's multi-process logic on CPU: world_size-2 gloo ranks.

bench.py runs one replica per GPU under torchrun (the path does not shard:
replicas only).  Its host logic is the job time, the maximum of the ranks'
timed milliseconds that every rank receives, the whole-job value (all
ranks' units over that time), and the reference arm, which rank 0 alone runs
while the other ranks exit 0 without work.  These tests run that logic in two
gloo processes; no GPU is involved.
"""
from __future__ import annotations

import importlib.util
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, local_ms, out_dir):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        bench = _bench()
        r, local, w = bench.dist_env()
        assert (r, local, w) == (rank, rank, world)
        dist.barrier()
        job_ms = bench.max_over_ranks(local_ms[rank], dist, device="cpu")
        value = bench.job_value(w, 1000.0, job_ms)
        with open(os.path.join(out_dir, f"rank{rank}.txt"), "w") as f:
            f.write(f"{job_ms!r} {value!r}\n")
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_job_time_is_the_max_over_ranks(tmp_path):
    port = _free_port()
    local_ms = [10.0, 12.5]
    mp.start_processes(_rank_main, args=(2, port, local_ms, str(tmp_path)), nprocs=2, join=True,
                       start_method="spawn")
    for rank in range(2):
        job_ms, value = (float(v) for v in (tmp_path / f"rank{rank}.txt").read_text().split())
        assert job_ms == 12.5
        # 2 replicas x 1000 units per step over the slowest rank's 12.5 ms
        assert value == pytest.approx(2 * 1000.0 / 12.5e-3)


def test_single_process_is_unchanged():
    bench = _bench()
    assert bench.max_over_ranks(7.25) == 7.25
    assert bench.job_value(1, 100.0, 2.0) == pytest.approx(100.0 / 2e-3)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch):
    """Under torchrun the reference arm's non-zero ranks exit 0 before any work
    (rank 0 alone times the CPU implementation and prints the line)."""
    bench = _bench()
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("LOCAL_RANK", "1")

    class Args:
        steps, warmup = 1, 3

    # the oracle is never built or run on this rank
    monkeypatch.setitem(sys.modules, "pyoracle", None)
    assert bench.run_reference(Args()) == 0
