"""The multi-GPU mode is replicas only: every rank runs its own copy of the
workload, no data moves between ranks, and the job's time is the slowest
rank's.  These CPU tests run bench.py's aggregation on 2 gloo ranks and
check that the reference arm does its work on rank 0 alone."""
from __future__ import annotations

import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out_dir: str) -> None:
    import torch.distributed as td

    sys.path.insert(0, str(ROOT))
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    td.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = 10.0 + 5.0 * rank                       # rank 1 is the slower one
        worst = bench.worst_over_ranks(ms, td)
        value = bench.replica_mlups(world, 1000, 50, worst)
        Path(out_dir, f"rank{rank}.txt").write_text(f"{worst} {value}")
    finally:
        td.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time(tmp_path):
    torch = pytest.importorskip("torch")
    world, port = 2, _free_port()
    torch.multiprocessing.spawn(_rank_main, args=(world, port, str(tmp_path)), nprocs=world, join=True)
    for r in range(world):
        worst, value = (float(v) for v in (tmp_path / f"rank{r}.txt").read_text().split())
        assert worst == 15.0
        assert value == pytest.approx(2 * 1000 * 50 / 15e-3 / 1e6)


def test_single_process_needs_no_collective():
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.worst_over_ranks(12.5, None) == 12.5
    assert bench.replica_mlups(1, 8, 2, 1.0) == pytest.approx(8 * 2 / 1e-3 / 1e6)


def test_reference_arm_runs_on_rank_zero_only(capsys):
    """under torchrun the reference arm's other ranks leave without work"""
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.reference_arm(None, 2, 1) is None
    assert capsys.readouterr().out == ""
