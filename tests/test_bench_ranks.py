"""CPU tests of the benchmark's multi-rank logic on the gloo backend (world size 2): the reported
time is the slowest rank's, and each rank runs its own replica of the island ring."""
from __future__ import annotations

import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _rank_main(rank: int, world: int, port: int, out_dir: str) -> None:
    import torch
    import torch.distributed as dist

    sys.path.insert(0, str(ROOT))
    sys.path.insert(0, str(ROOT / "speo-gpu-single-control_gb300"))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench

        got = bench.max_over_ranks(10.0 + 5.0 * rank, "cpu", world)
        from speo_gb300 import workloads

        specs, _ = workloads.config4_specs(bench.FUNC, rank=rank)
        seeds = sorted({s.seed for s in specs})
        Path(out_dir, f"r{rank}.txt").write_text(f"{got} {' '.join(map(str, seeds))}")
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_time_is_max_over_ranks_and_replicas_differ(tmp_path):
    import socket

    import torch.multiprocessing as mp

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    r0 = Path(tmp_path, "r0.txt").read_text().split()
    r1 = Path(tmp_path, "r1.txt").read_text().split()
    assert float(r0[0]) == float(r1[0]) == 15.0     # both ranks report the slowest rank's time
    s0, s1 = set(r0[1:]), set(r1[1:])
    assert len(s0) == len(s1) == 128                # one Philox seed per island
    assert not (s0 & s1)                            # independent replicas: no seed shared between ranks


def test_single_rank_is_identity():
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.max_over_ranks(3.5, "cpu", 1) == 3.5


def test_timed_generations_are_exactly_the_requested_steps():
    """bench.chunks splits any step count at the migration points (every 50 generations counted
    from the start of the run, warm-up included) and covers it exactly."""
    sys.path.insert(0, str(ROOT))
    import bench

    for done, n in ((0, 20), (5, 20), (0, 50), (45, 7), (5, 1000), (0, 1), (49, 1), (50, 123)):
        parts = list(bench.chunks(done, n))
        assert sum(k for k, _ in parts) == n
        pos = done
        for k, mig in parts:
            assert 1 <= k <= 50 and (pos % 50) + k <= 50
            pos += k
            assert mig == (pos % 50 == 0)
