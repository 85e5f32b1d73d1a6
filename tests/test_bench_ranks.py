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
        specs, _ = bench.island_specs(rank)
        seeds = sorted({s.seed for s in specs})
        Path(out_dir, f"r{rank}.txt").write_text(f"{got} {seeds[0]} {len(seeds)}")
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
    assert r0[1] != r1[1]                           # independent replicas: different Philox seeds
    assert r0[2] == r1[2] == "1"                    # one seed per rank (islands differ by row index)


def test_single_rank_is_identity():
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.max_over_ranks(3.5, "cpu", 1) == 3.5
