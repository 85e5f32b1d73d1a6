"""The island ring split over ranks (speo_gb300.ring), on CPU ranks under gloo.

Two ranks each hold a contiguous block of the ring in their own buffer and run their islands'
generations (the oracle's restatement, row numbers local to the block); migrations go through
RingBlock: the ring kernel on local rings plus one point-to-point message per rank. The result
must equal, row for row and bit for bit, the same generations with the ring migration of the
single-buffer ring over all islands (speo_ring_migrate's semantics), over several epochs.
"""
from __future__ import annotations

import os
import socket
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
N_LOCAL, P, D, LD, K, EPOCHS, GENS = 4, 16, 5, 8, 3, 4, 3


def _segments(block: int, world_rows_offset: int = 0):
    """The oracle segments of one block, row numbers local to its buffer."""
    from speo_gb300.instances import make_instance

    segs = []
    for j in range(N_LOCAL):
        isl = block * N_LOCAL + j
        o, M = make_instance(900 + isl, D)
        segs.append(dict(row0=j * P + world_rows_offset, P=P, D=D, ld=LD, func=9, strategy=4, F=0.5, CR=0.9,
                         lb=-100.0, ub=100.0, o=o, M=M, seed=3000 + isl))
    return segs


def _init_block(oracle, block: int, extra: int):
    segs = _segments(block)
    pop = np.zeros((N_LOCAL * P + extra, LD), dtype=np.float32)
    fit = np.zeros(N_LOCAL * P + extra, dtype=np.float32)
    for s in segs:
        rows = oracle.init_population(P, LD, D, s["lb"], s["ub"], s["seed"], row0=s["row0"])
        pop[s["row0"]:s["row0"] + P] = rows
        fit[s["row0"]:s["row0"] + P] = oracle.evaluate_rows(9, rows, D, s["o"], s["M"]).astype(np.float32)
    return segs, pop, fit


def _generations(oracle, segs, pop, fit, g0):
    n = N_LOCAL * P
    for g in range(GENS):
        p_out, f_out, _, _, err = oracle.generation(segs, g0 + g, pop[:n], fit[:n])
        assert err == 0
        pop[:n], fit[:n] = p_out, f_out


def _rank_main(rank: int, world: int, port: int, out_dir: str) -> None:
    import torch.distributed as dist

    for p in (str(ROOT / "speo-gpu-single-control_gb300"), str(ROOT / "oracle")):
        sys.path.insert(0, p)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import speo_oracle
        from speo_gb300.ring import HostRingOps, RingBlock

        blk = RingBlock(N_LOCAL, P, D, LD, K, rank, world)
        segs, pop, fit = _init_block(speo_oracle, rank, 2 * K)
        ops = HostRingOps(speo_oracle)
        for e in range(EPOCHS):
            _generations(speo_oracle, segs, pop, fit, e * GENS)
            blk.migrate(ops, pop, fit)
        np.savez(Path(out_dir, f"r{rank}.npz"), pop=pop[:N_LOCAL * P], fit=fit[:N_LOCAL * P])
        dist.barrier()
    finally:
        dist.destroy_process_group()


def _single_buffer_reference(oracle, world: int, isolated: bool = False):
    """The same generations with the ring over all islands (isolated: each block its own ring)."""
    blocks = [_init_block(oracle, b, 0) for b in range(world)]
    n = N_LOCAL * P
    N = N_LOCAL * world
    if isolated:
        ring = [dict(row0=i * P, P=P, D=D, ld=LD, ring_next=(i // N_LOCAL) * N_LOCAL + (i + 1) % N_LOCAL)
                for i in range(N)]
    else:
        ring = [dict(row0=i * P, P=P, D=D, ld=LD, ring_next=(i + 1) % N) for i in range(N)]
    for e in range(EPOCHS):
        for segs, pop, fit in blocks:
            _generations(oracle, segs, pop, fit, e * GENS)
        allp = np.concatenate([b[1] for b in blocks])
        allf = np.concatenate([b[2] for b in blocks])
        oracle.ring_migrate(ring, K, allp, allf)
        for b, (segs, pop, fit) in enumerate(blocks):
            pop[:] = allp[b * n:(b + 1) * n]
            fit[:] = allf[b * n:(b + 1) * n]
    return blocks


def test_two_rank_ring_equals_the_single_buffer_ring(tmp_path, oracle):
    import torch.multiprocessing as mp

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    ref = _single_buffer_reference(oracle, 2)
    iso = _single_buffer_reference(oracle, 2, isolated=True)
    differs = False
    for r in range(2):
        got = np.load(Path(tmp_path, f"r{r}.npz"))
        _, pop, fit = ref[r]
        assert np.array_equal(got["fit"], fit), f"rank {r} fitness"
        assert np.array_equal(got["pop"], pop), f"rank {r} rows"
        differs |= not np.array_equal(got["pop"], iso[r][1])
    assert differs   # the rows that crossed ranks changed the run


def test_one_rank_block_is_the_local_ring(oracle):
    """world = 1: RingBlock's migration is the plain ring over the block."""
    sys.path.insert(0, str(ROOT / "speo-gpu-single-control_gb300"))
    from speo_gb300.ring import HostRingOps, RingBlock

    segs, pop, fit = _init_block(oracle, 0, 2 * K)
    _generations(oracle, segs, pop, fit, 0)
    a_pop, a_fit = pop.copy(), fit.copy()
    RingBlock(N_LOCAL, P, D, LD, K, 0, 1).migrate(HostRingOps(oracle), pop, fit)
    ring = [dict(row0=i * P, P=P, D=D, ld=LD, ring_next=(i + 1) % N_LOCAL) for i in range(N_LOCAL)]
    oracle.ring_migrate(ring, K, a_pop, a_fit)
    assert np.array_equal(pop, a_pop) and np.array_equal(fit, a_fit)
