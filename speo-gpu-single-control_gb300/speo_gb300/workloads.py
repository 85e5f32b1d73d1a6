"""The benchmark configurations as segment tables (seeded synthetic instances).

  config 1  island model: 64 islands x P=100, D=30, rotated Rastrigin, ring best-5 -> worst-5
            every 50 generations
  config 2  precision: 256 islands x P=128, D=100, per island a seeded choice of rotated sphere /
            rotated Rastrigin with its own o and M; tensor-core split-FP16 evaluation, FP64 re-check
  config 3  batched uneven runs: 1024 independent runs, D ~ U{10,30,50,100}, P ~ U[50,200],
            each with its own o, M and objective; one launch per generation
  config 4  learned surrogate: 128 islands x P=256, D=50, rotated Rastrigin; MLP 50-256-256-1
            screening k=8 trials per target, archive 2^20, Adam lr 1e-3, batch 4096

Seeds follow the reference's run seed (node + fid)(run + fid) (src/main.cc:138).
"""
from __future__ import annotations

import numpy as np

from . import _lib
from .device import SegmentSpec, SegmentTable
from .instances import make_instance, run_seed

SPHERE, RASTRIGIN = _lib.FUNC_ROTATED_SPHERE, _lib.FUNC_ROTATED_RASTRIGIN


def config1_specs(rank: int = 0):
    seed = run_seed(1, RASTRIGIN, 1)
    inst = [make_instance(seed, 30)]
    specs = [SegmentSpec(pop_size=100, dim=30, func_id=RASTRIGIN, instance=0, seed=seed * 1000003 + rank,
                         ring_next=(i + 1) % 64) for i in range(64)]
    return specs, inst


def config2_specs(n_islands: int = 256):
    rng = np.random.default_rng(run_seed(1, 2, 1))
    specs, inst = [], []
    for i in range(n_islands):
        func = SPHERE if rng.integers(0, 2) == 0 else RASTRIGIN
        inst.append(make_instance(run_seed(1, func, 1) * 7919 + i, 100))
        specs.append(SegmentSpec(pop_size=128, dim=100, func_id=func, instance=i, seed=1000 + i))
    return specs, inst


def config3_specs(n_runs: int = 1024):
    rng = np.random.default_rng(run_seed(1, 3, 1))
    specs, inst = [], []
    for i in range(n_runs):
        D = int(rng.choice([10, 30, 50, 100]))
        P = int(rng.integers(50, 201))
        func = SPHERE if rng.integers(0, 2) == 0 else RASTRIGIN
        inst.append(make_instance(run_seed(1, func, i + 1), D))
        specs.append(SegmentSpec(pop_size=P, dim=D, func_id=func, instance=i, seed=5000 + i))
    return specs, inst


def config4_specs(func: int = RASTRIGIN, rank: int = 0):
    """Config 4's islands; `func` = SPHERE gives the same shape on the rotated sphere, where an
    error of 1e-8 is reachable and the evaluations needed to get there can be compared. `rank`
    gives an independent replica of the ring (its own Philox seeds, the same instance)."""
    seed = run_seed(1, func, 4)
    inst = [make_instance(seed, 50)]
    specs = [SegmentSpec(pop_size=256, dim=50, func_id=func, instance=0, seed=seed * 31 + i + 1000003 * rank,
                         ring_next=(i + 1) % 128) for i in range(128)]
    return specs, inst


def config4_uneven_specs(func: int = RASTRIGIN, rank: int = 0):
    """Config 4's instance on 144 islands of uneven size (P uniform in [160, 256], seeded; about
    30k rows, one island per SM): the screened and plain generations over islands of different
    sizes in one table."""
    seed = run_seed(1, func, 4)
    inst = [make_instance(seed, 50)]
    sizes = np.random.default_rng(seed + 77).integers(160, 257, 144)
    specs = [SegmentSpec(pop_size=int(sizes[i]), dim=50, func_id=func, instance=0,
                         seed=seed * 31 + i + 1000003 * rank, ring_next=(i + 1) % 144) for i in range(144)]
    return specs, inst


def table(specs, inst, device="cuda", tile_rows=_lib.TILE_SIMT, extra_rows=0):
    return SegmentTable(specs, inst, tile_rows=tile_rows, device=device, extra_rows=extra_rows)
