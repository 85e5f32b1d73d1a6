"""The library's tile-shape tuner (speo_autotune_tile_rows) on the GPU: every candidate tile
height gives the same rows bit for bit, and the tuner's choice is one of them, timed once per
shape bucket and then taken from its cache."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _batched(cuda, tile_rows, n_runs=48, seed=5):
    """Batched uneven runs (D in {10, 30, 50, 100}, P in [50, 200], own instance and objective each)."""
    from speo_gb300 import _lib
    from speo_gb300.device import SegmentSpec, SegmentTable
    from speo_gb300.instances import make_instance

    rng = np.random.default_rng(seed)
    specs, inst = [], []
    for i in range(n_runs):
        D = int(rng.choice([10, 30, 50, 100]))
        P = int(rng.integers(50, 201))
        func = _lib.FUNC_ROTATED_SPHERE if rng.integers(0, 2) == 0 else _lib.FUNC_ROTATED_RASTRIGIN
        inst.append(make_instance(700 + i, D))
        specs.append(SegmentSpec(pop_size=P, dim=D, func_id=func, instance=i, seed=40 + i))
    return SegmentTable(specs, inst, device=str(cuda), tile_rows=tile_rows)


def test_every_candidate_gives_the_same_rows(cuda):
    import torch
    from speo_gb300.device import AUTOTUNE_CANDIDATES

    states = []
    for tile in AUTOTUNE_CANDIDATES + (17,):
        tab = _batched(cuda, tile)
        tab.init_population()
        for _ in range(3):
            tab.generation()
        torch.cuda.synchronize()
        states.append((tab.pop[tab.cur].cpu().numpy(), tab.fit[tab.cur].cpu().numpy()))
    for pop, fit in states[1:]:
        assert np.array_equal(pop, states[0][0]) and np.array_equal(fit, states[0][1])


def test_tuner_picks_a_candidate_and_caches_it(cuda):
    from speo_gb300.device import AUTOTUNE_CANDIDATES

    a = _batched(cuda, "auto", seed=11)
    assert a.tile_rows in AUTOTUNE_CANDIDATES
    ms = a.autotune["ms"]
    assert all(v > 0 for v in ms.values())
    assert ms[a.tile_rows] == min(ms.values())
    b = _batched(cuda, "auto", seed=11)          # the same bucket: answered from the cache
    assert b.autotune["cached"] and b.tile_rows == a.tile_rows
    b.init_population()
    b.generation()
