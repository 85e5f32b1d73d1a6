"""The island-resident epoch with the rotation on the tensor cores (speo_generation_epoch_tc).

Its generations must equal, row for row and bit for bit, the composition of the entry points it
fuses: the trial rows of speo_generation (Philox draws, bit-exact against the oracle), their
split-FP16 tensor-core fitness from speo_evaluate_tc, and strict-`<` selection
(kernel_DE_CUDA.cu:312). Every generation's tensor-core fitness is also held to the FP32 bar
against the FP64 oracle (1e-5 relative), and the trials of the first generation to the oracle's
restatement of the reference's DE operator.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIT_RTOL_F32, FIT_ATOL_F32 = 1e-5, 1e-6


def _table(cuda, layout, tile_rows, seed=21):
    from speo_gb300.device import SegmentSpec, SegmentTable
    from speo_gb300.instances import make_instance

    instances, specs = [], []
    for i, (P, D, fid, strategy) in enumerate(layout):
        instances.append(make_instance(seed * 1000 + D * 10 + i, D))
        specs.append(SegmentSpec(pop_size=P, dim=D, func_id=fid, instance=i, seed=seed + 17 * i, strategy=strategy))
    return SegmentTable(specs, instances, device=str(cuda), tile_rows=tile_rows)


def _assert_fitness(gpu, ref, rtol=FIT_RTOL_F32, atol=FIT_ATOL_F32):
    gpu = np.asarray(gpu, dtype=np.float64)
    err = np.abs(gpu - ref)
    bad = err > rtol * np.abs(ref) + atol
    assert not bad.any(), f"max rel err {np.max(err / np.maximum(np.abs(ref), 1e-30)):.3e}"


def _composed(lib, tab, tab_tc, n, oracle):
    """n generations of speo_generation's trials + speo_evaluate_tc + strict-`<` selection on tab."""
    import torch
    from speo_gb300 import _lib

    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    T = torch.zeros_like(tab.pop[0])
    TF = torch.zeros_like(tab.fit[0])
    f_tc = torch.zeros_like(tab.fit[0])
    segs = tab.oracle_segments()
    for g in range(n):
        pin, fin = tab.pop[tab.cur].clone(), tab.fit[tab.cur].clone()
        gen = int(tab.gen[0].cpu())
        tab.generation(trial_out=T, trial_fit_out=TF)
        _lib.check(lib.speo_evaluate_tc(tab_tc.d_segs.data_ptr(), tab_tc.d_items.data_ptr(), tab_tc.n_items,
                                        tab_tc.dim_lo, tab_tc.dim_hi, T.data_ptr(), tab.rows, tab.ld, f_tc.data_ptr(),
                                        stream), "speo_evaluate_tc")
        win = f_tc < fin
        tab.pop[tab.cur].copy_(torch.where(win[:, None], T, pin))
        tab.fit[tab.cur].copy_(torch.where(win, f_tc, fin))
        torch.cuda.synchronize()
        t_np, f_np, p_np, fi_np = T.cpu().numpy(), f_tc.cpu().numpy(), pin.cpu().numpy(), fin.cpu().numpy()
        for s in segs:
            r = slice(s["row0"], s["row0"] + s["P"])
            _assert_fitness(f_np[r], oracle.evaluate_rows(s["func"], t_np[r], s["D"], s["o"], s["M"]))
            if g == 0:   # trials against the oracle's restatement of the reference's DE operator
                d = oracle.philox_draws(s["seed"], gen, pos0=s["row0"])
                cand = np.zeros_like(p_np[r])
                best = int(np.argmin(fi_np[r]))
                assert oracle.de_generate(cand, p_np[r], tab.ld, s["D"], np.arange(s["P"]), [s["CR"]], [s["F"]],
                                          [s["strategy"]], [best], s["lb"], s["ub"], d) == 0
                assert np.array_equal(t_np[r, :s["D"]], cand[:, :s["D"]])


@pytest.mark.parametrize("layout,gens", [
    ([(256, 50, 9, 4)] * 3, 6),                         # the learned-surrogate shape: two 128-row tiles
    ([(100, 30, 9, 4)] * 4, 6),                         # the island-model shape (D <= 32 column class)
    ([(129, 64, 31, 4), (200, 40, 9, 6)], 5),           # one live row in the second tile; best-row strategy
    ([(37, 10, 31, 4), (50, 7, 9, 1), (2, 16, 9, 4)], 8),  # one K step (second K half empty); tiny islands
])
def test_epoch_tc_equals_the_composed_generations(lib, oracle, cuda, layout, gens):
    import torch
    from speo_gb300 import _lib

    a = _table(cuda, layout, _lib.TILE_SIMT)
    b = _table(cuda, layout, _lib.TILE_SIMT)
    a_tc = _table(cuda, layout, _lib.TILE_TC)
    assert b.epoch_tc_fits()
    a.init_population()
    b.init_population()
    _composed(lib, a, a_tc, gens, oracle)
    b.epoch_tc(gens)
    torch.cuda.synchronize()
    assert int(b.gen[0].cpu()) == gens
    D = max(sp.dim for sp in b.specs)
    assert np.array_equal(a.fit[a.cur].cpu().numpy(), b.fit[b.cur].cpu().numpy())
    assert np.array_equal(a.pop[a.cur].cpu().numpy()[:, :D], b.pop[b.cur].cpu().numpy()[:, :D])


def test_epoch_tc_split_launches_continue_the_run(lib, oracle, cuda):
    """Two launches of 7 + 9 generations equal one of 16, and the ring migration between epochs
    composes with them as with the CUDA-core epochs."""
    import torch
    from speo_gb300 import _lib

    layout = [(256, 50, 9, 4)] * 4
    a = _table(cuda, layout, _lib.TILE_SIMT)
    b = _table(cuda, layout, _lib.TILE_SIMT)
    for t in (a, b):
        t.init_population()
    a.epoch_tc(16)
    b.epoch_tc(7)
    b.epoch_tc(9)
    torch.cuda.synchronize()
    assert np.array_equal(a.pop[a.cur].cpu().numpy(), b.pop[b.cur].cpu().numpy())
    assert np.array_equal(a.fit[a.cur].cpu().numpy(), b.fit[b.cur].cpu().numpy())
    assert int(a.gen[0].cpu()) == int(b.gen[0].cpu()) == 16


def test_epoch_tc_refuses_what_it_does_not_run(lib, cuda):
    """Islands beyond two 128-row tiles or D > 64 are refused by the host; an unsupported
    objective inside a launch is flagged and its rows are left as they were."""
    import torch
    from speo_gb300 import _lib

    assert lib.speo_epoch_tc_fits(257, 50) == 0 and lib.speo_epoch_tc_fits(256, 65) == 0
    assert lib.speo_epoch_tc_fits(256, 64) == 1
    tab = _table(cuda, [(64, 30, 4, 4)], _lib.TILE_SIMT)        # Rosenbrock: no tensor-core epoch
    tab.init_population()
    before = tab.pop[tab.cur].clone()
    tab.epoch_tc(2)
    torch.cuda.synchronize()
    assert torch.equal(before, tab.pop[tab.cur])
    bits = ctypes.c_uint32(0)
    assert lib.speo_device_error_bits(ctypes.byref(bits)) == 0
    assert bits.value == _lib.SPEO_DEVERR_BAD_SEGMENT


def test_island_run_equals_epochs_and_ring_calls(lib, cuda):
    """speo_island_run_tc (the island loop as one call, host fitness history) equals
    speo_generation_epoch_tc one generation at a time with speo_ring_migrate at every 10th
    generation of the run; the history holds every generation's fitness."""
    import ctypes

    import torch
    from speo_gb300 import _lib
    from speo_gb300.device import SegmentSpec, SegmentTable
    from speo_gb300.instances import make_instance

    def table():
        inst = [make_instance(4242, 50)]
        specs = [SegmentSpec(pop_size=256, dim=50, func_id=9, instance=0, seed=900 + i, ring_next=(i + 1) % 4)
                 for i in range(4)]
        return SegmentTable(specs, inst, device=str(cuda))

    a, b = table(), table()
    a.init_population()
    b.init_population()
    first, gens, interval, k = 3, 24, 10, 5
    for t in (a, b):                              # the run's first 3 generations, before the call
        t.epoch_tc(first)
    hist = torch.full((gens, a.rows), float("nan")).pin_memory()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.check(lib.speo_island_run_tc(a.d_segs.data_ptr(), 4, 50, 50, 256, a.pop[a.cur].data_ptr(),
                                      a.fit[a.cur].data_ptr(), a.rows, a.gen.data_ptr(), first, gens, interval, k,
                                      a.staging.data_ptr(), a.max_ld, hist.data_ptr(), stream), "speo_island_run_tc")
    want = []
    for g in range(first, first + gens):
        b.epoch_tc(1)
        want.append(b.fit[b.cur].cpu().numpy().copy())
        if (g + 1) % interval == 0:
            b.migrate(k)
    torch.cuda.synchronize()
    assert np.array_equal(a.pop[a.cur].cpu().numpy(), b.pop[b.cur].cpu().numpy())
    assert np.array_equal(a.fit[a.cur].cpu().numpy(), b.fit[b.cur].cpu().numpy())
    assert np.array_equal(hist.numpy(), np.stack(want))
    assert int(a.gen[0].cpu()) == int(b.gen[0].cpu()) == first + gens


def _island_run_vs_calls(lib, cuda, sizes, ring, D, gens, interval, k, first=0):
    """speo_island_run_tc without read-back against speo_generation_epoch_tc + speo_ring_migrate."""
    import ctypes

    import torch
    from speo_gb300 import _lib
    from speo_gb300.device import SegmentSpec, SegmentTable
    from speo_gb300.instances import make_instance

    def table():
        inst = [make_instance(777, D)]
        specs = [SegmentSpec(pop_size=sizes[i], dim=D, func_id=31 if i % 2 else 9, instance=0, seed=300 + i,
                             ring_next=ring[i]) for i in range(len(sizes))]
        return SegmentTable(specs, inst, device=str(cuda))

    a, b = table(), table()
    a.init_population()
    b.init_population()
    n = len(sizes)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.check(lib.speo_island_run_tc(a.d_segs.data_ptr(), n, D, D, max(sizes), a.pop[a.cur].data_ptr(),
                                      a.fit[a.cur].data_ptr(), a.rows, a.gen.data_ptr(), first, gens, interval, k,
                                      a.staging.data_ptr(), a.max_ld, None, stream), "speo_island_run_tc")
    done = 0
    while done < gens:
        step = min(gens - done, interval - (first + done) % interval)
        b.epoch_tc(step)
        done += step
        if (first + done) % interval == 0:
            b.migrate(k)
    torch.cuda.synchronize()
    assert np.array_equal(a.pop[a.cur].cpu().numpy(), b.pop[b.cur].cpu().numpy())
    assert np.array_equal(a.fit[a.cur].cpu().numpy(), b.fit[b.cur].cpu().numpy())
    assert int(a.gen[0].cpu()) == int(b.gen[0].cpu()) == gens
    bits = ctypes.c_uint32(0xFFFF)
    assert lib.speo_device_error_bits(ctypes.byref(bits)) == 0
    assert bits.value == 0


def test_island_run_migrates_inside_one_launch(lib, cuda):
    """Every island resident at once: the whole run (six migrations) is one cooperative launch
    whose migrations meet at a grid barrier; uneven islands, a ring of five and one island outside
    it (no successor, no predecessor). Bit-identical to separate epochs and ring calls."""
    sizes = [256, 100, 64, 200, 128, 77]
    ring = [1, 2, 3, 4, 0, -1]
    _island_run_vs_calls(lib, cuda, sizes, ring, 50, 60, 10, 5, first=0)
    _island_run_vs_calls(lib, cuda, sizes, ring, 20, 37, 8, 3, first=0)


def test_island_run_more_islands_than_resident_blocks(lib, cuda):
    """More islands than SMs (one resident block per SM): the run falls back to one launch per
    interval and speo_ring_migrate between them, with the same result."""
    import torch

    n = torch.cuda.get_device_properties(0).multi_processor_count + 8
    _island_run_vs_calls(lib, cuda, [16] * n, [(i + 1) % n for i in range(n)], 8, 12, 5, 2)
