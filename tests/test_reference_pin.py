"""Pins the oracle's DE restatement to the reference's own GPU kernels.

The reference's global_SetupRandomState / global_InitiPopulation / global_DE_FindBestIndividual-
InIsland / global_DE_GenerateNewPopulation (CUDA_EA_library/kernel_EA_CUDA.cu,
kernel_DE_CUDA.cu, compiled unmodified into oracle/_ref/*.fatbin) run on the GPU; this
project's capture kernel replays the same cuRAND XORWOW streams; the oracle, fed those streams
in the reference's draw order, must reproduce the reference's initial population and trial
vectors bit for bit. Shapes keep P a multiple of 16 (the reference skips the last P mod 16 rows)
and strategies that do not read the best row when there are several sub-islands (the
reference's best search ignores the sub-island offset, kernel_DE_CUDA.cu:133,142).
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

import ref_kernels as rk

pytestmark = pytest.mark.gpu


def fma_exact(a, b, c, dtype):
    """a*b + c rounded once to `dtype` (what the reference's contracted min + u*(max-min) does)."""
    from fractions import Fraction

    exact = Fraction(float(a)) * Fraction(float(b)) + Fraction(float(c))
    if dtype == np.float64:
        return float(exact)
    # float32: the exact value fits in a double (24 x 8 bit product), so one more rounding is exact
    return np.float32(float(exact))


def np2(D):
    y = 1
    while y < D:
        y <<= 1
    return max(32, y)


@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("P,D,nsub,strategies", [
    (64, 30, 4, [4, 5, 0, 8]),
    (96, 10, 2, [4, 1]),
    (32, 50, 1, [6]),          # best/1 with one sub-island
    (64, 100, 1, [4]),
])
def test_reference_kernels_match_oracle(oracle, cuda, prec, P, D, nsub, strategies):
    if not rk.available(prec):
        pytest.skip("reference fatbins not built (needs the reference sources at build time)")
    import torch
    from speo_gb300 import _lib

    f64 = prec == "f64"
    dt, npdt = (torch.float64, np.float64) if f64 else (torch.float32, np.float32)
    Pop = _lib.PopulationF64 if f64 else _lib.PopulationF32
    PI = _lib.ProblemInfoF64 if f64 else _lib.ProblemInfoF32
    DI = _lib.DEInfoF64 if f64 else _lib.DEInfoF32
    drv = rk.Driver()
    torch.zeros(1, device=cuda)                 # primary context current on this thread
    de_fat = rk.REF_DIR / f"ref_de_{prec}.fatbin"
    ea_fat = rk.REF_DIR / f"ref_ea_{prec}.fatbin"
    ld = np2(D)
    seed = 1234 + P + D
    n_states = P * 32
    states = torch.zeros(n_states * rk.CURAND_STATE_BYTES // 4 + 64, dtype=torch.int32, device=cuda)
    pop = torch.zeros(P, ld, dtype=dt, device=cuda)
    cand = torch.zeros(P, ld, dtype=dt, device=cuda)
    pfit = torch.zeros(P, dtype=dt, device=cuda)
    cfit = torch.zeros(P, dtype=dt, device=cuda)
    perm_np = np.random.default_rng(P).permutation(P).astype(np.int32)
    perm = torch.zeros(max(P, 64), dtype=torch.int32, device=cuda)   # the best search reads up to 32 entries
    perm[:P] = torch.from_numpy(perm_np)
    best = torch.zeros(max(nsub, 32), dtype=torch.int32, device=cuda)
    S = P // nsub
    CR = np.array([0.9 if i % 2 == 0 else 0.3 for i in range(nsub)], dtype=npdt)
    F = np.full(nsub, 0.5, dtype=npdt)
    info = (DI * nsub)(*[DI(float(CR[i]), float(F[i]), strategies[i % len(strategies)], S) for i in range(nsub)])
    d_info = torch.frombuffer(bytearray(bytes(info)), dtype=torch.uint8).to(cuda)
    problem = PI(D, 9, 1, 0, seed, 0, 0, 100.0, -100.0)
    P_pop = Pop(pop.data_ptr(), pfit.data_ptr())
    P_cand = Pop(cand.data_ptr(), cfit.data_ptr())
    island = _lib.IslandInfo(P, nsub, perm.data_ptr())
    grid, block = rk.de_config(P)

    # reference: seed the states and initialise the population
    drv.launch(drv.function(ea_fat, rk.K_SETUP), grid, block, [ctypes.c_void_p(states.data_ptr()), ctypes.c_int(seed)])
    drv.launch(drv.function(ea_fat, rk.K_INIT), grid, block, [P_pop, ctypes.c_void_p(states.data_ptr()), problem])

    # the same streams, replayed
    L = 96
    cap_t = torch.zeros(n_states, L, dtype=dt, device=cuda)
    cap_fn = drv.function(rk.CAPTURE, b"capture_uniform_f64" if f64 else b"capture_uniform_f32")
    drv.launch(cap_fn, ((n_states + 127) // 128, 1, 1), (128, 1, 1),
               [ctypes.c_ulonglong(seed), ctypes.c_int(n_states), ctypes.c_int(L), ctypes.c_void_p(cap_t.data_ptr())])
    cap = cap_t.cpu().numpy().astype(np.float64)
    loops = ld // 32
    init_draws = np.array([sum(1 for c in range(loops) if l + 32 * c < D) for l in range(32)], dtype=np.int32)
    cap_pos = np.tile(init_draws, P).astype(np.int32)

    # initial population: x = min + u * (max - min), u = the lane's c-th draw for element l + 32c
    got_pop = pop.cpu().numpy()
    lb, ub = npdt(-100.0), npdt(100.0)
    for e in range(D):
        l, c = e % 32, e // 32
        u = cap[np.arange(P) * 32 + l, c].astype(npdt)
        ref = np.array([fma_exact(ui, ub - lb, lb, npdt) for ui in u], dtype=npdt)
        assert np.array_equal(got_pop[:, e], ref), f"init element {e}"

    rng = np.random.default_rng(D)
    fit = rng.uniform(0, 100, P).astype(np.float32).astype(npdt)
    pfit.copy_(torch.from_numpy(fit))
    pop_np = got_pop.copy()
    draws = oracle.captured_draws(cap, cap_pos)
    for g in range(2):
        drv.launch(drv.function(de_fat, rk.K_BEST), (nsub, 1, 1), (32, 1, 1),
                   [ctypes.c_void_p(best.data_ptr()), P_pop, island, problem])
        drv.launch(drv.function(de_fat, rk.K_GEN), grid, block,
                   [P_cand, P_pop, ctypes.c_void_p(best.data_ptr()), island, ctypes.c_void_p(d_info.data_ptr()),
                    ctypes.c_void_p(states.data_ptr()), problem])
        best_ref = oracle.best_per_subisland(fit.astype(np.float32), nsub, perm_np) if nsub == 1 else None
        if nsub == 1:
            assert int(best.cpu()[0]) == int(best_ref[0])
        cand_ref = np.zeros_like(pop_np)
        err = oracle.de_generate(cand_ref, pop_np, ld, D, perm_np, CR, F,
                                 [strategies[i % len(strategies)] for i in range(nsub)],
                                 best_ref, float(lb), float(ub), draws, f64=f64)
        assert err == 0
        got = cand.cpu().numpy()
        assert np.array_equal(got[:, :D], cand_ref[:, :D]), f"generation {g}: {np.argwhere(got[:, :D] != cand_ref[:, :D])[:5]}"
    assert cap_pos.max() < L
