"""GPU parity tests: every entry point called through the C ABI against the CPU oracle.

Bars: trial vectors, donor/crossover draws, best ids, selection decisions and migrated rows
bit-exact; FP32 fitness within relative 1e-5 of the FP64 oracle (FP64 entry points 1e-12).
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIT_RTOL_F32 = 1e-5      # FP32 fitness vs FP64 oracle
FIT_ATOL_F32 = 1e-6      # absolute floor for fitness values near 0
FIT_RTOL_F64 = 1e-12


def np2(D):
    y = 1
    while y < D:
        y <<= 1
    return max(32, y)


def _assert_fitness(gpu, ref, rtol=FIT_RTOL_F32, atol=FIT_ATOL_F32):
    gpu = np.asarray(gpu, dtype=np.float64)
    err = np.abs(gpu - ref)
    bad = err > rtol * np.abs(ref) + atol
    assert not bad.any(), f"max rel err {np.max(err / np.maximum(np.abs(ref), 1e-30)):.3e} at {np.argmax(bad)}"


# ---------------------------------------------------------------------------------------------
# drop-in (reference-shaped) entry points
# ---------------------------------------------------------------------------------------------
class DropIn:
    def __init__(self, lib, cuda, P, D, nsub, f64, seed=1234):
        import torch
        from speo_gb300 import _lib

        self.torch, self._lib, self.lib = torch, _lib, lib
        self.P, self.D, self.nsub, self.f64 = P, D, nsub, f64
        self.ld = np2(D)
        self.dt = torch.float64 if f64 else torch.float32
        self.np_dt = np.float64 if f64 else np.float32
        z = lambda *s: torch.zeros(*s, dtype=self.dt, device=cuda)
        self.pop, self.cand = z(P, self.ld), z(P, self.ld)
        self.pfit, self.cfit = z(P), z(P)
        self.rng = torch.zeros(16, dtype=torch.int32, device=cuda)
        self.best = torch.zeros(nsub, dtype=torch.int32, device=cuda)
        self.perm = torch.arange(P, dtype=torch.int32, device=cuda)
        self.Pop = _lib.PopulationF64 if f64 else _lib.PopulationF32
        self.PI = _lib.ProblemInfoF64 if f64 else _lib.ProblemInfoF32
        self.DI = _lib.DEInfoF64 if f64 else _lib.DEInfoF32
        self.sfx = "" if f64 else "_f32"
        self.seed = seed
        self.problem = self.PI(D, 9, 1, 0, seed, 0, 0, 100.0, -100.0)

    def pops(self):
        return (self.Pop(self.pop.data_ptr(), self.pfit.data_ptr()), self.Pop(self.cand.data_ptr(),
                                                                              self.cfit.data_ptr()))

    def island(self):
        return self._lib.IslandInfo(self.P, self.nsub, self.perm.data_ptr())

    def call(self, name, *args):
        st = getattr(self.lib, name + self.sfx)(*args)
        self._lib.check(st, name)
        self._lib.check(self.lib.API_CheckCUDAError(), "API_CheckCUDAError")


@pytest.mark.parametrize("P,D", [(100, 30), (64, 10), (17, 1), (33, 100)])
def test_dropin_init_matches_oracle(lib, oracle, cuda, P, D):
    d = DropIn(lib, cuda, P, D, 1, False, seed=99)
    pop, _ = d.pops()
    d.call("API_Initilize", pop, d.rng.data_ptr(), d.island(), d.problem)
    ref = oracle.init_population(P, d.ld, D, -100.0, 100.0, 99)
    assert np.array_equal(d.pop.cpu().numpy(), ref)       # every row, also past 16*floor(P/16)
    st = d.rng.cpu().numpy()
    assert st[0] == 99 and st[1] == 0 and st[2] == 0 and st[3] == 0


@pytest.mark.parametrize("f64", [False, True])
@pytest.mark.parametrize("P,D,nsub", [(100, 30, 4), (64, 10, 1), (96, 100, 3), (8, 1, 2), (40, 33, 10), (2048, 10, 1),
                                      (3000, 30, 2), (40, 256, 2)])   # last: D = SPEO_MAX_DIM
def test_dropin_generate_matches_oracle(lib, oracle, cuda, f64, P, D, nsub):
    import torch

    d = DropIn(lib, cuda, P, D, nsub, f64, seed=P * 7 + D)
    scratch = d.Pop(d.cand.data_ptr(), d.cfit.data_ptr())
    d.call("API_Initilize", scratch, d.rng.data_ptr(), d.island(), d.problem)     # key + gen = 0
    rng = np.random.default_rng(P + D)
    pop = np.zeros((P, d.ld), dtype=d.np_dt)
    pop[:, :D] = rng.uniform(-100, 100, (P, D)).astype(np.float32)
    fit = rng.uniform(0, 1000, P).astype(np.float32).astype(d.np_dt)
    fit[rng.integers(0, P)] = fit[rng.integers(0, P)]          # ties
    perm = rng.permutation(P).astype(np.int32)
    S = P // nsub
    strat = np.array([i % 9 for i in range(nsub)], dtype=np.int32)
    CR = np.array([0.9 if i % 2 == 0 else 0.1 for i in range(nsub)], dtype=d.np_dt)
    F = np.full(nsub, 0.5, dtype=d.np_dt)
    info = (d.DI * nsub)(*[d.DI(float(CR[i]), float(F[i]), int(strat[i]), S) for i in range(nsub)])
    d_info = torch.frombuffer(bytearray(bytes(info)), dtype=torch.uint8).to(cuda)
    d.pop.copy_(torch.from_numpy(pop))
    d.pfit.copy_(torch.from_numpy(fit))
    d.perm.copy_(torch.from_numpy(perm))
    d.cand.zero_()
    pop_s, cand_s = d.pops()
    for gen in range(2):
        d.call("API_DE_GenerateNewPopulation", cand_s, pop_s, d.best.data_ptr(), d.island(), d_info.data_ptr(),
               d.rng.data_ptr(), d.problem)
        best_ref = oracle.best_per_subisland(fit.astype(np.float32), nsub, perm)
        assert np.array_equal(d.best.cpu().numpy(), best_ref)
        cand_ref = np.zeros_like(pop) if gen == 0 else cand_ref
        err = oracle.de_generate(cand_ref, pop, d.ld, D, perm, CR, F, strat, best_ref, -100.0, 100.0,
                                 oracle.philox_draws(d.seed, gen), f64=f64)
        assert err == 0
        got = d.cand.cpu().numpy()
        assert np.array_equal(got, cand_ref), f"gen {gen}: {np.argwhere(got != cand_ref)[:5]}"
        assert int(d.rng.cpu()[2]) == gen + 1                    # generation counter advanced once


@pytest.mark.parametrize("gens,pinned,history,P,D,nsub,fid,strats", [
    (60, True, True, 200, 30, 2, 9, (4, 6)),         # config-1 sub-islands, several fused launches
    (30, True, True, 4000, 30, 80, 9, (4, 6)),       # 80 sub-islands of 50: one block each (2 x 80 > SMs)
    (7, False, False, 200, 30, 2, 9, (4, 6)),        # pageable buffer, last generation only
    (21, True, True, 111, 50, 3, 4, (2, 4, 7)),      # odd sub-islands of 37, best-row strategies, Rosenbrock
    (6, True, True, 256, 100, 4, 31, (5, 3, 8, 0)),  # D = 100
    (5, True, False, 64, 10, 1, 10, (1,)),           # unrotated Schwefel, one sub-island
    (22, True, False, 4096, 100, 1, 9, (4,)),        # too large for one block: three calls, graph blocks
    (4, True, True, 4096, 100, 1, 9, (4,)),          # the same with every generation's fitness
    (9, True, True, 200, 30, 2, 23, (4, 6)),         # composition: three calls, every generation's fitness
    (24, True, False, 300, 50, 3, 30, (4, 6, 2)),    # composition of hybrids: graph blocks
    (5, False, True, 120, 20, 2, 21, (6,)),          # hybrid, pageable buffer
    (4, True, True, 64, 256, 2, 9, (4, 6)),          # D = SPEO_MAX_DIM
])
@pytest.mark.parametrize("f64", [False, True])
def test_de_run_matches_the_dropin_loop(lib, cuda, f64, gens, pinned, history, P, D, nsub, fid, strats):
    """speo_de_run_f32 / _f64 (the reference's DE_CUDA::Run loop, natively: sub-islands resident in
    shared memory for blocks of generations, in FP32 on two-block clusters when the GPU has SMs for
    two blocks per sub-island, or the three calls replayed as a CUDA graph) gives the same
    populations, candidates, best ids, generation counter and per-generation fitness as the drop-in
    calls issued one by one."""
    import torch
    from speo_gb300.instances import make_instance_multi

    o, M, S = make_instance_multi(77, D, fid)       # component 0 = make_instance(77, D)
    nc, ld = o.shape[0], np2(D)
    dt = np.float64 if f64 else np.float32
    rot = np.zeros((nc, ld, D), dtype=dt)
    rot[:, :D] = M.transpose(0, 2, 1)
    shift = np.zeros((nc, ld), dtype=dt)
    shift[:, :D] = o
    shuf = np.zeros((nc, ld), dtype=np.int32)
    shuf[:, :D] = S
    d_rot, d_sh = torch.from_numpy(rot).to(cuda), torch.from_numpy(shift).to(cuda)
    d_sf = torch.from_numpy(shuf).to(cuda)
    rng = np.random.default_rng(9)
    pop0 = np.zeros((P, ld), dtype=dt)
    pop0[:, :D] = rng.uniform(-100, 100, (P, D))
    runs = []
    perm = np.random.default_rng(P + D).permutation(P).astype(np.int32)
    for mode in ("calls", "driver"):
        d = DropIn(lib, cuda, P, D, nsub, f64, seed=4321)
        d.problem.function_ID = fid
        evaluate = getattr(d.lib, "API_evaluateFitness" + d.sfx)
        d.perm.copy_(torch.from_numpy(perm))
        info = (d.DI * nsub)(*[d.DI(0.9 if i % 2 == 0 else 0.1, 0.5, strats[i % len(strats)], P // nsub)
                               for i in range(nsub)])
        d_info = torch.frombuffer(bytearray(bytes(info)), dtype=torch.uint8).to(cuda)
        pop_s, cand_s = d.pops()
        d.call("API_Initilize", cand_s, d.rng.data_ptr(), d.island(), d.problem)
        d.pop.copy_(torch.from_numpy(pop0))
        args = (None, None, d.pop.data_ptr(), d_sh.data_ptr(), d_rot.data_ptr(), d_sf.data_ptr(), None, None, None, P,
                D, 0.0, fid)
        evaluate(d.pfit.data_ptr(), *args)
        if mode == "calls":
            per_gen = []
            for _ in range(gens):
                d.call("API_DE_GenerateNewPopulation", cand_s, pop_s, d.best.data_ptr(), d.island(),
                       d_info.data_ptr(), d.rng.data_ptr(), d.problem)
                evaluate(d.cfit.data_ptr(), None, None, d.cand.data_ptr(), d_sh.data_ptr(), d_rot.data_ptr(),
                         d_sf.data_ptr(), None, None, None, P, D, 0.0, fid)
                d.call("API_DE_SelectSurvival", pop_s, cand_s, d.island(), d.problem)
                per_gen.append(d.pfit.cpu().numpy())
            h = np.stack(per_gen)
        else:
            h = torch.zeros((gens if history else 1) * P, dtype=d.dt)
            if pinned:
                h = h.pin_memory()
            run = getattr(d.lib, "speo_de_run" + ("_f64" if f64 else "_f32"))
            d._lib.check(run(pop_s, cand_s, d.rng.data_ptr(), d.island(), d_info.data_ptr(), d.best.data_ptr(),
                             d.problem, d_sh.data_ptr(), d_rot.data_ptr(), d_sf.data_ptr(), gens, h.data_ptr(),
                             int(history), None), "speo_de_run")
            h = h.numpy().reshape(-1, P)
        d._lib.check(d.lib.API_CheckCUDAError(), "API_CheckCUDAError")
        runs.append((d.pop.cpu().numpy(), d.pfit.cpu().numpy(), h.copy(),
                     int(d.rng.cpu()[2]), d.cand.cpu().numpy(), d.cfit.cpu().numpy(), d.best.cpu().numpy()))
    (pa, fa, ha, ga, ca, cfa, ba), (pb, fb, hb, gb, cb, cfb, bb) = runs
    assert np.array_equal(pa, pb)
    assert np.array_equal(fa, fb)
    if history:
        assert np.array_equal(hb, ha)      # every generation's fitness read back
    else:
        assert np.array_equal(hb[0], fb)   # the last generation's fitness read back
    assert ga == gb == gens
    assert np.array_equal(ca, cb) and np.array_equal(cfa, cfb) and np.array_equal(ba, bb)


# P = 5000 spans several batches of 2048 rows per block; D = 1 and 3 have no 16-byte bulk part
# in FP32 (rows copied element by element), D = 30 a ragged tail, D = 100 and 256 none.
@pytest.mark.parametrize("P,D", [(100, 30), (5000, 1), (5000, 3), (5000, 4), (5000, 30), (5000, 100), (777, 256)])
@pytest.mark.parametrize("f64", [False, True])
def test_dropin_select_matches_oracle(lib, oracle, cuda, f64, P, D):
    import torch

    d = DropIn(lib, cuda, P, D, 1, f64)
    rng = np.random.default_rng(4)
    pop = rng.uniform(-100, 100, (P, d.ld)).astype(d.np_dt)
    cand = rng.uniform(-100, 100, (P, d.ld)).astype(d.np_dt)
    pf = rng.uniform(0, 10, P).astype(d.np_dt)
    cf = rng.uniform(0, 10, P).astype(d.np_dt)
    cf[::7] = pf[::7]                                   # ties keep the parent
    cf[3] = np.nan
    for t, a in ((d.pop, pop), (d.cand, cand), (d.pfit, pf), (d.cfit, cf)):
        t.copy_(torch.from_numpy(a))
    pop_s, cand_s = d.pops()
    d.call("API_DE_SelectSurvival", pop_s, cand_s, d.island(), d.problem)
    oracle.select(pop, pf, cand, cf, d.ld, D, f64=f64)
    assert np.array_equal(d.pop.cpu().numpy(), pop)
    assert np.array_equal(d.pfit.cpu().numpy(), pf)


# Per-function fitness bars (rtol, atol) against the FP64 oracle. The defaults are the FP32 /
# FP64 bars above; the exceptions are ill-conditioned in the input: the elliptic, bent-cigar and
# discus functions (1-3) weight single coordinates up to 1e6 times the rest, so the FP32 rounding
# of one rotated coordinate can dominate a row's error; Weierstrass (6) and Katsuura
# (12) amplify z by up to 3^20 and 2^32 in their high harmonics, Schwefel (10, 11) and Ackley (5)
# cancel terms of size ~400 D and ~20 near the optimum, and HappyCat / HGBat (13, 14) take
# |r2 - D|^(1/4) and |r2^2 - s^2|^(1/2), which turn an FP32 rounding of r2 near the optimum into
# a visible absolute error.
ALL_FUNCS = list(range(1, 17)) + [31]
TOL32 = {1: (1e-4, 1e-6), 2: (1e-4, 1e-6), 3: (1e-4, 1e-6), 5: (1e-5, 2e-5), 6: (2e-3, 5e-2), 10: (2e-4, 5e-2),
         11: (2e-4, 5e-2), 12: (2e-4, 1e-5), 13: (1e-5, 5e-3), 14: (1e-5, 5e-3)}
TOL64 = {5: (1e-12, 1e-12), 6: (1e-10, 1e-10), 10: (1e-11, 1e-8), 11: (1e-11, 1e-8), 12: (1e-10, 1e-12),
         13: (1e-12, 1e-9), 14: (1e-12, 1e-9)}


def _tol(fid, f64):
    return (TOL64 if f64 else TOL32).get(fid, (FIT_RTOL_F64, 1e-12) if f64 else (FIT_RTOL_F32, FIT_ATOL_F32))


@pytest.mark.parametrize("f64", [False, True])
@pytest.mark.parametrize("fid", ALL_FUNCS)
@pytest.mark.parametrize("P,D", [(100, 10), (130, 30), (64, 50), (70, 100), (5, 200), (3, 256)])
def test_dropin_evaluate_matches_oracle(lib, oracle, cuda, f64, fid, P, D):
    """API_evaluateFitness for every implemented function id (CEC2014 1-16, rotated sphere 31)."""
    import torch
    from speo_gb300.instances import make_instance

    o, M = make_instance(P * 31 + D, D)
    ld = np2(D)
    rng = np.random.default_rng(D)
    X = np.zeros((P, ld), dtype=np.float32)
    X[:, :D] = rng.uniform(-100, 100, (P, D))
    X[0, :D] = o
    X[1, :D] = o + rng.normal(0, 1e-3, D).astype(np.float32)
    dt = torch.float64 if f64 else torch.float32
    rot = np.zeros((ld, D), dtype=np.float32)        # reference layout: B[k][j] = M[j][k], zero rows k >= D
    rot[:D, :] = M.T
    shift = np.zeros(ld, dtype=np.float32)
    shift[:D] = o
    tX, trot, tsh = (torch.from_numpy(a).to(cuda, dt) for a in (X, rot, shift))
    f = torch.zeros(P, dtype=dt, device=cuda)
    fn = lib.API_evaluateFitness if f64 else lib.API_evaluateFitness_f32
    fn(f.data_ptr(), None, None, tX.data_ptr(), tsh.data_ptr(), trot.data_ptr(), None, None, None, None, P, D, 0.0,
       fid)
    from speo_gb300 import _lib
    _lib.check(lib.API_CheckCUDAError(), "API_evaluateFitness")
    ref = oracle.evaluate_rows(fid, X, D, o, M)
    rtol, atol = _tol(fid, f64)
    assert abs(float(f[0])) <= atol                    # f(o) - f* = 0
    _assert_fitness(f.cpu().numpy(), ref, rtol=rtol, atol=atol)


def test_segment_evaluate_all_functions(oracle, cuda):
    """speo_evaluate on one table holding a segment of every function id (D = 30, one launch)."""
    import torch

    layout = [(40, 30, fid, 4) for fid in ALL_FUNCS]
    tab = _table(cuda, layout)
    tab.init_population()
    out = torch.zeros_like(tab.fit[0])
    tab.evaluate(which=tab.cur, out=out)
    torch.cuda.synchronize()
    pop, got = tab.pop[tab.cur].cpu().numpy(), out.cpu().numpy()
    for s in tab.oracle_segments():
        r = slice(s["row0"], s["row0"] + s["P"])
        rtol, atol = _tol(s["func"], False)
        _assert_fitness(got[r], oracle.evaluate_rows(s["func"], pop[r], s["D"], s["o"], s["M"]), rtol=rtol,
                        atol=atol)


def test_evaluate_tc_flags_functions_it_does_not_implement(lib, cuda):
    """The tensor-core evaluation implements the rotated single-matrix ids; a tile of an unrotated
    id (here 10) is skipped and raises SPEO_DEVERR_BAD_SEGMENT."""
    import ctypes

    import torch
    from speo_gb300 import _lib

    tab = _table(cuda, [(64, 30, 10, 4)], tile_rows=_lib.TILE_TC)
    tab.init_population()
    bits = ctypes.c_uint32()
    _lib.check(lib.speo_device_error_bits(ctypes.byref(bits)), "clear flags")
    out = torch.full_like(tab.fit[0], -1.0)
    tab.evaluate(which=tab.cur, use_tc=True, out=out)
    _lib.check(lib.speo_device_error_bits(ctypes.byref(bits)), "read flags")
    assert bits.value & _lib.SPEO_DEVERR_BAD_SEGMENT
    assert torch.all(out == -1.0)


# ---- hybrid (17-22) and composition (23-30) functions -------------------------------------
# FP32 tolerances: the hybrids sum groups of the bodies above (Schwefel, Weierstrass and Katsuura
# groups carry their own FP32 error), and the compositions mix components whose FP32 errors are
# those of their bodies, rescaled; the FP32 mixing weights come from logarithms (relative error
# ~|l| 2^-24 for |l| up to ~200). Measured on GB300 over D = 10-100 and points at, near and far
# from every component's optimum: relative error <= 1e-5 above 5e-2; the absolute floor covers
# the unrotated Schwefel component of 24 (418.98 D - sum cancels in FP32 near its optimum).
MULTI_FUNCS = list(range(17, 31))
TOL32_MULTI = (2e-5, 5e-2)
TOL64_MULTI = (1e-11, 1e-8)


def _multi_points(rng, o, P, D):
    X = rng.uniform(-100, 100, (P, D)).astype(np.float32)
    X[0] = o[0]                                                       # the optimum (component 0)
    X[1] = o[0] + rng.normal(0, 1e-3, D).astype(np.float32)
    X[2] = np.clip(o[-1] + rng.normal(0, 1.0, D), -100, 100).astype(np.float32)
    return X


@pytest.mark.parametrize("f64", [False, True])
@pytest.mark.parametrize("fid", MULTI_FUNCS)
@pytest.mark.parametrize("P,D", [(100, 10), (90, 20), (130, 30), (64, 50), (70, 100)])
def test_dropin_evaluate_multi_matches_oracle(lib, oracle, cuda, f64, fid, P, D):
    """API_evaluateFitness for the hybrid and composition functions on the reference's device layout
    (component c's shift at c*np2, M^T at c*np2*D, shuffle at c*np2; CEC2014_CUDA.cc:160-281)."""
    import torch
    from speo_gb300 import _lib
    from speo_gb300.instances import make_instance_multi

    o, M, S = make_instance_multi(P * 31 + D, D, fid)
    nc, ld = o.shape[0], np2(D)
    rng = np.random.default_rng(fid * 1000 + D)
    X = np.zeros((P, ld), dtype=np.float32)
    X[:, :D] = _multi_points(rng, o, P, D)
    rot = np.zeros((nc, ld, D), dtype=np.float32)
    rot[:, :D, :] = M.transpose(0, 2, 1)
    shift = np.zeros((nc, ld), dtype=np.float32)
    shift[:, :D] = o
    shuf = np.zeros((nc, ld), dtype=np.int32)
    shuf[:, :D] = S
    dt = torch.float64 if f64 else torch.float32
    tX, trot, tsh = (torch.from_numpy(a).to(cuda, dt) for a in (X, rot, shift))
    tsf = torch.from_numpy(shuf).to(cuda)
    f = torch.full((P,), -1.0, dtype=dt, device=cuda)
    fn = lib.API_evaluateFitness if f64 else lib.API_evaluateFitness_f32
    fn(f.data_ptr(), None, None, tX.data_ptr(), tsh.data_ptr(), trot.data_ptr(), tsf.data_ptr(), None, None, None, P, D,
       0.0, fid)
    _lib.check(lib.API_CheckCUDAError(), "API_evaluateFitness")
    ref = oracle.evaluate_rows_multi(fid, X, D, o, M, S)
    rtol, atol = TOL64_MULTI if f64 else TOL32_MULTI
    assert abs(float(f[0])) <= atol                    # f(o_1) - f* = 0
    _assert_fitness(f.cpu().numpy(), ref, rtol=rtol, atol=atol)


@pytest.mark.parametrize("fid", [23, 24, 29, 30, 17])
def test_multi_tiles_do_not_change_results(lib, cuda, fid):
    """A row's fitness does not depend on how the rows are tiled: a 4096-row call (16-row tiles)
    and a 20000-row call (64-row tiles) agree bit for bit on their common rows, in both precisions."""
    import torch
    from speo_gb300 import _lib
    from speo_gb300.instances import make_instance_multi

    D, ld, n_big, n_small = 50, 64, 20000, 4096
    o, M, S = make_instance_multi(fid + 5, D, fid)
    nc = o.shape[0]
    rot = np.zeros((nc, ld, D), dtype=np.float32)
    rot[:, :D] = M.transpose(0, 2, 1)
    shift = np.zeros((nc, ld), dtype=np.float32)
    shift[:, :D] = o
    shuf = np.zeros((nc, ld), dtype=np.int32)
    shuf[:, :D] = S
    X = np.zeros((n_big, ld), dtype=np.float32)
    X[:, :D] = np.random.default_rng(fid).uniform(-100, 100, (n_big, D))
    for dt, fn in ((torch.float32, lib.API_evaluateFitness_f32), (torch.float64, lib.API_evaluateFitness)):
        tX, tr, ts = (torch.from_numpy(a).to(cuda, dt) for a in (X, rot, shift))
        tsf = torch.from_numpy(shuf).to(cuda)
        outs = []
        for n in (n_big, n_small):
            f = torch.full((n,), -1.0, dtype=dt, device=cuda)
            fn(f.data_ptr(), None, None, tX.data_ptr(), ts.data_ptr(), tr.data_ptr(), tsf.data_ptr(), None, None, None,
               n, D, 0.0, fid)
            _lib.check(lib.API_CheckCUDAError(), "API_evaluateFitness")
            outs.append(f.cpu().numpy())
        assert np.array_equal(outs[0][:n_small], outs[1])


def _table_multi(cuda, layout, seed=11):
    """layout: (P, D, fid); one multi-component instance (o, M, S) per entry."""
    from speo_gb300 import _lib
    from speo_gb300.device import SegmentSpec, SegmentTable
    from speo_gb300.instances import make_instance_multi

    instances, specs = [], []
    for i, (P, D, fid) in enumerate(layout):
        instances.append(make_instance_multi(seed * 1000 + D * 37 + fid, D, fid))
        specs.append(SegmentSpec(pop_size=P, dim=D, func_id=fid, instance=i, seed=seed + i))
    return SegmentTable(specs, instances, device=str(cuda), tile_rows=_lib.TILE_SIMT)


def test_segment_evaluate_multi_functions(oracle, cuda):
    """speo_evaluate on one table holding every hybrid / composition id next to ids 1-16 and 31, at
    D = 10, 30 (one column group) and 50 (the next); each segment against the oracle."""
    import torch

    layout = [(40 + fid, D, fid) for fid in MULTI_FUNCS for D in (10, 30)] + [(70, 50, 23), (66, 50, 30)]
    layout += [(50, 30, 9), (50, 30, 4)]
    tab = _table_multi(cuda, layout)
    tab.init_population()
    out = torch.zeros_like(tab.fit[0])
    tab.evaluate(which=tab.cur, out=out)
    torch.cuda.synchronize()
    pop, got = tab.pop[tab.cur].cpu().numpy(), out.cpu().numpy()
    for s in tab.oracle_segments():
        r = slice(s["row0"], s["row0"] + s["P"])
        ref = oracle.evaluate_rows_multi(s["func"], pop[r], s["D"], s["o"], s["M"], s["S"])
        rtol, atol = TOL32_MULTI if s["func"] in MULTI_FUNCS else _tol(s["func"], False)
        _assert_fitness(got[r], ref, rtol=rtol, atol=atol)


def test_best_reeval_f64_multi_functions(oracle, cuda):
    """speo_best_reeval_f64 on hybrid / composition segments: argmin row and its FP64 value."""
    layout = [(64, 30, fid) for fid in MULTI_FUNCS] + [(48, 10, 29), (48, 50, 26)]
    tab = _table_multi(cuda, layout)
    tab.init_population()
    rows, errs = tab.best_f64()
    fit = tab.fit[tab.cur].cpu().numpy()
    pop = tab.pop[tab.cur].cpu().numpy()
    for i, s in enumerate(tab.oracle_segments()):
        seg_fit = fit[s["row0"]:s["row0"] + s["P"]]
        assert int(rows[i]) == s["row0"] + int(np.argmin(seg_fit))
        ref = oracle.objective_multi(s["func"], pop[int(rows[i]), :s["D"]], s["o"], s["M"], s["S"])
        assert float(errs[i]) == pytest.approx(ref, rel=1e-10, abs=1e-9)


def test_fused_generation_flags_multi_functions(lib, cuda):
    """The fused generation kernels implement ids 1-16 and 31: a hybrid / composition segment is
    skipped and raises SPEO_DEVERR_BAD_SEGMENT (the drop-in loop evaluates those ids instead)."""
    import ctypes

    from speo_gb300 import _lib

    tab = _table_multi(cuda, [(64, 30, 23)])
    tab.init_population()
    bits = ctypes.c_uint32()
    _lib.check(lib.speo_device_error_bits(ctypes.byref(bits)), "clear flags")
    assert bits.value == 0
    tab.generation()
    _lib.check(lib.speo_device_error_bits(ctypes.byref(bits)), "read flags")
    assert bits.value & _lib.SPEO_DEVERR_BAD_SEGMENT


# ---------------------------------------------------------------------------------------------
# extended entry points: fused generation, migration, FP64 best re-evaluation
# ---------------------------------------------------------------------------------------------
def _table(cuda, layout, n_inst=None, ring=False, seed=7, tile_rows=None):
    from speo_gb300.device import SegmentSpec, SegmentTable
    from speo_gb300.instances import make_instance

    dims = sorted({D for (_, D, _, _) in layout})
    inst = {}
    instances = []
    specs = []
    for i, (P, D, fid, strategy) in enumerate(layout):
        key = (D, fid if n_inst is None else i % n_inst)
        if key not in inst:
            inst[key] = len(instances)
            instances.append(make_instance(seed * 1000 + D * 10 + len(instances), D))
        specs.append(SegmentSpec(pop_size=P, dim=D, func_id=fid, instance=inst[key], seed=seed + i,
                                 strategy=strategy, ring_next=((i + 1) % len(layout)) if ring else -1))
    from speo_gb300 import _lib

    return SegmentTable(specs, instances, device=str(cuda), tile_rows=tile_rows or _lib.TILE_SIMT)


def _check_generations(tab, oracle, n_gen=3):
    import torch

    segs = tab.oracle_segments()
    # initial population and its fitness
    pop0 = tab.pop[tab.cur].cpu().numpy()
    for s in segs:
        ref = oracle.init_population(s["P"], tab.ld, s["D"], s["lb"], s["ub"], s["seed"], row0=s["row0"])
        assert np.array_equal(pop0[s["row0"]:s["row0"] + s["P"]], ref)
        fref = oracle.evaluate_rows(s["func"], ref, s["D"], s["o"], s["M"])
        _assert_fitness(tab.fit[tab.cur].cpu().numpy()[s["row0"]:s["row0"] + s["P"]], fref)
    trial = torch.zeros_like(tab.pop[0])
    tfit = torch.zeros_like(tab.fit[0])
    for g in range(n_gen):
        pin = tab.pop[tab.cur].cpu().numpy()
        fin = tab.fit[tab.cur].cpu().numpy()
        tab.generation(trial_out=trial, trial_fit_out=tfit)
        torch.cuda.synchronize()
        tf = tfit.cpu().numpy()
        pout_ref, fout_ref, trials_ref, sel, err = oracle.generation(segs, g, pin, fin, trial_fit=tf)
        assert err == 0
        got_trials = trial.cpu().numpy()
        for s in segs:
            r = slice(s["row0"], s["row0"] + s["P"])
            D = s["D"]
            assert np.array_equal(got_trials[r, :D], trials_ref[r, :D]), f"gen {g} trials differ"
            _assert_fitness(tf[r], oracle.evaluate_rows(s["func"], trials_ref[r], D, s["o"], s["M"]))
            assert np.array_equal(tab.pop[tab.cur].cpu().numpy()[r, :D], pout_ref[r, :D])
        assert np.array_equal(tab.fit[tab.cur].cpu().numpy(), fout_ref)
        assert int(tab.gen.cpu()[0]) == g + 1 and int(tab.gen.cpu()[1]) == 0


@pytest.mark.parametrize("layout", [
    [(100, 30, 9, 4), (100, 30, 9, 4), (100, 30, 31, 4)],            # config-1 islands, tiles 50 + 50
    [(128, 100, 9, 4), (128, 100, 31, 5)],                            # config-2 shape
    [(64, 50, 9, 2), (70, 50, 9, 6), (33, 50, 31, 3)],                # strategies that use the best row
    [(4, 1, 31, 4), (9, 3, 9, 8), (5, 7, 31, 0)],                     # smallest populations / dims
    [(40, 200, 9, 4)],                                                # largest column class
    [(40, 30, 4, 4), (40, 30, 8, 4), (40, 20, 15, 6), (33, 20, 16, 4), (40, 10, 1, 2)],  # other CEC2014 ids
])
def test_fused_generation_matches_oracle(oracle, cuda, layout):
    tab = _table(cuda, layout)
    tab.init_population()
    _check_generations(tab, oracle)


def test_mixed_dims_single_launch_matches_oracle(oracle, cuda):
    """Batched uneven runs (config-3 shape, scaled down): D and P differ per segment; one
    kernel launch per generation."""
    rng = np.random.default_rng(11)
    layout = [(int(rng.integers(50, 201)), int(rng.choice([10, 30, 50, 100])), int(rng.choice([9, 31])), 4)
              for _ in range(12)]
    tab = _table(cuda, layout, n_inst=12)
    tab.init_population()
    _check_generations(tab, oracle, n_gen=2)


def test_ring_migration_matches_oracle(oracle, cuda):
    import torch

    tab = _table(cuda, [(100, 30, 9, 4)] * 6, ring=True)
    tab.init_population()
    tab.generation()
    pop = tab.pop[tab.cur].cpu().numpy().copy()
    fit = tab.fit[tab.cur].cpu().numpy().copy()
    fit[3] = fit[4]                                     # a tie inside segment 0
    tab.fit[tab.cur].copy_(torch.from_numpy(fit))
    tab.migrate(5)
    torch.cuda.synchronize()
    oracle.ring_migrate(tab.oracle_segments(), 5, pop, fit)
    assert np.array_equal(tab.pop[tab.cur].cpu().numpy(), pop)
    assert np.array_equal(tab.fit[tab.cur].cpu().numpy(), fit)


def test_best_reeval_f64_matches_oracle(oracle, cuda):
    tab = _table(cuda, [(100, 30, 9, 4), (128, 100, 31, 4), (60, 10, 9, 4)])
    tab.init_population()
    for _ in range(3):
        tab.generation()
    rows, errs = tab.best_f64()
    fit = tab.fit[tab.cur].cpu().numpy()
    pop = tab.pop[tab.cur].cpu().numpy()
    for i, s in enumerate(tab.oracle_segments()):
        seg_fit = fit[s["row0"]:s["row0"] + s["P"]]
        assert int(rows[i]) == s["row0"] + int(np.argmin(seg_fit))
        ref = oracle.objective(s["func"], pop[int(rows[i]), :s["D"]], s["o"], s["M"])
        assert float(errs[i]) == pytest.approx(ref, rel=1e-12, abs=1e-12)


def test_no_device_error_flags(lib, cuda):
    import ctypes

    tab = _table(cuda, [(100, 30, 9, 4)])
    tab.init_population()
    tab.generation()
    bits = ctypes.c_uint32(0xFFFF)
    assert lib.speo_device_error_bits(ctypes.byref(bits)) == 0
    assert bits.value == 0


# ---------------------------------------------------------------------------------------------
# tcgen05 evaluation (each row y and M scaled by powers of two and split two ways into FP16,
# three products, FP32 accumulation): each rotated coordinate keeps ~2^-22 relative error per term
# (the dropped y_lo M_lo), so the rotated Rastrigin and sphere are held to the FP32 bar of 1e-5.
# ---------------------------------------------------------------------------------------------


@pytest.mark.parametrize("layout", [
    [(100, 30, 9, 4)] * 3,                              # config-1 islands, one 100-row tile each
    [(128, 100, 9, 4), (128, 100, 31, 4)],              # config-2 islands
    [(300, 50, 31, 4), (257, 50, 9, 4)],                # several tiles per segment, ragged last tile
    [(64, 10, 9, 4), (33, 16, 31, 4), (70, 2, 9, 4)],   # mixed small D, one launch
    [(200, 128, 9, 4)],                                 # largest D of the tensor-core path
])
def test_evaluate_tc_matches_oracle(oracle, cuda, layout):
    import torch
    from speo_gb300 import _lib

    tab = _table(cuda, layout, n_inst=len(layout), tile_rows=_lib.TILE_TC)
    tab.init_population()
    pop = tab.pop[tab.cur].cpu().numpy()
    pop_dev = tab.pop[tab.cur]
    for s in tab.oracle_segments()[:1]:           # include x = o (f = 0 exactly) and x ~ o
        pop[s["row0"], :s["D"]] = s["o"]
        pop[s["row0"] + 1, :s["D"]] = s["o"] + np.float32(1e-3)
    pop_dev.copy_(torch.from_numpy(pop))
    out = torch.full_like(tab.fit[0], float("nan"))
    tab.evaluate(use_tc=True, out=out)
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    worst = 0.0
    for s in tab.oracle_segments():
        r = slice(s["row0"], s["row0"] + s["P"])
        ref = oracle.evaluate_rows(s["func"], pop[r], s["D"], s["o"], s["M"])
        rel = np.abs(got[r] - ref) / np.maximum(np.abs(ref), 1e-30)
        worst = max(worst, float(np.max(np.where(ref > 1e-3, rel, 0))))
        _assert_fitness(got[r], ref, rtol=FIT_RTOL_F32, atol=FIT_ATOL_F32)
    assert got[0] == 0.0
    print(f"max relative error of the split-FP16 tensor-core fitness: {worst:.2e}")


@pytest.mark.parametrize("func", [9, 31])
def test_evaluate_tc_row_scaling_near_optimum(cuda, func):
    """Rows at x = o + d with |d| from 1e2 down to 1e-6 (and a row of mixed magnitudes): each row's
    power-of-two scale keeps the FP16 parts of small y normal, so the tensor-core fitness agrees with
    the CUDA-core FP32 evaluation of the same rows (the same y = x - o in FP32) to the FP32 bar."""
    import torch
    from speo_gb300 import _lib

    P, D = 128, 100
    tab = _table(cuda, [(P, D, func, 4)], n_inst=1, tile_rows=_lib.TILE_TC)
    tab_s = _table(cuda, [(P, D, func, 4)], n_inst=1, tile_rows=_lib.TILE_SIMT)
    tab.init_population()
    s = tab.oracle_segments()[0]
    rng = np.random.default_rng(17)
    pop = tab.pop[tab.cur].cpu().numpy()
    mags = 10.0 ** rng.uniform(-6, 2, P)
    for r in range(P):
        pop[r, :D] = (s["o"] + mags[r] * rng.standard_normal(D)).astype(np.float32)
    pop[0, :D] = (s["o"] + np.where(np.arange(D) % 2 == 0, 1e-5, 10.0)).astype(np.float32)
    tab.pop[tab.cur].copy_(torch.from_numpy(pop))
    tab_s.pop[tab_s.cur].copy_(torch.from_numpy(pop))
    tc_fit = torch.full_like(tab.fit[0], float("nan"))
    simt_fit = torch.full_like(tab_s.fit[0], float("nan"))
    tab.evaluate(use_tc=True, out=tc_fit)
    tab_s.evaluate(use_tc=False, out=simt_fit)
    torch.cuda.synchronize()
    a, b = tc_fit.cpu().numpy()[:P], simt_fit.cpu().numpy()[:P]
    assert np.all(np.isfinite(a))
    np.testing.assert_allclose(a, b, rtol=FIT_RTOL_F32, atol=0)


@pytest.mark.parametrize("layout", [[(128, 100, 9, 4)] * 3 + [(100, 30, 31, 6)], [(200, 50, 4, 4), (70, 64, 13, 2)]])
def test_generation_tc_matches_oracle(oracle, cuda, layout):
    """speo_generation_tc: one trial per target (the draws of speo_make_trials with k = 1),
    tcgen05 split-FP16 evaluation, strict-`<` selection, generation counter advanced; two
    generations. Selection decisions are checked against the FP64 oracle's fitness wherever the
    trial and the parent differ by more than the fitness bar."""
    import torch
    from speo_gb300 import _lib

    tab = _table(cuda, layout, n_inst=len(layout), tile_rows=_lib.TILE_TC)
    tab.init_population()
    trial = torch.zeros(tab.rows, tab.ld, device=cuda)
    tfit = torch.zeros(tab.rows, device=cuda)
    for g in range(2):
        pin, fin = tab.pop[tab.cur].cpu().numpy(), tab.fit[tab.cur].cpu().numpy()
        tab.tc_generation(trial, tfit)
        torch.cuda.synchronize()
        assert int(tab.gen[0].cpu()) == g + 1
        got_t, got_f = trial.cpu().numpy(), tfit.cpu().numpy()
        pout, fout = tab.pop[tab.cur].cpu().numpy(), tab.fit[tab.cur].cpu().numpy()
        for s in tab.oracle_segments():
            r0, P, D = s["row0"], s["P"], s["D"]
            seg = pin[r0:r0 + P]
            best = int(np.argmin(fin[r0:r0 + P]))
            cand = np.zeros_like(seg)
            d = oracle.philox_draws(s["seed"], g, pos0=r0, tag_hi=1 << 8)
            assert oracle.de_generate(cand, seg, tab.ld, D, np.arange(P), [s["CR"]], [s["F"]], [s["strategy"]], [best],
                                      s["lb"], s["ub"], d) == 0
            assert np.array_equal(got_t[r0:r0 + P, :D], cand[:, :D])
            ref = oracle.evaluate_rows(s["func"], cand, D, s["o"], s["M"])
            rtol, atol = _tc_tol(s["func"])
            _assert_fitness(got_f[r0:r0 + P], ref, rtol=rtol, atol=atol)
            win = got_f[r0:r0 + P] < fin[r0:r0 + P]
            parent = fin[r0:r0 + P].astype(np.float64)
            clear = np.abs(ref - parent) > 2 * (rtol * np.abs(ref) + atol)
            assert np.array_equal(win[clear], (ref < parent)[clear])
            assert np.array_equal(fout[r0:r0 + P], np.where(win, got_f[r0:r0 + P], fin[r0:r0 + P]))
            assert np.array_equal(pout[r0:r0 + P, :D], np.where(win[:, None], got_t[r0:r0 + P, :D], seg[:, :D]))


# The rotated bodies other than 9 / 31 on the tensor cores: the split product leaves each z_j
# with an absolute error of ~2^-18 |x - o| |m_j|, which the bodies amplify as the CUDA-core
# path's FP32 rounding is amplified (discus 3 weights z_0 by 1e6, Katsuura 12 and Weierstrass 6
# multiply z by up to 2^32 and 3^20 in their high harmonics). These bars held for the three
# products of two-way splits (max relative error 1.1e-3 for 3, 1.8e-3 for 12, 3.3e-4 for 6 and
# <= 1.6e-4 for the others at D = 10-100), which leave three times the error.
TC_TOL = {1: (2e-4, 1e-4), 2: (1e-4, 1e-4), 3: (4e-3, 1e-4), 4: (1e-4, 1e-4), 5: (5e-4, 1e-4), 6: (2e-3, 5e-2),
          7: (1e-4, 1e-4), 11: (3e-4, 5e-2), 12: (6e-3, 1e-4), 13: (1e-4, 5e-3), 14: (1e-4, 5e-3),
          15: (3e-4, 1e-4), 16: (1e-3, 1e-4)}
TC_FUNCS = sorted(TC_TOL)


def _tc_tol(fid):
    return TC_TOL.get(fid, (FIT_RTOL_F32, FIT_ATOL_F32))


@pytest.mark.parametrize("D", [10, 30, 64, 100])
def test_evaluate_tc_generic_functions(oracle, cuda, D):
    """speo_evaluate_tc on one table of every rotated CEC2014 body other than 9 / 31 (row
    accumulator epilogue, one tile row per thread) against the FP64 oracle."""
    import torch
    from speo_gb300 import _lib

    fids = TC_FUNCS
    tab = _table(cuda, [(150, D, f, 4) for f in fids], n_inst=len(fids), tile_rows=_lib.TILE_TC)
    tab.init_population()
    out = torch.full_like(tab.fit[0], float("nan"))
    tab.evaluate(use_tc=True, out=out)
    torch.cuda.synchronize()
    pop, got = tab.pop[tab.cur].cpu().numpy(), out.cpu().numpy()
    for s in tab.oracle_segments():
        r = slice(s["row0"], s["row0"] + s["P"])
        ref = oracle.evaluate_rows(s["func"], pop[r], s["D"], s["o"], s["M"])
        rtol, atol = _tc_tol(s["func"])
        _assert_fitness(got[r], ref, rtol=rtol, atol=atol)


# ---------------------------------------------------------------------------------------------
# island-resident epochs
# ---------------------------------------------------------------------------------------------
@pytest.mark.parametrize("cluster", [1, 2])
@pytest.mark.parametrize("layout,gens", [
    ([(100, 30, 9, 4)] * 8, 7),                         # config-1 islands
    ([(256, 50, 9, 4)] * 3, 5),                         # config-4 islands
    ([(40, 20, 31, 2), (64, 17, 9, 7), (5, 3, 31, 5)], 6),  # best-row strategies, tiny islands
    ([(50, 30, 10, 4), (50, 30, 4, 4), (50, 30, 12, 6), (50, 30, 16, 4)], 4),  # other CEC2014 ids
    ([(37, 30, 9, 4), (23, 30, 31, 6), (37, 30, 9, 2)], 3),  # odd populations (shared-memory padding)
])
def test_epoch_equals_per_generation_launches(oracle, cuda, layout, gens, cluster):
    """Island-resident epochs, one block or a two-block cluster per island, bit-identical to the
    same number of per-generation launches."""
    import torch

    a = _table(cuda, layout)
    b = _table(cuda, layout)
    a.init_population()
    b.init_population()
    assert a.epoch_fits()
    for _ in range(gens):
        a.generation()
    b.epoch(gens, cluster)
    torch.cuda.synchronize()
    assert np.array_equal(a.pop[a.cur].cpu().numpy(), b.pop[b.cur].cpu().numpy())
    assert np.array_equal(a.fit[a.cur].cpu().numpy(), b.fit[b.cur].cpu().numpy())
    assert int(b.gen.cpu()[0]) == gens and int(b.gen.cpu()[1]) == 0
    # and one more epoch against the oracle, generation by generation
    segs = b.oracle_segments()
    pop = b.pop[b.cur].cpu().numpy()
    fit = b.fit[b.cur].cpu().numpy()
    b.epoch(2, cluster)
    torch.cuda.synchronize()
    for g in range(2):
        pop, fit, trials, _, err = oracle.generation(segs, gens + g, pop, fit)
        assert err == 0
    got_pop = b.pop[b.cur].cpu().numpy()
    # The oracle evaluates in FP64 (its fitness values differ from FP32 in the last bits), so
    # selections can differ only where the two values straddle a parent's fitness: rows agree.
    same_rows = np.mean(np.all(got_pop == pop, axis=1))
    assert same_rows > 0.99, same_rows
