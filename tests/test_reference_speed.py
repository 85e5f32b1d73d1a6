"""The reference's own GPU generation loop beside this library's, on the same GPU and workload.

The reference's kernels (CUDA_EA_library/kernel_EA_CUDA.cu, kernel_DE_CUDA.cu, kernel_CEC2014_CUDA.cu,
compiled unmodified for sm_103a into oracle/_ref/*.fatbin; FP64 as shipped, FP32 through the
real = float shim) run DE_CUDA::Run's sequence (DE_CUDA.cc:200-216): best search, generate, F9
shift-and-rotate + Rastrigin, select, with the device synchronisation its CudaCheckError does
after each DE launch (kernel_DE_CUDA.cu:23-46). This library runs the same sequence through its
drop-in entry points with the same synchronisations, and as one speo_de_run_f32 / _f64 call.
Workload: one island of 6400 rows in 64 sub-islands of 100, D = 30, F9, DE/rand/1/bin CR 0.9
F 0.5. Prints one JSON line with the rates; asserts this library's loop is the faster one.
"""
from __future__ import annotations

import ctypes
import json
import time

import numpy as np
import pytest

import ref_kernels as rk

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_generation_loop_against_reference_kernels(lib, cuda, prec, capsys):
    if not rk.available(prec, ("de", "ea", "cec")):
        pytest.skip("reference fatbins not built (needs the reference sources at build time)")
    import torch
    from speo_gb300 import _lib
    from speo_gb300.instances import make_instance

    f64 = prec == "f64"
    dt = torch.float64 if f64 else torch.float32
    es = 8 if f64 else 4
    Pop = _lib.PopulationF64 if f64 else _lib.PopulationF32
    PI = _lib.ProblemInfoF64 if f64 else _lib.ProblemInfoF32
    DI = _lib.DEInfoF64 if f64 else _lib.DEInfoF32
    real = ctypes.c_double if f64 else ctypes.c_float
    P, D, nsub, G, seed = 6400, 30, 64, 200, 4321
    ld, S = 32, P // nsub
    drv = rk.Driver()
    torch.zeros(1, device=cuda)
    de_fat, ea_fat, cec_fat = (rk.REF_DIR / f"ref_{k}_{prec}.fatbin" for k in ("de", "ea", "cec"))
    o, M = make_instance(77, D)
    mt = np.zeros((ld, D), dtype=np.float64)          # the reference's B operand: mt[k][j] = M[j][k]
    mt[:D] = M.T
    sh = np.zeros(ld, dtype=np.float64)
    sh[:D] = o
    d_mt, d_sh = torch.from_numpy(mt).to(cuda, dt), torch.from_numpy(sh).to(cuda, dt)
    info = (DI * nsub)(*[DI(0.9, 0.5, 4, S) for _ in range(nsub)])
    d_info = torch.frombuffer(bytearray(bytes(info)), dtype=torch.uint8).to(cuda)
    problem = PI(D, 9, 1, 0, seed, 0, 0, 100.0, -100.0)
    rates = {}

    def buffers():
        z = lambda *s: torch.zeros(*s, dtype=dt, device=cuda)
        b = dict(pop=z(P, ld), cand=z(P, ld), pfit=z(P), cfit=z(P), rot=z(P, ld),
                 perm=torch.arange(P, dtype=torch.int32, device=cuda),
                 best=torch.zeros(max(nsub, 32), dtype=torch.int32, device=cuda))
        b["P"] = Pop(b["pop"].data_ptr(), b["pfit"].data_ptr())
        b["C"] = Pop(b["cand"].data_ptr(), b["cfit"].data_ptr())
        b["ii"] = _lib.IslandInfo(P, nsub, b["perm"].data_ptr())
        return b

    # ---- the reference's kernels -------------------------------------------------------------
    b = buffers()
    states = torch.zeros(P * 32 * rk.CURAND_STATE_BYTES // 4 + 64, dtype=torch.int32, device=cuda)
    grid, block = rk.de_config(P)
    f_best, f_gen, f_sel = (drv.function(de_fat, k) for k in (rk.K_BEST, rk.K_GEN, rk.K_SEL))
    f_sr, f_f8 = drv.function(cec_fat, rk.K_SR[prec]), drv.function(cec_fat, rk.K_F8[prec])
    drv.launch(drv.function(ea_fat, rk.K_SETUP), grid, block, [ctypes.c_void_p(states.data_ptr()), ctypes.c_int(seed)])
    drv.launch(drv.function(ea_fat, rk.K_INIT), grid, block, [b["P"], ctypes.c_void_p(states.data_ptr()), problem])
    vp = lambda t: ctypes.c_void_p(t.data_ptr())

    def ref_evaluate(x, fit):  # F9 -> f8 -> ShiftAndRotation + global_f8 (kernel_CEC2014_CUDA.cu:1005-1018, 224-235)
        i = ctypes.c_int
        drv.launch(f_sr, ((D - 1) // 16 + 1, (P - 1) // 16 + 1, 1), (16, 16, 1),
                   [vp(x), vp(d_mt), vp(b["rot"]), vp(d_sh), i(P), i(ld), i(ld), i(D), i(P), i(ld), i(1)],
                   smem=16 * 16 * es, sync=False)
        drv.launch(f_f8, (1, P // 16, 1), (32, 16, 1),
                   [vp(fit), vp(b["rot"]), i(D), i(D), real(0.0), real(0.0512), real(1.0), real(0.0)],
                   smem=es * 32 * 16, sync=False)

    def ref_generation():
        drv.launch(f_best, (nsub, 1, 1), (32, 1, 1), [vp(b["best"]), b["P"], b["ii"], problem])
        drv.launch(f_gen, grid, block, [b["C"], b["P"], vp(b["best"]), b["ii"], vp(d_info), vp(states), problem])
        ref_evaluate(b["cand"], b["cfit"])
        drv.launch(f_sel, grid, block, [b["P"], b["C"], problem])

    ref_evaluate(b["pop"], b["pfit"])
    for _ in range(5):
        ref_generation()
    t0 = time.perf_counter()
    for _ in range(G):
        ref_generation()
    drv.check(drv.cu.cuCtxSynchronize(), "sync")
    rates["reference_kernels"] = P * G / (time.perf_counter() - t0)
    ref_best = float(b["pfit"].min())

    # ---- this library: the drop-in calls with the same synchronisations ------------------------
    b = buffers()
    rng = torch.zeros(16, dtype=torch.int32, device=cuda)
    sfx = "" if f64 else "_f32"
    init, gen, sel = (getattr(lib, n + sfx) for n in ("API_Initilize", "API_DE_GenerateNewPopulation",
                                                      "API_DE_SelectSurvival"))
    ev = getattr(lib, "API_evaluateFitness" + sfx)
    _lib.check(init(b["P"], rng.data_ptr(), b["ii"], problem), "API_Initilize")
    eargs = (d_sh.data_ptr(), d_mt.data_ptr(), None, None, None, None, P, D, 0.0, 9)
    ev(b["pfit"].data_ptr(), None, None, b["pop"].data_ptr(), *eargs)

    def generation():
        _lib.check(gen(b["C"], b["P"], b["best"].data_ptr(), b["ii"], d_info.data_ptr(), rng.data_ptr(), problem), "gen")
        _lib.check(lib.API_CheckCUDAError(), "sync")
        ev(b["cfit"].data_ptr(), None, None, b["cand"].data_ptr(), *eargs)
        _lib.check(sel(b["P"], b["C"], b["ii"], problem), "sel")
        _lib.check(lib.API_CheckCUDAError(), "sync")

    for _ in range(5):
        generation()
    t0 = time.perf_counter()
    for _ in range(G):
        generation()
    rates["library_dropin_calls"] = P * G / (time.perf_counter() - t0)
    # the same loop as one library call
    h = torch.zeros(P, dtype=dt).pin_memory()
    de_run = getattr(lib, "speo_de_run_" + prec)
    run = lambda k: _lib.check(de_run(b["P"], b["C"], rng.data_ptr(), b["ii"], d_info.data_ptr(), b["best"].data_ptr(),
                                      problem, d_sh.data_ptr(), d_mt.data_ptr(), None, k, h.data_ptr(), 0, None), "run")
    run(25)
    t0 = time.perf_counter()
    run(G * 5)
    rates["library_speo_de_run_" + prec] = P * G * 5 / (time.perf_counter() - t0)
    with capsys.disabled():
        print("\n" + json.dumps({"reference_speed": {"precision": prec, "rows": P, "dim": D, "subislands": nsub,
                                                     "function": 9, "evals_per_s": rates,
                                                     "reference_best_after_205_gens": ref_best}}))
    assert rates["library_dropin_calls"] > rates["reference_kernels"]


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_published_configuration_against_reference_kernels(lib, cuda, prec, capsys):
    """The reference's published configuration (CEC2014 F23, D = 100, one island of 4096 rows,
    DE/rand/1/bin CR 0.9 F 0.5) through the reference's own kernels on this GPU: best search,
    generate, CompFunc1's launch sequence (4 x ShiftAndRotation + f4/f1/f2/f3, Shift + f1, CalW,
    CombineFitness; kernel_CEC2014_CUDA.cu:1416-1451), select, with the reference's
    synchronisations; beside this library's drop-in calls (same synchronisations) and
    speo_de_run_f32 / _f64."""
    if not rk.available(prec, ("de", "ea", "cec")):
        pytest.skip("reference fatbins not built (needs the reference sources at build time)")
    import torch
    from speo_gb300 import _lib
    from speo_gb300.instances import make_instance_multi

    f64 = prec == "f64"
    dt = torch.float64 if f64 else torch.float32
    es = 8 if f64 else 4
    Pop = _lib.PopulationF64 if f64 else _lib.PopulationF32
    PI = _lib.ProblemInfoF64 if f64 else _lib.ProblemInfoF32
    DI = _lib.DEInfoF64 if f64 else _lib.DEInfoF32
    real = ctypes.c_double if f64 else ctypes.c_float
    P, D, nsub, G, seed, fid, nc = 4096, 100, 1, 20, 99, 23, 5
    ld = 128
    drv = rk.Driver()
    torch.zeros(1, device=cuda)
    de_fat, ea_fat, cec_fat = (rk.REF_DIR / f"ref_{k}_{prec}.fatbin" for k in ("de", "ea", "cec"))
    o, M, S = make_instance_multi(5, D, fid)
    rot = np.zeros((nc, ld, D), dtype=np.float64)
    rot[:, :D] = M.transpose(0, 2, 1)
    sh = np.zeros((nc, ld), dtype=np.float64)
    sh[:, :D] = o
    d_rot, d_sh = torch.from_numpy(rot).to(cuda, dt), torch.from_numpy(sh).to(cuda, dt)
    info = (DI * nsub)(DI(0.9, 0.5, 4, P))
    d_info = torch.frombuffer(bytearray(bytes(info)), dtype=torch.uint8).to(cuda)
    problem = PI(D, fid, 1, 0, seed, 0, 0, 100.0, -100.0)
    vp = lambda t: ctypes.c_void_p(t.data_ptr())
    i_ = ctypes.c_int
    rates = {}

    def buffers():
        z = lambda *s: torch.zeros(*s, dtype=dt, device=cuda)
        b = dict(pop=z(P, ld), cand=z(P, ld), pfit=z(P), cfit=z(P), rotd=z(P, ld), tmp=z(nc * P), wi=z(P * nc),
                 perm=torch.arange(P, dtype=torch.int32, device=cuda),
                 best=torch.zeros(32, dtype=torch.int32, device=cuda))
        b["P"] = Pop(b["pop"].data_ptr(), b["pfit"].data_ptr())
        b["C"] = Pop(b["cand"].data_ptr(), b["cfit"].data_ptr())
        b["ii"] = _lib.IslandInfo(P, nsub, b["perm"].data_ptr())
        return b

    # ---- the reference's kernels -------------------------------------------------------------
    b = buffers()
    sigma = torch.tensor([10.0, 20.0, 30.0, 40.0, 50.0], dtype=dt, device=cuda)
    states = torch.zeros(P * 32 * rk.CURAND_STATE_BYTES // 4 + 64, dtype=torch.int32, device=cuda)
    grid, block = rk.de_config(P)
    f_best, f_gen, f_sel = (drv.function(de_fat, k) for k in (rk.K_BEST, rk.K_GEN, rk.K_SEL))
    f_sr = drv.function(cec_fat, rk.K_SR[prec])
    fn = {n: drv.function(cec_fat, rk.K_FN[prec][n]) for n in (1, 2, 3, 4)}
    f_shift, f_calw, f_comb = (drv.function(cec_fat, k[prec]) for k in (rk.K_SHIFT, rk.K_CALW, rk.K_COMBINE))
    drv.launch(drv.function(ea_fat, rk.K_SETUP), grid, block, [vp(states), ctypes.c_int(seed)])
    drv.launch(drv.function(ea_fat, rk.K_INIT), grid, block, [b["P"], vp(states), problem])
    cfg_grid, cfg_block, cfg_smem = (1, P // 16, 1), (32, 16, 1), es * 32 * 16   # Configuration (:56-73)
    sr_grid = ((D - 1) // 16 + 1, (P - 1) // 16 + 1, 1)
    tmp_ptr = lambda c: ctypes.c_void_p(b["tmp"].data_ptr() + c * P * es)
    sh_ptr = lambda c: ctypes.c_void_p(d_sh.data_ptr() + c * ld * es)
    rot_ptr = lambda c: ctypes.c_void_p(d_rot.data_ptr() + c * ld * D * es)
    body = [(4, 1.0, 2.048 / 100, 1.0, 0.0), (1, 0.0, 1.0, 1e-6, 100.0), (2, 0.0, 1.0, 1e-26, 200.0),
            (3, 0.0, 1.0, 1e-6, 300.0), (1, 0.0, 1.0, 1e-6, 400.0)]

    def ref_evaluate(x, fit):  # CompFunc1 (kernel_CEC2014_CUDA.cu:1416-1451)
        for c, (k, shift_v, rate, wi, bias) in enumerate(body):
            if c < 4:
                drv.launch(f_sr, sr_grid, (16, 16, 1), [vp(x), rot_ptr(c), vp(b["rotd"]), sh_ptr(c), i_(P), i_(ld),
                                                        i_(ld), i_(D), i_(P), i_(ld), i_(1)],
                           smem=16 * 16 * es, sync=False)
            else:
                drv.launch(f_shift, cfg_grid, cfg_block, [vp(b["rotd"]), vp(x), sh_ptr(c), i_(P), i_(D), i_(1)],
                           sync=False)
            drv.launch(fn[k], cfg_grid, cfg_block, [tmp_ptr(c), vp(b["rotd"]), i_(D), i_(D), real(shift_v),
                                                    real(rate), real(wi), real(bias)], smem=cfg_smem, sync=False)
        drv.launch(f_calw, cfg_grid, cfg_block, [vp(b["wi"]), vp(x), vp(d_sh), vp(sigma), i_(D), i_(nc)],
                   smem=cfg_smem, sync=False)
        drv.launch(f_comb, (P // 512, 1, 1), (512, 1, 1), [vp(fit), vp(b["tmp"]), i_(nc), vp(b["wi"]), i_(P),
                                                           real(1.0), real(0.0)], sync=False)

    def ref_generation():
        drv.launch(f_best, (nsub, 1, 1), (32, 1, 1), [vp(b["best"]), b["P"], b["ii"], problem])
        drv.launch(f_gen, grid, block, [b["C"], b["P"], vp(b["best"]), b["ii"], vp(d_info), vp(states), problem])
        ref_evaluate(b["cand"], b["cfit"])
        drv.launch(f_sel, grid, block, [b["P"], b["C"], problem])

    ref_evaluate(b["pop"], b["pfit"])
    drv.check(drv.cu.cuCtxSynchronize(), "sync")
    for _ in range(3):
        ref_generation()
    t0 = time.perf_counter()
    for _ in range(G):
        ref_generation()
    drv.check(drv.cu.cuCtxSynchronize(), "sync")
    rates["reference_kernels"] = P * G / (time.perf_counter() - t0)

    # ---- this library ------------------------------------------------------------------------
    b = buffers()
    rng = torch.zeros(16, dtype=torch.int32, device=cuda)
    sfx = "" if f64 else "_f32"
    init, gen, sel = (getattr(lib, n + sfx) for n in ("API_Initilize", "API_DE_GenerateNewPopulation",
                                                      "API_DE_SelectSurvival"))
    ev = getattr(lib, "API_evaluateFitness" + sfx)
    _lib.check(init(b["P"], rng.data_ptr(), b["ii"], problem), "API_Initilize")
    eargs = (d_sh.data_ptr(), d_rot.data_ptr(), None, None, None, None, P, D, 0.0, fid)
    ev(b["pfit"].data_ptr(), None, None, b["pop"].data_ptr(), *eargs)

    def generation():
        _lib.check(gen(b["C"], b["P"], b["best"].data_ptr(), b["ii"], d_info.data_ptr(), rng.data_ptr(), problem), "gen")
        _lib.check(lib.API_CheckCUDAError(), "sync")
        ev(b["cfit"].data_ptr(), None, None, b["cand"].data_ptr(), *eargs)
        _lib.check(sel(b["P"], b["C"], b["ii"], problem), "sel")
        _lib.check(lib.API_CheckCUDAError(), "sync")

    for _ in range(3):
        generation()
    t0 = time.perf_counter()
    for _ in range(G):
        generation()
    rates["library_dropin_calls"] = P * G / (time.perf_counter() - t0)
    h = torch.zeros(P, dtype=dt).pin_memory()
    de_run = getattr(lib, "speo_de_run_" + prec)
    run = lambda k: _lib.check(de_run(b["P"], b["C"], rng.data_ptr(), b["ii"], d_info.data_ptr(), b["best"].data_ptr(),
                                      problem, d_sh.data_ptr(), d_rot.data_ptr(), None, k, h.data_ptr(), 0, None),
                               "run")
    run(10)
    t0 = time.perf_counter()
    run(G * 5)
    rates["library_speo_de_run_" + prec] = P * G * 5 / (time.perf_counter() - t0)
    with capsys.disabled():
        print("\n" + json.dumps({"published_configuration_speed": {"precision": prec, "rows": P, "dim": D,
                                                                   "function": fid, "evals_per_s": rates}}))
    if not f64:
        assert rates["library_dropin_calls"] > rates["reference_kernels"]

