"""Benchmark of the island-model DE generation loop on GB300.

Workload (the island-model configuration the headline metric is quoted on): 64 islands x
P = 100, D = 30, rotated Rastrigin z = M (0.0512 (x - o)) (CEC2014 F9 form, f - f*), F = 0.5,
CR = 0.9, DE/rand/1/bin, ring migration of each island's best 5 into the next island's worst
5 every 50 generations; seeded synthetic o ~ U[-80, 80]^30 and Haar M.

A step is one generation over all islands (6400 exact evaluations). `value` is exact
evaluations/s over the whole job with the population resident in HBM; `e2e` is the same rate
through the reference-shaped C ABI (API_DE_GenerateNewPopulation_f32 / API_evaluateFitness_f32
/ API_DE_SelectSurvival_f32) with host buffers, the initial upload and a per-generation
fitness read-back inside the timed region.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl speo|reference]
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parent
sys.path.insert(0, str(REPO / "speo-gpu-single-control_gb300"))
sys.path.insert(0, str(REPO / "oracle"))

METRIC = "exact-eval gens/s & evals/s to 1e-8 error: surrogate vs plain DE, same GB300"
N_ISLANDS, POP, DIM, FUNC = 64, 100, 30, 9
INTERVAL, MIGRANTS = 50, 5
SEED = 9 * 2  # run_seed(node 1, function 9, run 1) = (1 + 9) * (1 + 9) is used below


def run_seed() -> int:
    from speo_gb300.instances import run_seed as rs

    return rs(1, FUNC, 1)


def peaks() -> dict:
    p = REPO / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": d["hbm_gbs"], "src": "measured"}
    return {"hbm_gbs": 6800.0, "src": "fallback"}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except FileNotFoundError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            out, _ = self.proc.communicate(timeout=10)
            self.lines = [ln for ln in out.splitlines() if ln.strip()]

    def summary(self) -> dict:
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in getattr(self, "lines", []):
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for name, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def flush_l2(buf) -> None:
    buf.add_(1.0)   # writes 512 MB, > 4x the 129 MB L2


def island_specs(rank: int):
    """Config 1's island ring for one rank: under torchrun each rank runs an independent replica
    of the ring (its own Philox seeds, the same instance), so per-GPU work is fixed as N grows."""
    from speo_gb300.device import SegmentSpec
    from speo_gb300.instances import make_instance

    seed = run_seed()
    inst = [make_instance(seed, DIM)]
    specs = [SegmentSpec(pop_size=POP, dim=DIM, func_id=FUNC, instance=0, seed=seed * 1000003 + rank,
                         ring_next=(i + 1) % N_ISLANDS) for i in range(N_ISLANDS)]
    return specs, inst


def island_table(device: str, rank: int):
    from speo_gb300.device import SegmentTable

    specs, inst = island_specs(rank)
    # tiles of 50 rows: two balanced tiles per island
    return SegmentTable(specs, inst, tile_rows=50, device=device)


def max_over_ranks(value: float, device: str, world: int) -> float:
    """The largest of the ranks' values (the job's time is its slowest rank's)."""
    if world <= 1:
        return value
    import torch

    t = torch.tensor([value], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def capture(torch, fn):
    """CUDA graph of fn() (fn run once outside capture first to set kernel attributes)."""
    g = torch.cuda.CUDAGraph()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        fn()
        with torch.cuda.graph(g, stream=s):
            fn()
    torch.cuda.current_stream().wait_stream(s)
    return g


def capture_epoch(tab, torch):
    """One CUDA graph = INTERVAL generations + the ring migration. Islands that fit one block's
    shared memory run the epoch as one resident launch; otherwise INTERVAL fused launches (an
    even number, so the double buffers end where they started)."""
    assert INTERVAL % 2 == 0
    if tab.epoch_fits():
        def epoch():
            tab.epoch(INTERVAL)
            tab.migrate(MIGRANTS)
        return capture(torch, epoch), "resident"

    def epoch():
        for _ in range(INTERVAL):
            tab.generation()
        tab.migrate(MIGRANTS)
    return capture(torch, epoch), "per-generation"


def time_graph(torch, graph, reps, flush):
    flush_l2(flush)
    s = torch.cuda.current_stream()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(s)
    for _ in range(reps):
        graph.replay()
    b.record(s)
    torch.cuda.synchronize()
    return a.elapsed_time(b) / reps


def bench_speo(args) -> dict:
    import torch

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = f"cuda:{local}"
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    from speo_gb300 import _lib

    L = _lib.load()
    tab = island_table(dev, rank)
    tab.init_population()
    graph, mode = capture_epoch(tab, torch)
    epochs_w = max(1, (args.warmup + INTERVAL - 1) // INTERVAL)
    epochs = max(1, (args.steps + INTERVAL - 1) // INTERVAL)
    steps = epochs * INTERVAL
    for _ in range(epochs_w):
        graph.replay()
    torch.cuda.synchronize()
    flush = torch.empty(128 * 1024 * 1024, dtype=torch.float32, device=dev)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(epochs)]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        for i in range(epochs):
            flush_l2(flush)                        # L2 flushed between timed epochs
            ev[i][0].record()
            graph.replay()
            ev[i][1].record()
        torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    ms = max_over_ranks(sum(a.elapsed_time(b) for a, b in ev), dev, world)
    evals_per_step = N_ISLANDS * POP
    value = evals_per_step * steps * world / (ms / 1e3)

    # ---- dominant kernel: average duration of one launch (graphs of back-to-back launches) ------
    alg_bytes_gen = evals_per_step * (5 * DIM * 4 + 2 * 4)   # 4 row reads + 1 row write + 2 fitness
    reps = 40
    if mode == "resident":
        kg = capture(torch, lambda: tab.epoch(INTERVAL))
        launch_ms = time_graph(torch, kg, reps, flush)
        if 2 * N_ISLANDS <= torch.cuda.get_device_properties(dev).multi_processor_count:
            kernel = (f"k_island_epoch2<1> ({INTERVAL} generations per launch, each island resident in the "
                      f"shared memory of a two-block cluster: {2 * N_ISLANDS} blocks)")
        else:
            kernel = f"k_island_epoch<1> ({INTERVAL} generations per launch, islands resident in shared memory)"
        alg_bytes = alg_bytes_gen * INTERVAL
    else:
        kg = capture(torch, lambda: [tab.generation() for _ in range(INTERVAL)])
        launch_ms = time_graph(torch, kg, reps, flush) / INTERVAL
        kernel = "k_generation<1> (fused generate+evaluate+select)"
        alg_bytes = alg_bytes_gen
    # the per-generation fused kernel on the same islands, for comparison
    pg = capture(torch, lambda: [tab.generation() for _ in range(INTERVAL)])
    per_gen_us = time_graph(torch, pg, 10, flush) / INTERVAL * 1e3
    pk = peaks()
    achieved = alg_bytes / (launch_ms / 1e3) / 1e9
    rows, errs = tab.best_f64()
    best_err = float(errs.min().item())

    out = {
        "metric": METRIC, "value": value, "unit": "evals/s", "n_gpus": world, "steps": steps,
        "warmup": epochs_w * INTERVAL, "ms_per_step": ms / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp32", "data": "synthetic",
        "config": {"workload": "island model: 64 islands x P=100, D=30, rotated Rastrigin (F9 form), "
                               "DE/rand/1/bin F=0.5 CR=0.9, ring best-5 -> worst-5 every 50 generations",
                   "islands": N_ISLANDS, "pop_size": POP, "dim": DIM, "migration_interval": INTERVAL,
                   "migrants": MIGRANTS, "step": "one generation over all islands (6400 exact evaluations)",
                   "l2": "flushed (512 MB write) before each timed 50-generation epoch; the population "
                         "(1.5 MB) stays L2-resident within an epoch as in a real run",
                   "graph": "one CUDA graph per epoch: the 50 generations (one island-resident launch, or 50 "
                            "fused launches when an island does not fit shared memory) + 2 migration launches"},
        "gens_per_s": steps * world / (ms / 1e3) / world,
        "best_error_f64_after_run": best_err,
        "roofline": {"kernel": kernel, "bound": "hbm",
                     "achieved": achieved, "peak": pk["hbm_gbs"], "unit": "GB/s", "frac": achieved / pk["hbm_gbs"],
                     "traffic": EPOCH_TRAFFIC_BYTES if mode == "resident" else None,
                     "traffic_src": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one k_island_epoch2 launch "
                                    "at this workload (the island is read once per launch; its writes stay in L2)"
                     if mode == "resident" else None,
                     "peak_src": pk["src"],
                     "alg_bytes_per_launch": alg_bytes, "launch_us": launch_ms * 1e3,
                     "note": "achieved = algorithmic bytes of a streaming generation (5 D s + 2 s per "
                             "individual-generation) / launch time"},
        "per_generation_kernel_us": per_gen_us,
        "epoch_mode": mode,
        "gpu_launches": epochs * ((1 if mode == "resident" else INTERVAL) + 2),
        "clocks": clk.summary(),
    }
    if rank != 0:  # the remaining sections are single-GPU measurements: rank 0 alone
        return out
    if not args.no_ops:
        out["operators_bandwidth_scale"] = bench_operators(L, dev, torch, pk)
    if not args.no_configs:
        out["config2_precision"] = bench_config2(L, dev, torch, flush)
        out["config3_batched"] = bench_config3(L, dev, torch, flush)
        out["config4_surrogate_vs_plain"] = bench_config4(L, dev, torch, args.c4_gens)
        out["surrogate_mlp"] = bench_mlp(L, dev, torch)
        out["published_config"] = bench_published(L, dev, torch)
    if not args.no_e2e:
        out["e2e"] = bench_e2e(L, dev, torch, args)
        # the same end-to-end loop in the reference's shipped precision
        out["e2e_fp64"] = bench_e2e(L, dev, torch, args, f64=True)
    if rank == 0 and not args.no_cpu:
        out["cpu_baseline"] = cpu_baseline(sample_s=args.cpu_sample_s)
    return out


def bench_operators(L, dev, torch, pk, n_isl: int = 16384) -> dict:
    """Operator kernels on a bandwidth-scale population (measurement-only variant): 16384 islands
    x P = 128, D = 100 = 2^21 rows, 0.84 GB per FP32 buffer (> 6x L2), so every launch streams
    from HBM. Each kernel is timed alone with CUDA events (median of several launches, L2
    flushed before each); achieved = algorithmic bytes / time."""
    from speo_gb300 import _lib
    from speo_gb300.device import SegmentSpec, SegmentTable
    from speo_gb300.instances import make_instance

    P, D = 128, 100
    inst = [make_instance(run_seed() + 1, D)]
    specs = [SegmentSpec(pop_size=P, dim=D, func_id=FUNC, instance=0, seed=77 + i) for i in range(n_isl)]
    tab = SegmentTable(specs, inst, tile_rows=_lib.TILE_SIMT, device=dev)
    tab_tc = SegmentTable(specs, inst, tile_rows=_lib.TILE_TC, device=dev)
    tab.init_population()
    rows = tab.rows
    flush = torch.empty(128 * 1024 * 1024, dtype=torch.float32, device=dev)
    s = 4

    def timed(fn, reps=7):
        fn()
        ts = []
        for _ in range(reps):
            flush_l2(flush)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            fn()
            b.record()
            torch.cuda.synchronize()
            ts.append(a.elapsed_time(b))
        return float(np.median(ts)) / 1e3

    out = {"workload": f"{n_isl} islands x P={P}, D={D} ({rows} rows, {rows * D * s / 1e9:.2f} GB per buffer)",
           "peak_gbs": pk["hbm_gbs"], "kernels": {}}

    def rec(name, sec, bytes_):
        gbs = bytes_ / sec / 1e9
        out["kernels"][name] = {"us": sec * 1e6, "alg_bytes": bytes_, "achieved_gbs": gbs,
                                "frac": gbs / pk["hbm_gbs"]}

    # fused generation (CUDA-core rotation), segment layout ld = 100
    rec("k_generation<4> fused generate+evaluate+select", timed(lambda: tab.generation()), rows * (5 * D * s + 2 * s))
    # tcgen05 evaluation: read D floats, write 1
    tab_tc.pop[0].copy_(tab.pop[tab.cur])
    out_fit = torch.empty(rows, device=dev)
    rec("k_evaluate_tc (TMA + tcgen05 BF16x3)", timed(lambda: tab_tc.evaluate(which=0, use_tc=True, out=out_fit)),
        rows * (D * s + s))
    rec("k_eval_seg<4> (CUDA-core evaluation)", timed(lambda: tab.evaluate(which=tab.cur, out=out_fit)),
        rows * (D * s + s))
    # drop-in operators in the reference layout (ld = np2 = 128), FP32
    ld = 128
    pop = torch.zeros(rows, ld, device=dev)
    pop[:, :D] = tab.pop[tab.cur][:, :D]
    cand = torch.zeros(rows, ld, device=dev)
    pfit = tab.fit[tab.cur].clone()
    cfit = torch.empty(rows, device=dev)
    rng_state = torch.zeros(16, dtype=torch.int32, device=dev)
    perm = torch.arange(rows, dtype=torch.int32, device=dev)
    best = torch.zeros(n_isl, dtype=torch.int32, device=dev)
    info = (_lib.DEInfoF32 * n_isl)(*[_lib.DEInfoF32(0.9, 0.5, 4, P) for _ in range(n_isl)])
    d_info = torch.frombuffer(bytearray(bytes(info)), dtype=torch.uint8).to(dev)
    ii = _lib.IslandInfo(rows, n_isl, perm.data_ptr())
    pi = _lib.ProblemInfoF32(D, FUNC, 1, 0, 5, 0, 0, 100.0, -100.0)
    Pp = _lib.PopulationF32(pop.data_ptr(), pfit.data_ptr())
    Cp = _lib.PopulationF32(cand.data_ptr(), cfit.data_ptr())
    L.speo_set_stream(ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    _lib.check(L.API_Initilize_f32(Cp, rng_state.data_ptr(), ii, pi), "API_Initilize_f32")
    rec("API_DE_GenerateNewPopulation_f32 (best search + generate)",
        timed(lambda: L.API_DE_GenerateNewPopulation_f32(Cp, Pp, best.data_ptr(), ii, d_info.data_ptr(),
                                                         rng_state.data_ptr(), pi)),
        rows * (4 * D * s + D * s) + rows * s)
    # selection moves a row only where the trial wins: bytes = both fitness values for every row
    # + (read trial row + write it + write fitness) for each winner, counted from this state
    L.API_evaluateFitness_f32(cfit.data_ptr(), None, None, cand.data_ptr(), tab.inst_shift[0].data_ptr(),
                              tab.inst_rot[0].data_ptr(), None, None, None, None, rows, D, 0.0, FUNC)
    torch.cuda.synchronize()
    pfit0 = pfit.clone()
    winners = int((cfit < pfit0).sum().item())

    def select_once():
        pfit.copy_(pfit0)
        L.API_DE_SelectSurvival_f32(Pp, Cp, ii, pi)

    t_copy = timed(lambda: pfit.copy_(pfit0))
    rec("API_DE_SelectSurvival_f32", max(timed(select_once) - t_copy, 1e-9),
        rows * 2 * s + winners * (2 * D * s + s))
    out["kernels"]["API_DE_SelectSurvival_f32"]["winners"] = winners
    L.speo_set_stream(None)
    _lib.check(L.API_CheckCUDAError(), "operators")
    del tab, tab_tc, pop, cand
    torch.cuda.empty_cache()
    return out


def bench_config2(L, dev, torch, flush) -> dict:
    """Config 2: 256 islands x 128, D = 100, mixed objectives; the rotation runs on the tcgen05
    tensor cores in BF16x3 (trial generation, tensor-core evaluation and selection per generation,
    20 generations per CUDA graph). Precision: tensor-core and CUDA-core FP32 fitness of 4096
    sampled rows against the FP64 oracle; FP64 re-evaluation of every island's best."""
    import speo_oracle
    from speo_gb300 import _lib
    from speo_gb300 import workloads as w

    specs, inst = w.config2_specs(256)
    tab = w.table(specs, inst, device=dev, tile_rows=_lib.TILE_TC)
    tab.init_population()
    trial = torch.zeros(tab.rows, tab.ld, device=dev)
    tfit = torch.zeros(tab.rows, device=dev)
    G = 20
    g = capture(torch, lambda: [tab.tc_generation(trial, tfit) for _ in range(G)])
    for _ in range(2):
        g.replay()
    ms = time_graph(torch, g, 5, flush) / G
    fit_tc = torch.empty(tab.rows, device=dev)
    fit_cc = torch.empty(tab.rows, device=dev)
    tab.evaluate(use_tc=True, out=fit_tc)
    tab.evaluate(out=fit_cc)
    torch.cuda.synchronize()
    pop = tab.pop[tab.cur].cpu().numpy()
    rng = np.random.default_rng(2)
    sample = rng.choice(tab.rows, 4096, replace=False)
    ref = np.empty(len(sample))
    owner = np.repeat(np.arange(len(specs)), [sp.pop_size for sp in specs])
    for j, r in enumerate(sample):
        sp = specs[owner[r]]
        o, M = inst[sp.instance]
        ref[j] = speo_oracle.evaluate_rows(sp.func_id, pop[r:r + 1], sp.dim, o, M)[0]
    rel_tc = np.abs(fit_tc.cpu().numpy()[sample] - ref) / np.maximum(np.abs(ref), 1e-30)
    rel_cc = np.abs(fit_cc.cpu().numpy()[sample] - ref) / np.maximum(np.abs(ref), 1e-30)
    rows, errs = tab.best_f64()
    return {"workload": "256 islands x P=128, D=100, per island rotated sphere or rotated Rastrigin (seeded), "
                        "BF16x3 tcgen05 evaluation",
            "ms_per_generation": ms, "gens_per_s": 1e3 / ms, "evals_per_s": tab.rows / (ms / 1e3),
            "launches_per_generation": 3,
            "fitness_rel_err_vs_fp64": {"tcgen05_bf16x3": {"max": float(rel_tc.max()), "median": float(np.median(rel_tc)),
                                                           "p99": float(np.quantile(rel_tc, 0.99))},
                                        "cuda_core_fp32": {"max": float(rel_cc.max()), "median": float(np.median(rel_cc)),
                                                           "p99": float(np.quantile(rel_cc, 0.99))},
                                        "rows_sampled": int(len(sample))},
            "best_error_f64_min_over_islands": float(errs.min().item())}


def bench_config3(L, dev, torch, flush) -> dict:
    """Config 3: 1024 independent runs with D ~ U{10,30,50,100}, P ~ U[50,200], each with its own
    instance and objective; one launch per generation (the mixed-class kernel), 20 generations per
    CUDA graph. The tile size is tuned by measurement over the candidates."""
    from speo_gb300 import workloads as w

    specs, inst = w.config3_specs(1024)
    evals = sum(sp.pop_size for sp in specs)
    tuned = {}
    for tile in (32, 48, 64):
        tab = w.table(specs, inst, device=dev, tile_rows=tile)
        tab.init_population()
        g = capture(torch, lambda: [tab.generation() for _ in range(20)])
        g.replay()
        tuned[tile] = time_graph(torch, g, 5, flush) / 20
    best = min(tuned, key=tuned.get)
    ms = tuned[best]
    return {"workload": f"1024 runs, D in {{10,30,50,100}}, P in [50,200] ({evals} rows), mixed objectives",
            "ms_per_generation": ms, "gens_per_s": 1e3 / ms, "evals_per_s": evals / (ms / 1e3),
            "launches_per_generation": 1, "autotune_tile_rows_ms": {str(k): v for k, v in tuned.items()},
            "tile_rows": best}


# DRAM bytes of one 50-generation island-resident launch of this workload (64 x 100, D = 30), from
# an ncu capture (dram__bytes_read.sum 932,352 + dram__bytes_write.sum 0): the algorithmic bytes of
# the same 50 streaming generations are 194.6 MB.
EPOCH_TRAFFIC_BYTES = 932352
C4_TRAIN_STEPS = 48   # Adam steps per generation: 48 x 4096 = 6 passes over a generation's 32768 new rows
C4_EXPLORE = 0.05     # fraction of targets that take a uniformly drawn trial instead of the screened one


def _c4_run(L, dev, torch, func: int, mode: str, max_gens: int, log_every: int = 10, stop_at: float | None = None,
            train_steps: int = 16, explore: float = 0.25, train_k: int = 8, use_graph: bool = True):
    """One config-4 run (plain or surrogate-screened) logging the FP64 best error every
    `log_every` generations; stops early once the error reaches `stop_at`. Blocks of `log_every`
    generations replay one CUDA graph after the first (eager) block."""
    import ctypes as C

    from speo_gb300 import _lib
    from speo_gb300 import workloads as w

    specs, inst = w.config4_specs(func)
    tab = w.table(specs, inst, device=dev)
    tab.init_population()
    surr = None
    if mode == "surrogate":
        surr = C.c_void_p()
        _lib.check(L.speo_surrogate_create(C.byref(surr), 50, 256, 1 << 20, 4096, 1e-3, 0.01, 4242),
                   "speo_surrogate_create")
    assert log_every % 2 == 0 and 50 % log_every == 0

    def block():  # log_every generations (an even number: the double buffers end where they began)
        if mode == "plain":
            if tab.epoch_fits():
                tab.epoch(log_every)
            else:
                for _ in range(log_every):
                    tab.generation()
        else:
            for _ in range(log_every):
                tab.surrogate_generation(surr, k=train_k, train_steps=train_steps, explore=explore)

    curve, t_total, graph = [], 0.0, None
    try:
        for g0 in range(0, max_gens, log_every):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            if graph is None:
                block()   # first block eagerly: scratch allocation, archive seeding
            else:
                graph.replay()
            if (g0 + log_every) % 50 == 0:
                tab.migrate(5)
            b.record()
            torch.cuda.synchronize()
            t_total += a.elapsed_time(b) / 1e3
            if graph is None and use_graph:  # later blocks replay one CUDA graph (not executed by capture)
                graph = torch.cuda.CUDAGraph()
                cs = torch.cuda.Stream()
                cs.wait_stream(torch.cuda.current_stream())
                with torch.cuda.stream(cs), torch.cuda.graph(graph, stream=cs):
                    block()
                torch.cuda.current_stream().wait_stream(cs)
            rows, errs = tab.best_f64()
            curve.append({"gen": g0 + log_every, "exact_evals": (g0 + log_every) * tab.rows, "wall_s": t_total,
                          "best_err": float(errs.min().item())})
            if stop_at is not None and curve[-1]["best_err"] <= stop_at:
                break
    finally:
        if surr is not None:
            L.speo_surrogate_destroy(surr)
    gens = curve[-1]["gen"]
    hit = next((c for c in curve if c["best_err"] <= 1e-8), None)
    kept = curve[:: max(1, len(curve) // 40)]
    if kept[-1] is not curve[-1]:
        kept.append(curve[-1])
    return {"curve": kept, "final_err": curve[-1]["best_err"], "generations": gens, "wall_s": t_total,
            "gens_per_s": gens / t_total, "exact_evals_per_s": gens * tab.rows / t_total,
            "exact_evals_to_1e-8": None if hit is None else hit["exact_evals"],
            "wall_s_to_1e-8": None if hit is None else hit["wall_s"]}, curve


def bench_config4(L, dev, torch, gens: int) -> dict:
    """Config 4: 128 islands x 256, D = 50. Plain DE against the surrogate-screened DE (MLP
    50-256-256-1, screening and training on the tensor cores in BF16 with FP32 accumulation,
    archive 2^20, Adam lr 1e-3, batch 4096, k = 8 trials per target, C4_TRAIN_STEPS Adam steps per
    generation, C4_EXPLORE exploration picks; blocks of 10 generations replay a CUDA graph); ring migration
    of 5 every 50 generations in both, both spend 32768 exact evaluations per generation. Best
    FP64 error every 10 generations; wall time from CUDA events around the generations only.
    (a) rotated Rastrigin for `gens` generations; (b) the rotated sphere of the same shape run to
    an error of 1e-8 (capped), which gives the exact evaluations each method needs to get there."""
    from speo_gb300 import _lib

    out = {"workload": "128 islands x P=256, D=50; surrogate MLP 50-256-256-1 (BF16 tcgen05 screening and "
                       "training), k=8", "train_steps_per_gen": C4_TRAIN_STEPS, "explore": C4_EXPLORE}
    ras = {"objective": "rotated Rastrigin", "generations": gens}
    curves = {}
    for mode in ("plain", "surrogate"):
        ras[mode], curves[mode] = _c4_run(L, dev, torch, _lib.FUNC_ROTATED_RASTRIGIN, mode, gens,
                                          train_steps=C4_TRAIN_STEPS, explore=C4_EXPLORE)
    target = ras["plain"]["final_err"]
    hit = next((c for c in curves["surrogate"] if c["best_err"] <= target), None)
    ras["surrogate_reaches_plain_final_error"] = None if hit is None else {
        "at_gen": hit["gen"], "exact_evals_ratio_plain_over_surrogate": curves["plain"][-1]["exact_evals"]
        / hit["exact_evals"], "wall_ratio_plain_over_surrogate": ras["plain"]["wall_s"] / hit["wall_s"]}
    out["rastrigin"] = ras
    sph = {"objective": "rotated sphere", "target_err": 1e-8}
    sph["plain"], _ = _c4_run(L, dev, torch, _lib.FUNC_ROTATED_SPHERE, "plain", 4000, stop_at=1e-8)
    sph["surrogate"], _ = _c4_run(L, dev, torch, _lib.FUNC_ROTATED_SPHERE, "surrogate", 1500, stop_at=1e-8,
                                  train_steps=C4_TRAIN_STEPS, explore=C4_EXPLORE)
    light, _ = _c4_run(L, dev, torch, _lib.FUNC_ROTATED_SPHERE, "surrogate", 1500, stop_at=1e-8, train_steps=16,
                       explore=C4_EXPLORE)
    sph["surrogate_16_steps"] = {k: v for k, v in light.items() if k != "curve"}
    ep, es = sph["plain"]["exact_evals_to_1e-8"], sph["surrogate"]["exact_evals_to_1e-8"]
    wp, ws = sph["plain"]["wall_s_to_1e-8"], sph["surrogate"]["wall_s_to_1e-8"]
    sph["exact_evals_ratio_plain_over_surrogate"] = ep / es if ep and es else None
    sph["wall_ratio_plain_over_surrogate"] = wp / ws if wp and ws else None
    out["sphere_to_1e-8"] = sph
    return out


def bench_mlp(L, dev, torch, steps: int = 16) -> dict:
    """The surrogate network's kernels at config 4's shapes (MLP 50-256-256-1): the tcgen05 screening
    forward over 262,144 trials (8 per target, 32,768 targets) and `steps` tcgen05 training steps on
    batches of 4096 drawn from an archive holding 32,768 rows; CUDA events, medians of 5."""
    import ctypes as C

    from speo_gb300 import _lib

    s = C.c_void_p()
    _lib.check(L.speo_surrogate_create(C.byref(s), 50, 256, 1 << 20, 4096, 1e-3, 0.01, 4242), "speo_surrogate_create")
    st = torch.cuda.current_stream().cuda_stream
    try:
        g = torch.Generator(device=dev).manual_seed(7)
        X = (torch.rand(32768, 52, device=dev, generator=g) * 200 - 100)
        X[:, 50:] = 0
        f = torch.rand(32768, device=dev, generator=g) * 1e4
        _lib.check(L.speo_surrogate_archive_append(s, X.data_ptr(), 32768, 52, f.data_ptr(), st), "append")
        T = (torch.rand(262144, 52, device=dev, generator=g) * 200 - 100)
        T[:, 50:] = 0
        y = torch.empty(262144, device=dev)

        def timed(fn, reps=5):
            fn()
            ts = []
            for _ in range(reps):
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record()
                fn()
                b.record()
                torch.cuda.synchronize()
                ts.append(a.elapsed_time(b) / 1e3)
            return float(np.median(ts))

        t_fwd = timed(lambda: _lib.check(L.speo_surrogate_forward_bf16(s, T.data_ptr(), 262144, 52, y.data_ptr(), st),
                                         "forward_bf16"))
        t_train = timed(lambda: _lib.check(L.speo_surrogate_train(s, steps, None, st), "train"))
        _lib.check(L.speo_surrogate_set_mode(s, 0), "set_mode")
        t_fwd32 = timed(lambda: _lib.check(L.speo_surrogate_forward(s, T.data_ptr(), 262144, 52, y.data_ptr(), st),
                                           "forward"))
        t_train32 = timed(lambda: _lib.check(L.speo_surrogate_train(s, steps, None, st), "train"))
    finally:
        L.speo_surrogate_destroy(s)
    flop_fwd = 262144 * 2 * (50 * 256 + 256 * 256 + 256)
    return {"workload": "MLP 50-256-256-1: screening forward of 262,144 trials; training steps of batch 4096",
            "forward_bf16_us": t_fwd * 1e6, "forward_bf16_tflops": flop_fwd / t_fwd / 1e12,
            "forward_fp32_simt_us": t_fwd32 * 1e6,
            "train_step_bf16_us": t_train / steps * 1e6, "train_step_fp32_simt_us": t_train32 / steps * 1e6,
            "train_steps_timed": steps}


def bench_e2e(L, dev, torch, args, f64: bool = False) -> dict:
    """Reference-shaped C ABI with host buffers: initial population + instance uploaded from
    pinned host memory, then per generation generate / evaluate / select and a read-back of
    the generation's fitness vector; all inside the timed region. f64: the same in the
    reference's shipped precision (`real` = double) through speo_de_run_f64 and the FP64 entry
    points."""
    from speo_gb300 import _lib
    from speo_gb300.instances import make_instance

    n = N_ISLANDS * POP
    ld = 32
    npt = np.float64 if f64 else np.float32
    tdt = torch.float64 if f64 else torch.float32
    es = 8 if f64 else 4
    sfx = "" if f64 else "_f32"
    Pop = _lib.PopulationF64 if f64 else _lib.PopulationF32
    PI = _lib.ProblemInfoF64 if f64 else _lib.ProblemInfoF32
    DI = _lib.DEInfoF64 if f64 else _lib.DEInfoF32
    init, gen, ev, sel = (getattr(L, f + sfx) for f in ("API_Initilize", "API_DE_GenerateNewPopulation",
                                                        "API_evaluateFitness", "API_DE_SelectSurvival"))
    de_run = L.speo_de_run_f64 if f64 else L.speo_de_run_f32
    run_name = "speo_de_run_f64" if f64 else "speo_de_run_f32"
    o, M = make_instance(run_seed(), DIM)
    rot = np.zeros((ld, DIM), dtype=npt)
    rot[:DIM] = M.T
    sh = np.zeros(ld, dtype=npt)
    sh[:DIM] = o
    rng = np.random.default_rng(0)
    h_pop = torch.from_numpy(rng.uniform(-100, 100, (n, ld)).astype(npt)).pin_memory()
    h_pop[:, DIM:] = 0
    h_rot = torch.from_numpy(rot).pin_memory()
    h_sh = torch.from_numpy(sh).pin_memory()
    h_fit = torch.zeros(n, dtype=tdt).pin_memory()
    pop, cand = torch.empty(n, ld, dtype=tdt, device=dev), torch.zeros(n, ld, dtype=tdt, device=dev)
    pfit, cfit = torch.empty(n, dtype=tdt, device=dev), torch.empty(n, dtype=tdt, device=dev)
    d_rot, d_sh = torch.empty(ld, DIM, dtype=tdt, device=dev), torch.empty(ld, dtype=tdt, device=dev)
    rng_state = torch.zeros(16, dtype=torch.int32, device=dev)
    perm = torch.arange(n, dtype=torch.int32, device=dev)
    best = torch.zeros(N_ISLANDS, dtype=torch.int32, device=dev)
    info = (DI * N_ISLANDS)(*[DI(0.9, 0.5, 4, POP) for _ in range(N_ISLANDS)])
    h_info = torch.frombuffer(bytearray(bytes(info)), dtype=torch.uint8).pin_memory()
    d_info = torch.empty_like(h_info, device=dev)
    ii = _lib.IslandInfo(n, N_ISLANDS, perm.data_ptr())
    pi = PI(DIM, FUNC, 1, 0, run_seed(), 0, 0, 100.0, -100.0)
    P = Pop(pop.data_ptr(), pfit.data_ptr())
    C = Pop(cand.data_ptr(), cfit.data_ptr())
    stream = torch.cuda.current_stream()
    L.speo_set_stream(ctypes.c_void_p(stream.cuda_stream))
    _lib.check(init(C, rng_state.data_ptr(), ii, pi), "API_Initilize" + sfx)
    steps = max(100, min(args.steps, 2000))
    h_hist = torch.zeros(steps * n, dtype=tdt).pin_memory()  # every generation's fitness

    def upload():
        pop.copy_(h_pop, non_blocking=True)
        d_rot.copy_(h_rot, non_blocking=True)
        d_sh.copy_(h_sh, non_blocking=True)
        d_info.copy_(h_info, non_blocking=True)
        ev(pfit.data_ptr(), None, None, pop.data_ptr(), d_sh.data_ptr(), d_rot.data_ptr(), None, None, None, None, n,
           DIM, 0.0, FUNC)

    def run_native(nsteps):  # the reference's DE_CUDA::Run loop as one library call (C++ host loop)
        upload()
        _lib.check(de_run(P, C, rng_state.data_ptr(), ii, d_info.data_ptr(), best.data_ptr(), pi, d_sh.data_ptr(),
                          d_rot.data_ptr(), None, nsteps, h_hist.data_ptr(), 1, stream.cuda_stream), run_name)
        stream.synchronize()

    def run_python(nsteps):  # the same calls issued one by one from Python (ctypes)
        upload()
        for _ in range(nsteps):
            gen(C, P, best.data_ptr(), ii, d_info.data_ptr(), rng_state.data_ptr(), pi)
            ev(cfit.data_ptr(), None, None, cand.data_ptr(), d_sh.data_ptr(), d_rot.data_ptr(), None, None, None, None,
               n, DIM, 0.0, FUNC)
            sel(P, C, ii, pi)
            h_fit.copy_(pfit, non_blocking=True)
        stream.synchronize()

    out = {}
    for name, fn in (("native", run_native), ("python", run_python)):
        fn(20)
        t0 = time.perf_counter()
        fn(steps)
        out[name] = n * steps / (time.perf_counter() - t0)
    _lib.check(L.API_CheckCUDAError(), "e2e")
    L.speo_set_stream(None)
    h2d = (n * ld + ld * DIM + ld) * es + len(bytes(info))
    return {"value": out["native"], "unit": "evals/s", "h2d_bytes_per_step": h2d / steps,
            "d2h_bytes_per_step": n * es, "steps": steps, "dtype": "fp64" if f64 else "fp32",
            "path": f"{run_name} (64 sub-islands of 100): the generations of API_DE_GenerateNewPopulation{sfx} + "
                    f"API_evaluateFitness{sfx} + API_DE_SelectSurvival{sfx}, bit-identical, with the sub-islands "
                    "resident in shared memory for up to 100 generations per launch; every generation's fitness vector "
                    "read back to pinned host memory (one copy per launch)",
            "python_loop_value": out["python"],
            "python_loop_path": "the same entry points called one by one from Python (ctypes), per-call host cost"}


# The reference's published runs (CEC2014 composition functions, D = 100, 4096 individuals per
# GPU, FP64, DE/rand/1/bin CR = 0.9 F = 0.5): per-GPU Mevals/s of its 2-GPU runs, whole loop with
# its host-staged migration (R/bin/Results/SPEO_GPU.csv).
PUBLISHED_2GPU_MEVALS = {23: 2.94, 24: 3.84, 25: 3.61, 26: 2.25, 27: 2.30, 28: 2.71, 29: 2.87, 30: 2.43}


def bench_published(L, dev, torch, gens: int = 300, gens64: int = 60, fids=range(23, 31), fp64: bool = True) -> dict:
    """F23-F30 at D = 100, one island of 4096 rows (one sub-island), through the drop-in entry
    points on device-resident data: the FP32 loop and the FP64 loop (the reference's precision),
    each as one speo_de_run_f32 / _f64 call (the generations of API_DE_GenerateNewPopulation +
    API_evaluateFitness + API_DE_SelectSurvival; last fitness read back); plus the evaluation
    kernel alone (CUDA events). No migration (one island per GPU; the reference's numbers include its MPI
    migration, 19-38% of its wall time at 2 GPUs)."""
    from speo_gb300 import _lib
    from speo_gb300.instances import make_instance_multi

    n, D, ld = 4096, 100, 128
    out = {"workload": "CEC2014 F23-F30, D=100, island of 4096, DE/rand/1/bin CR=0.9 F=0.5, synthetic instances",
           "functions": {}}
    stream = torch.cuda.current_stream()
    L.speo_set_stream(ctypes.c_void_p(stream.cuda_stream))
    for fid in fids:
        o, M, S = make_instance_multi(run_seed() + fid, D, fid)
        nc = o.shape[0]
        rot = np.zeros((nc, ld, D), dtype=np.float32)
        rot[:, :D] = M.transpose(0, 2, 1)
        sh = np.zeros((nc, ld), dtype=np.float32)
        sh[:, :D] = o
        sf = np.zeros((nc, ld), dtype=np.int32)
        sf[:, :D] = S
        rec = {}
        for f64 in (False, True) if fp64 else (False,):
            dt = torch.float64 if f64 else torch.float32
            sfx = "" if f64 else "_f32"
            Pop = _lib.PopulationF64 if f64 else _lib.PopulationF32
            PI = _lib.ProblemInfoF64 if f64 else _lib.ProblemInfoF32
            DI = _lib.DEInfoF64 if f64 else _lib.DEInfoF32
            pop, cand = torch.zeros(n, ld, dtype=dt, device=dev), torch.zeros(n, ld, dtype=dt, device=dev)
            pfit, cfit = torch.zeros(n, dtype=dt, device=dev), torch.zeros(n, dtype=dt, device=dev)
            d_rot, d_sh = torch.from_numpy(rot).to(dev, dt), torch.from_numpy(sh).to(dev, dt)
            d_sf = torch.from_numpy(sf).to(dev)
            rng_state = torch.zeros(16, dtype=torch.int32, device=dev)
            perm = torch.arange(n, dtype=torch.int32, device=dev)
            best = torch.zeros(1, dtype=torch.int32, device=dev)
            info = (DI * 1)(DI(0.9, 0.5, 4, n))
            d_info = torch.frombuffer(bytearray(bytes(info)), dtype=torch.uint8).to(dev)
            ii = _lib.IslandInfo(n, 1, perm.data_ptr())
            pi = PI(D, fid, 1, 0, run_seed(), 0, 0, 100.0, -100.0)
            P, C = Pop(pop.data_ptr(), pfit.data_ptr()), Pop(cand.data_ptr(), cfit.data_ptr())
            _lib.check(getattr(L, "API_Initilize" + sfx)(P, rng_state.data_ptr(), ii, pi), "API_Initilize")
            ev = getattr(L, "API_evaluateFitness" + sfx)
            eargs = (d_sh.data_ptr(), d_rot.data_ptr(), d_sf.data_ptr(), None, None, None, n, D, 0.0, fid)
            ev(pfit.data_ptr(), None, None, pop.data_ptr(), *eargs)
            # the evaluation kernel alone
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            for _ in range(3):
                ev(cfit.data_ptr(), None, None, pop.data_ptr(), *eargs)
            reps = 20
            e0.record(stream)
            for _ in range(reps):
                ev(cfit.data_ptr(), None, None, pop.data_ptr(), *eargs)
            e1.record(stream)
            torch.cuda.synchronize()
            eval_us = e0.elapsed_time(e1) * 1e3 / reps
            h = torch.zeros(n, dtype=dt).pin_memory()
            de_run = L.speo_de_run_f64 if f64 else L.speo_de_run_f32

            def run(k):
                _lib.check(de_run(P, C, rng_state.data_ptr(), ii, d_info.data_ptr(), best.data_ptr(), pi,
                                  d_sh.data_ptr(), d_rot.data_ptr(), d_sf.data_ptr(), k, h.data_ptr(), 0,
                                  stream.cuda_stream), "speo_de_run")
                stream.synchronize()
            k = gens64 if f64 else gens
            run(10)
            t0 = time.perf_counter()
            run(k)
            dt_s = time.perf_counter() - t0
            _lib.check(L.API_CheckCUDAError(), "published")
            v = n * k / dt_s
            rec["fp64" if f64 else "fp32"] = {
                "evals_per_s": v, "us_per_gen": dt_s / k * 1e6, "eval_kernel_us": eval_us,
                "vs_published_per_gpu": v / (PUBLISHED_2GPU_MEVALS[fid] * 1e6),
                "best_error": float(pfit.min())}
        out["functions"][str(fid)] = rec
    L.speo_set_stream(None)
    out["published_per_gpu_mevals"] = PUBLISHED_2GPU_MEVALS
    return out


def cpu_workload_sample(sample_s: float, threads: int):
    """FP64 island loop of the oracle port on the host cores: (evals/s, gens done)."""
    import speo_oracle
    from speo_gb300.instances import make_instance

    o, M = make_instance(run_seed(), DIM)
    ld = 32
    n = N_ISLANDS * POP
    pop = speo_oracle.init_population(n, ld, DIM, -100.0, 100.0, run_seed()).astype(np.float64)
    fit = speo_oracle.evaluate_rows(FUNC, pop.astype(np.float32), DIM, o, M)
    gens, total_evals, t_used = 0, 0, 0.0
    chunk = 2
    while t_used < sample_s:
        t0 = time.perf_counter()
        total_evals += speo_oracle.run_islands_f64(N_ISLANDS, POP, DIM, ld, FUNC, 0.5, 0.9, -100.0, 100.0, o, M,
                                                   run_seed(), gens, chunk, INTERVAL, MIGRANTS, pop, fit, threads)
        t_used += time.perf_counter() - t0
        gens += chunk
        chunk = min(chunk * 2, 200)
    return total_evals / t_used, gens, t_used


def cpu_baseline(sample_s: float = 12.0) -> dict:
    threads = os.cpu_count() or 1
    rate, gens, t = cpu_workload_sample(sample_s, threads)
    return {"value": rate, "unit": "evals/s", "cores": threads, "kind": "port",
            "sample": f"{gens} generations of the same 64x100 D=30 island workload in FP64 "
                      f"(oracle restatement of the reference's DE + CEC2014 objective), {t:.1f} s, "
                      f"{threads} threads over islands"}


def bench_reference(args) -> dict:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return None
    threads = os.cpu_count() or 1
    rate, gens, t = cpu_workload_sample(min(60.0, max(10.0, 0.002 * args.steps)), threads)
    return {"metric": METRIC, "value": rate, "unit": "evals/s", "n_gpus": 0, "steps": gens, "warmup": 0,
            "ms_per_step": t * 1e3 / gens, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "fp64", "data": "synthetic", "impl": "reference",
            "config": {"workload": "island model: 64 islands x P=100, D=30, rotated Rastrigin (F9 form), "
                                   "DE/rand/1/bin F=0.5 CR=0.9, ring best-5 -> worst-5 every 50 generations"},
            "cpu_baseline": {"value": rate, "unit": "evals/s", "cores": threads, "kind": "port",
                             "sample": f"{gens} generations, {t:.1f} s (the reference's compiled CPU objective "
                                       "cannot run on the Arm box; the oracle port restates it)"},
            "e2e": {"value": rate, "unit": "evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20000)
    ap.add_argument("--warmup", type=int, default=500)
    ap.add_argument("--impl", default="speo", choices=["speo", "reference"])
    ap.add_argument("--cpu-sample-s", type=float, default=12.0)
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer C-ABI leg (profiling runs)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-baseline leg (profiling runs)")
    ap.add_argument("--no-ops", action="store_true", help="skip the bandwidth-scale operator measurements")
    ap.add_argument("--ops-only", action="store_true", help="only the bandwidth-scale operator measurements")
    ap.add_argument("--ops-islands", type=int, default=16384, help="islands of 128 rows in the operator variant")
    ap.add_argument("--no-configs", action="store_true", help="skip the config 2 / 3 / 4 sections")
    ap.add_argument("--c4-gens", type=int, default=200, help="generations of each config-4 run")
    ap.add_argument("--configs-only", action="store_true", help="only the config 2 / 3 / 4 sections")
    ap.add_argument("--c4-only", action="store_true", help="only the config 4 section")
    ap.add_argument("--mlp-case", action="store_true", help="only the surrogate network's kernels at config-4 shapes")
    ap.add_argument("--e2e-only", action="store_true", help="only the end-to-end drop-in measurement")
    ap.add_argument("--published-only", action="store_true",
                    help="only the reference's published configuration (F23-F30, D=100, 4096 rows)")
    ap.add_argument("--published-fids", default="23-30", help="function ids a-b of the published configuration")
    ap.add_argument("--published-fp32-only", action="store_true", help="skip the FP64 leg of the published configuration")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.e2e_only:
        import torch
        from speo_gb300 import _lib

        torch.cuda.set_device(0)
        L = _lib.load()
        print(json.dumps({"e2e": bench_e2e(L, "cuda:0", torch, args),
                          "e2e_fp64": bench_e2e(L, "cuda:0", torch, args, f64=True)}))
        return
    if args.published_only:
        import torch
        from speo_gb300 import _lib

        torch.cuda.set_device(0)
        a, b = (int(v) for v in args.published_fids.split("-"))
        print(json.dumps({"published_config": bench_published(_lib.load(), "cuda:0", torch, fids=range(a, b + 1),
                                                               fp64=not args.published_fp32_only)}))
        return
    if args.mlp_case:
        import torch
        from speo_gb300 import _lib

        torch.cuda.set_device(0)
        print(json.dumps({"surrogate_mlp": bench_mlp(_lib.load(), "cuda:0", torch)}))
        return
    if args.c4_only:
        import torch
        from speo_gb300 import _lib

        torch.cuda.set_device(0)
        print(json.dumps({"config4_surrogate_vs_plain": bench_config4(_lib.load(), "cuda:0", torch, args.c4_gens)}))
        return
    if args.configs_only:
        import torch
        from speo_gb300 import _lib

        torch.cuda.set_device(0)
        L = _lib.load()
        flush = torch.empty(128 * 1024 * 1024, dtype=torch.float32, device="cuda:0")
        print(json.dumps({"config2_precision": bench_config2(L, "cuda:0", torch, flush),
                          "config3_batched": bench_config3(L, "cuda:0", torch, flush),
                          "config4_surrogate_vs_plain": bench_config4(L, "cuda:0", torch, args.c4_gens)}))
        return
    if args.ops_only:
        import torch
        from speo_gb300 import _lib

        torch.cuda.set_device(0)
        print(json.dumps(bench_operators(_lib.load(), "cuda:0", torch, peaks(), args.ops_islands)))
        return
    out = bench_reference(args) if args.impl == "reference" else bench_speo(args)
    if out is not None and int(os.environ.get("RANK", "0")) == 0:
        print(json.dumps(out))


if __name__ == "__main__":
    main()
