"""Benchmark of the island-model DE generation loop on GB300.

Headline workload (the learned-surrogate configuration): 128 islands x P = 256, D = 50, rotated
Rastrigin z = M (0.0512 (x - o)) (CEC2014 F9 form, f - f*), F = 0.5, CR = 0.9, DE/rand/1/bin,
ring migration of each island's best 5 into the next island's worst 5 every 50 generations;
seeded synthetic o ~ U[-80, 80]^50 and Haar M.

A step is one generation over all islands (32,768 exact evaluations). After --warmup untimed
generations, exactly --steps generations are timed. Generations run island-resident (one
launch per stretch between migrations); the L2 is flushed (512 MB write) before each launch.
`value` is the plain DE loop's exact evaluations/s over the whole job with the population
resident in HBM. `e2e` is the same loop through the reference-shaped C ABI (speo_de_run_f32 =
the generations of API_DE_GenerateNewPopulation_f32 / API_evaluateFitness_f32 /
API_DE_SelectSurvival_f32, plus the ring migration) with host buffers: the initial population
and instance uploaded and every generation's fitness vector read back inside the timed region.
`surrogate` sets the surrogate-screened DE beside the plain DE on the same GPU (exact
evaluations and wall time to an FP64 error of 1e-8 on the rotated sphere of the same shape, and
to the plain run's final error on the rotated Rastrigin).

The last stdout line is the JSON record (a few KB). --full also measures the secondary
sections (64 x 100 island ring at D = 30, operators at bandwidth scale, precision, batched runs,
network kernels, the reference's published configuration) into --sections-out.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl speo|reference] [--full]
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

METRIC = "exact-eval gens/s & evals to 1e-8 error: surrogate vs plain DE, same GB300"
N_ISLANDS, POP, DIM, FUNC = 128, 256, 50, 9
INTERVAL, MIGRANTS = 50, 5
E2E_REPEATS = 5  # the end-to-end loops are timed this many times each (wall clock); the median is reported
EVALS_PER_STEP = N_ISLANDS * POP
WORKLOAD = ("learned-surrogate configuration, plain DE leg: 128 islands x P=256, D=50, rotated Rastrigin "
            "(F9 form, scale 0.0512), DE/rand/1/bin F=0.5 CR=0.9, ring best-5 -> worst-5 every 50 generations")
# FP32 FMA lanes of one SM (four partitions of 32): the CUDA-core roofline of the resident kernels
FP32_FMA_PER_SM_CLK = 128


def peaks() -> dict:
    p = REPO / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": d["hbm_gbs"], "bf16_tflops": d.get("bf16_tflops"), "src": "measured"}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "src": "fallback"}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            time.sleep(0.3)   # the first sample lands before the timed work starts
        except FileNotFoundError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            out, _ = self.proc.communicate(timeout=10)
            self.lines = [ln for ln in out.splitlines() if ln.strip()]

    def summary(self) -> dict:
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
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


def chunks(done: int, n: int, interval: int = INTERVAL):
    """Split n generations, starting after `done` generations, at the migration points: yields
    (generations, migrate_after) with a migration after every generation count that is a multiple
    of `interval` (src/island_EA.cc:94-99 migrates when gen % interval == 0)."""
    while n > 0:
        k = min(n, interval - done % interval)
        done += k
        n -= k
        yield k, done % interval == 0


def headline_table(dev: str, rank: int = 0, func: int = FUNC, extra_rows: int = 0):
    from speo_gb300 import workloads as w

    specs, inst = w.config4_specs(func, rank=rank)
    return w.table(specs, inst, device=dev, extra_rows=extra_rows)


def ring_migration(tab, dev: str, rank: int, world: int):
    """The ring step of the headline: on one GPU the library's ring over the 128 islands; across
    ranks, one global ring over all ranks' islands (contiguous blocks of 128 per rank, boundary
    migrants through point-to-point messages into local ghost rows, speo_gb300.ring)."""
    if world == 1:
        return lambda: tab.migrate(MIGRANTS)
    from speo_gb300.ring import DeviceRingOps, RingBlock

    blk, ops = RingBlock(N_ISLANDS, POP, DIM, tab.ld, MIGRANTS, rank, world), DeviceRingOps(dev)
    return lambda: blk.migrate(ops, tab.pop[tab.cur], tab.fit[tab.cur])


def run_plain(epoch, migrate, n: int, done: int) -> int:
    """n plain generations (island-resident launches, ring migration at the migration points)."""
    for k, mig in chunks(done, n):
        epoch(k)
        if mig:
            migrate()
    return done + n


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
    tab = headline_table(dev, rank, extra_rows=2 * MIGRANTS if world > 1 else 0)
    use_tc = args.epoch == "tc" or (args.epoch == "auto" and tab.epoch_tc_fits())
    if not (tab.epoch_tc_fits() if use_tc else tab.epoch_fits()):
        raise RuntimeError("the headline islands do not fit one block's shared memory on this GPU")
    epoch = tab.epoch_tc if use_tc else tab.epoch
    migrate = ring_migration(tab, dev, rank, world)
    # one GPU, tensor-core epochs: the migrations run inside one cooperative launch of all the
    # generations (speo_island_epochs_tc); otherwise a launch per interval and migration launches
    fused = world == 1 and use_tc and not args.launch_per_interval
    tab.init_population()
    flush = torch.empty(128 * 1024 * 1024, dtype=torch.float32, device=dev)
    plan = [(args.steps, False)] if fused else list(chunks(args.warmup, args.steps))
    ev = [tuple(torch.cuda.Event(enable_timing=True) for _ in range(3)) for _ in plan]
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    # the clock sampler (an nvidia-smi process) starts before the warm-up, so that its start-up is
    # over when the timed region begins; it samples until after the timed region
    with ClockSampler(local) as clk:
        # bring a fresh GPU to its working clocks first: about 50 ms of untimed memory writes
        for _ in range(300):
            flush_l2(flush)
        torch.cuda.synchronize()
        if fused:
            tab.island_epochs_tc(args.warmup, 0, INTERVAL, MIGRANTS)   # exactly W untimed generations
            done = args.warmup
        else:
            done = run_plain(epoch, migrate, args.warmup, 0)       # exactly W untimed generations
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        for (k, mig), (a, b, c) in zip(plan, ev):
            # L2 flushed before every launch; the second pass keeps the GPU busy while the host
            # issues the launch, so the timed region (from the GPU's event) holds no idle gap
            flush_l2(flush)
            flush_l2(flush)
            a.record()
            if fused:
                tab.island_epochs_tc(k, done, INTERVAL, MIGRANTS)
            else:
                epoch(k)
            b.record()
            if mig:
                migrate()
            c.record()
        torch.cuda.synchronize()
        # the dominant kernel alone, 50-generation launches back to back (clocks still sampled)
        kg = capture(torch, lambda: epoch(INTERVAL))
        launch50_ms = time_graph(torch, kg, 20, flush)
    if world > 1:
        torch.distributed.barrier()
    step_ms = sum(a.elapsed_time(c) for a, _, c in ev)
    kern_ms = sum(a.elapsed_time(b) for a, b, _ in ev)
    ms = max_over_ranks(step_ms, dev, world)
    value = EVALS_PER_STEP * args.steps * world / (ms / 1e3)
    n_mig = (done + args.steps) // INTERVAL - done // INTERVAL if fused else sum(1 for _, m in plan if m)
    rows, errs = tab.best_f64()
    best_err = float(errs.min().item())

    pk = peaks()
    clocks = clk.summary()
    alg_bytes_gen = EVALS_PER_STEP * (5 * DIM * 4 + 2 * 4)  # 4 row reads + 1 row write + 2 fitness per eval
    achieved = alg_bytes_gen * args.steps / (kern_ms / 1e3) / 1e9
    gens_per_launch = args.steps / len(plan)
    if use_tc:
        kernel = (f"k_island_epoch_tc<2> (one 512-thread block per island, {N_ISLANDS} blocks, the island and its "
                  "trials in shared memory, the rotation on tcgen05: three split-FP16 products per K step into TMEM "
                  "accumulators; " + ("all the timed generations in one cooperative launch, each ring migration "
                                      "inside it at a grid barrier)" if fused else "up to 50 generations per launch)"))
    elif 2 * N_ISLANDS <= sms:
        kernel = f"k_island_epoch2<2> (two-block cluster per island, {2 * N_ISLANDS} blocks)"
    else:
        kernel = (f"k_island_epoch<2> (one 512-thread block per island, {N_ISLANDS} blocks; up to 50 generations "
                  "per launch with the island, its trials and M^T in shared memory)")
    traffic = EPOCH_LAUNCH_TRAFFIC_BYTES["tc" if use_tc else "simt"]
    rot_flop_gen = EVALS_PER_STEP * 2 * DIM * DIM
    kp = (DIM + 15) // 16 * 16
    # executed split products: three FP16 products per K step, M = 128 rows per tile, N = K = kp
    tensor_flop_gen = N_ISLANDS * ((POP + 127) // 128) * 3 * 2 * 128 * kp * kp
    sm_mhz = clocks["sm_max_mhz"] or 2070.0
    fp32_peak = sms * FP32_FMA_PER_SM_CLK * 2 * sm_mhz * 1e6 / 1e12
    fp32_achieved = rot_flop_gen * args.steps / (kern_ms / 1e3) / 1e12
    out = {
        "metric": METRIC, "value": value, "unit": "evals/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp32", "data": "synthetic (seeded o ~ U[-80,80]^50, Haar M, uniform init)",
        "config": {"workload": WORKLOAD, "islands": N_ISLANDS, "pop_size": POP, "dim": DIM, "func_id": FUNC,
                   "migration_interval": INTERVAL, "migrants": MIGRANTS,
                   "step": f"one generation over all islands ({EVALS_PER_STEP} exact evaluations)",
                   "l2": "flushed (512 MB write) before every timed launch; each island stays resident in shared "
                         "memory for the whole launch",
                   "launches": (f"1 cooperative island-resident launch of {args.steps} generations with the {n_mig} "
                                "ring migrations inside it" if fused else
                                f"{len(plan)} island-resident launches + {2 * n_mig} migration launches")},
        "gens_per_s": args.steps / (ms / 1e3),
        "best_error_f64": best_err,
        "roofline": {"kernel": kernel, "bound": "hbm", "achieved": achieved, "peak": pk["hbm_gbs"], "unit": "GB/s",
                     "frac": achieved / pk["hbm_gbs"], "traffic": traffic,
                     "traffic_src": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch of this kernel on "
                                    "this workload (the island is read once per launch; its writes stay in L2)",
                     "peak_src": f"{pk['src']} (MEASURED_PEAKS hbm_gbs)",
                     "alg_bytes_per_launch": alg_bytes_gen * gens_per_launch, "generations_per_launch": gens_per_launch,
                     "kernel_ms_timed": kern_ms, "launch_us_50_generations": launch50_ms * 1e3,
                     "note": "achieved = streaming-equivalent bytes (5 D s + 2 s per individual-generation) / kernel "
                             "time; the island stays in shared memory, so DRAM traffic is far below them",
                     "fp32": {"achieved_tflops": fp32_achieved, "peak_tflops": fp32_peak, "frac": fp32_achieved / fp32_peak,
                              "flop_per_eval": 2 * DIM * DIM,
                              "peak_src": f"nominal: {sms} SMs x {FP32_FMA_PER_SM_CLK} FP32 FMA/clk x 2 x {sm_mhz:.0f} MHz"},
                     **({"tensor": {"achieved_tflops": tensor_flop_gen * args.steps / (kern_ms / 1e3) / 1e12,
                                    "peak_tflops": pk["bf16_tflops"],
                                    "frac": tensor_flop_gen * args.steps / (kern_ms / 1e3) / 1e12 / pk["bf16_tflops"],
                                    "flop_per_step": tensor_flop_gen,
                                    "peak_src": f"{pk['src']} (MEASURED_PEAKS bf16_tflops, burst)"}} if use_tc else {})},
        "gpu_launches": len(plan) if fused else len(plan) + 2 * n_mig,
        "clocks": clocks,
    }
    if rank != 0:
        return out
    if not args.no_surrogate:
        out["surrogate"] = bench_surrogate(L, dev, torch)
    if not args.no_e2e:
        out["e2e"] = bench_e2e(L, dev, torch, max(args.steps, 100))
        d = bench_e2e_dropin(L, dev, torch, max(args.steps, 100))
        out["e2e_dropin"] = {"value": d["value"], "unit": d["unit"], "path": d["path"]}
    if not args.no_cpu:
        out["cpu_baseline"] = cpu_baseline(sample_s=args.cpu_sample_s)
    return out


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one island-resident launch of the
# headline workload, from an ncu capture of that launch (45 generations; the island is read once per
# launch and its writes stay in L2, so the figure does not grow with the generations per launch).
EPOCH_LAUNCH_TRAFFIC_BYTES = {"simt": 7040512 + 11008, "tc": 7065344 + 191232}
C4_TRAIN_STEPS = 48   # Adam steps per generation: 48 x 4096 = 6 passes over a generation's 32768 new rows
C4_EXPLORE = 0.05     # fraction of targets that take a uniformly drawn trial instead of the screened one
# Training batch x Adam steps per generation at about the same samples per generation (k = 8,
# training every generation): larger batches fill more SMs per step.
# Trials screened per target and Adam steps per generation at the default batch (4096) and rate.
SURROGATE_K_GRID = [dict(k=k, train_steps=st, train_every=1) for k in (8, 12, 16) for st in (48, 64)]
SURROGATE_BATCH_GRID = [dict(k=8, train_steps=st, train_every=1, train_batch=b, lr=lr)
                        for b, st, lr in ((4096, 48, 1e-3), (8192, 24, 1e-3), (8192, 24, 2e-3), (16384, 12, 2e-3),
                                          (16384, 12, 4e-3), (16384, 24, 2e-3), (32768, 6, 4e-3), (32768, 6, 8e-3),
                                          (32768, 12, 4e-3))]


def c4_run(L, dev, torch, func: int, mode: str, max_gens: int, log_every: int = 10, stop_at: float | None = None,
           train_steps: int = 16, explore: float = 0.25, train_k: int = 8, train_every: int = 1,
           use_graph: bool = True, train_batch: int = 4096, lr: float = 1e-3, uneven: bool = False):
    """One run of the headline shape (plain or surrogate-screened) logging the FP64 best error
    every `log_every` generations; stops early once the error reaches `stop_at`. Blocks of
    `log_every` generations replay one CUDA graph after the first (eager) block. The surrogate
    trains `train_steps` Adam steps in every `train_every`-th generation of a block."""
    import ctypes as C

    from speo_gb300 import _lib
    from speo_gb300 import workloads as w

    specs, inst = (w.config4_uneven_specs if uneven else w.config4_specs)(func)
    tab = w.table(specs, inst, device=dev)
    tab.init_population()
    surr = None
    if mode == "surrogate":
        surr = C.c_void_p()
        _lib.check(L.speo_surrogate_create(C.byref(surr), 50, 256, 1 << 20, train_batch, lr, 0.01, 4242),
                   "speo_surrogate_create")
    assert log_every % 2 == 0 and INTERVAL % log_every == 0 and log_every % train_every == 0

    def block():  # log_every generations (an even number: the double buffers end where they began)
        if mode == "plain":
            tab.epoch(log_every)
        else:
            for i in range(log_every):
                steps = train_steps if (i + 1) % train_every == 0 else 0
                tab.surrogate_generation(surr, k=train_k, train_steps=steps, explore=explore)

    curve, t_total, graph = [], 0.0, None
    try:
        for g0 in range(0, max_gens, log_every):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            if graph is None:
                block()   # first block eagerly: scratch allocation, archive seeding
            else:
                graph.replay()
            if (g0 + log_every) % INTERVAL == 0:
                tab.migrate(MIGRANTS)
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
    hit = next((c for c in curve if stop_at is not None and c["best_err"] <= stop_at), None)
    return {"final_err": curve[-1]["best_err"], "generations": gens, "wall_s": t_total,
            "gens_per_s": gens / t_total, "exact_evals_per_s": gens * tab.rows / t_total,
            "exact_evals_to_target": None if hit is None else hit["exact_evals"],
            "wall_s_to_target": None if hit is None else hit["wall_s"]}, curve


def first_reach(curve, target):
    return next((c for c in curve if c["best_err"] <= target), None)


def bench_surrogate(L, dev, torch, ras_gens: int = 200, schedule: dict | None = None, uneven: bool = False) -> dict:
    """Surrogate-screened DE against the plain DE on the headline shape, same GPU: (a) the
    rotated sphere of the same shape run to an FP64 error of 1e-8 (capped), which gives the
    exact evaluations and wall time each method needs to get there; (b) the rotated Rastrigin
    for `ras_gens` generations, and where the surrogate first reaches the plain run's final
    error. Both methods spend 32,768 exact evaluations per generation."""
    from speo_gb300 import _lib

    sch = dict(train_steps=C4_TRAIN_STEPS, explore=C4_EXPLORE, train_k=8, train_every=1)
    if schedule:
        sch.update(schedule)
    out = {"network": "MLP 50-256-256-1, BF16 tcgen05 screening and training, FP32 accumulate, Adam lr 1e-3, "
                      "batch 4096, archive 2^20, k=8 trials per target", "schedule": sch}
    sp, _ = c4_run(L, dev, torch, _lib.FUNC_ROTATED_SPHERE, "plain", 4000, stop_at=1e-8, uneven=uneven)
    ss, _ = c4_run(L, dev, torch, _lib.FUNC_ROTATED_SPHERE, "surrogate", 1500, stop_at=1e-8, uneven=uneven, **sch)
    sph = {"target": 1e-8,
           "plain": {k: sp[k] for k in ("generations", "exact_evals_to_target", "wall_s_to_target", "final_err")},
           "surrogate": {k: ss[k] for k in ("generations", "exact_evals_to_target", "wall_s_to_target", "final_err")}}
    ep, es = sp["exact_evals_to_target"], ss["exact_evals_to_target"]
    wp, ws = sp["wall_s_to_target"], ss["wall_s_to_target"]
    sph["exact_evals_ratio_plain_over_surrogate"] = ep / es if ep and es else None
    sph["wall_ratio_plain_over_surrogate"] = wp / ws if wp and ws else None
    out["rotated_sphere"] = sph
    rp, cp = c4_run(L, dev, torch, _lib.FUNC_ROTATED_RASTRIGIN, "plain", ras_gens, uneven=uneven)
    rs, cs = c4_run(L, dev, torch, _lib.FUNC_ROTATED_RASTRIGIN, "surrogate", ras_gens, uneven=uneven, **sch)
    hit = first_reach(cs, rp["final_err"])
    hit_p = first_reach(cp, rp["final_err"])
    out["rotated_rastrigin"] = {
        "generations": ras_gens, "plain_final_err": rp["final_err"], "surrogate_final_err": rs["final_err"],
        "plain_gens_per_s": rp["gens_per_s"], "surrogate_gens_per_s": rs["gens_per_s"],
        "surrogate_reaches_plain_final_error": None if hit is None else {
            "at_gen": hit["gen"], "exact_evals_ratio_plain_over_surrogate": hit_p["exact_evals"] / hit["exact_evals"],
            "wall_ratio_plain_over_surrogate": hit_p["wall_s"] / hit["wall_s"]},
        "note": "1e-8 is not reached by either method on the rotated Rastrigin at D=50 (multimodal); the "
                "comparison is at the smallest error both reach"}
    return out


def bench_surrogate_sweep(L, dev, torch, ks=(2, 4, 8), steps=(1, 4, 16, 48), every=(1, 5, 10),
                          ras_gens: int = 200, grid: list | None = None) -> dict:
    """The surrogate's schedule against the plain DE on the headline shape: trials per target k,
    Adam steps per training generation, and training every G-th generation. For each point, the
    exact evaluations and wall time to an FP64 error of 1e-8 on the rotated sphere, and the
    exact evaluations and wall time to the plain run's 200-generation error on the rotated
    Rastrigin, each as a ratio plain / surrogate (> 1: the surrogate needs less). The Pareto
    front is over (exact-evaluation ratio, wall ratio). `grid`, if given, lists the points
    instead (dicts of k, train_steps, train_every and optionally train_batch and lr)."""
    from speo_gb300 import _lib

    sp, _ = c4_run(L, dev, torch, _lib.FUNC_ROTATED_SPHERE, "plain", 4000, stop_at=1e-8)
    rp, cp = c4_run(L, dev, torch, _lib.FUNC_ROTATED_RASTRIGIN, "plain", ras_gens)
    target = rp["final_err"]
    hit_p = first_reach(cp, target)
    points = []
    if grid is None:
        grid = [dict(k=k, train_steps=st, train_every=ev) for k in ks for st in steps for ev in every]
    for g in grid:
        k, st, ev = g["k"], g["train_steps"], g["train_every"]
        sch = dict(train_steps=st, explore=C4_EXPLORE, train_k=k, train_every=ev,
                   train_batch=g.get("train_batch", 4096), lr=g.get("lr", 1e-3))
        ss, _ = c4_run(L, dev, torch, _lib.FUNC_ROTATED_SPHERE, "surrogate", 1500, stop_at=1e-8, **sch)
        rs, cs = c4_run(L, dev, torch, _lib.FUNC_ROTATED_RASTRIGIN, "surrogate", ras_gens, **sch)
        pt = {"k": k, "train_steps": st, "train_every": ev, "train_batch": sch["train_batch"], "lr": sch["lr"],
              "gens_per_s": rs["gens_per_s"]}
        if ss["exact_evals_to_target"]:
            pt["sphere"] = {"evals_ratio": sp["exact_evals_to_target"] / ss["exact_evals_to_target"],
                            "wall_ratio": sp["wall_s_to_target"] / ss["wall_s_to_target"],
                            "generations": ss["generations"]}
        else:
            pt["sphere"] = {"reached": False, "final_err": ss["final_err"]}
        hit = first_reach(cs, target)
        pt["rastrigin"] = ({"evals_ratio": hit_p["exact_evals"] / hit["exact_evals"],
                            "wall_ratio": hit_p["wall_s"] / hit["wall_s"], "at_gen": hit["gen"]}
                           if hit else {"reached": False, "final_err": rs["final_err"]})
        points.append(pt)

    def front(key):
        pts = [p for p in points if "evals_ratio" in p[key]]
        return [(p["k"], p["train_steps"], p["train_every"], p["train_batch"], p["lr"]) for p in pts
                if not any(q[key]["evals_ratio"] >= p[key]["evals_ratio"] and q[key]["wall_ratio"] >= p[key]["wall_ratio"]
                           and (q[key]["evals_ratio"], q[key]["wall_ratio"]) != (p[key]["evals_ratio"], p[key]["wall_ratio"])
                           for q in pts)]
    return {"plain": {"sphere_generations_to_1e-8": sp["generations"], "sphere_wall_s": sp["wall_s_to_target"],
                      "rastrigin_final_err": target, "gens_per_s": rp["gens_per_s"]},
            "points": points, "pareto_sphere": front("sphere"), "pareto_rastrigin": front("rastrigin"),
            "note": "points as (k, Adam steps per training generation, training every G generations); ratios are "
                    "plain / surrogate, so the north-star target is evals_ratio >= 5 and wall_ratio >= 3"}


def bench_e2e(L, dev, torch, steps: int) -> dict:
    """The headline loop over host buffers through the C ABI's island loop (speo_island_run_tc: the
    reference's IslandEA::Execute, generations and ring migration, as one call): the initial
    population, o and M^T uploaded from pinned host memory, the initial fitness evaluated (tensor
    cores), then
    `steps` generations with every generation's fitness vector read back to pinned host memory
    (on a second stream while the next launch runs); all inside the timed region (wall clock, the
    median of E2E_REPEATS runs)."""
    from speo_gb300 import _lib

    tab = headline_table(dev)
    n, ld = tab.rows, tab.ld
    rng = np.random.default_rng(0)
    h_pop = torch.from_numpy(rng.uniform(-100, 100, (n, ld)).astype(np.float32)).pin_memory()
    h_pop[:, DIM:] = 0
    h_sh = tab.inst_shift[0].cpu().pin_memory()
    h_rot = tab.inst_rot[0].cpu().pin_memory()
    h_hist = torch.zeros(steps * n, dtype=torch.float32).pin_memory()   # every generation's fitness
    stream = torch.cuda.current_stream()

    def run(nsteps):
        tab.pop[tab.cur].copy_(h_pop, non_blocking=True)
        tab.inst_shift[0].copy_(h_sh, non_blocking=True)
        tab.inst_rot[0].copy_(h_rot, non_blocking=True)
        tab.gen.zero_()
        tab.evaluate(use_tc=True)
        _lib.check(L.speo_island_run_tc(tab.d_segs.data_ptr(), N_ISLANDS, DIM, DIM, POP, tab.pop[tab.cur].data_ptr(),
                                        tab.fit[tab.cur].data_ptr(), n, tab.gen.data_ptr(), 0, nsteps, INTERVAL,
                                        MIGRANTS, tab.staging.data_ptr(), tab.max_ld, h_hist.data_ptr(),
                                        stream.cuda_stream), "speo_island_run_tc")

    run(20)
    torch.cuda.synchronize()
    dts = []
    for _ in range(E2E_REPEATS):
        t0 = time.perf_counter()
        run(steps)
        torch.cuda.synchronize()
        dts.append(time.perf_counter() - t0)
    dt = float(np.median(dts))
    h2d = (n * ld + h_sh.numel() + h_rot.numel()) * 4
    return {"value": n * steps / dt, "unit": "evals/s", "h2d_bytes_per_step": h2d / steps, "d2h_bytes_per_step": n * 4,
            "steps": steps, "repeats": E2E_REPEATS, "wall_s_each": [round(x, 6) for x in dts], "dtype": "fp32",
            "path": "speo_island_run_tc (the island loop of 128 islands of 256 as one C-ABI call: cooperative "
                    "tensor-core island-resident launches of 200 generations with the ring migration every 50 "
                    "generations inside them); "
                    "initial rows, o and M^T uploaded and the initial fitness evaluated inside the timed region, every "
                    "generation's fitness vector read back to pinned host memory"}


def bench_e2e_dropin(L, dev, torch, steps: int) -> dict:
    """The headline loop through the reference-shaped C ABI with host buffers: the initial
    population, o, M^T and the per-sub-island DEInfo uploaded from pinned host memory, the
    initial API_evaluateFitness_f32, then `steps` generations of speo_de_run_f32 (128 sub-islands
    of 256 in the reference layout, np2 = 64) with every generation's fitness vector read back to
    pinned host memory, and speo_ring_migrate (best 5 -> next sub-island's worst 5) every 50
    generations; all inside the timed region (wall clock, synchronous calls; the median of
    E2E_REPEATS runs)."""
    from speo_gb300 import _lib
    from speo_gb300 import workloads as w

    n, ld = EVALS_PER_STEP, 64
    specs, inst = w.config4_specs(FUNC)
    o, M = inst[0]
    seed = specs[0].seed
    rot = np.zeros((ld, DIM), dtype=np.float32)
    rot[:DIM] = M.T
    sh = np.zeros(ld, dtype=np.float32)
    sh[:DIM] = o
    rng = np.random.default_rng(0)
    h_pop = torch.from_numpy(rng.uniform(-100, 100, (n, ld)).astype(np.float32)).pin_memory()
    h_pop[:, DIM:] = 0
    h_rot, h_sh = torch.from_numpy(rot).pin_memory(), torch.from_numpy(sh).pin_memory()
    pop, cand = torch.empty(n, ld, device=dev), torch.zeros(n, ld, device=dev)
    pfit, cfit = torch.empty(n, device=dev), torch.empty(n, device=dev)
    d_rot, d_sh = torch.empty(ld, DIM, device=dev), torch.empty(ld, device=dev)
    rng_state = torch.zeros(16, dtype=torch.int32, device=dev)
    perm = torch.arange(n, dtype=torch.int32, device=dev)
    best = torch.zeros(N_ISLANDS, dtype=torch.int32, device=dev)
    info = (_lib.DEInfoF32 * N_ISLANDS)(*[_lib.DEInfoF32(0.9, 0.5, 4, POP) for _ in range(N_ISLANDS)])
    h_info = torch.frombuffer(bytearray(bytes(info)), dtype=torch.uint8).pin_memory()
    d_info = torch.empty_like(h_info, device=dev)
    segs = (_lib.Segment * N_ISLANDS)()
    for i in range(N_ISLANDS):  # the sub-islands as ring segments (identity permutation)
        s = segs[i]
        s.row0, s.pop_size, s.dim, s.ld, s.func_id, s.ring_next = i * POP, POP, DIM, ld, FUNC, (i + 1) % N_ISLANDS
    d_segs = torch.frombuffer(bytearray(bytes(segs)), dtype=torch.uint8).to(dev)
    staging = torch.zeros(N_ISLANDS * MIGRANTS * (ld + 1), device=dev)
    ii = _lib.IslandInfo(n, N_ISLANDS, perm.data_ptr())
    pi = _lib.ProblemInfoF32(DIM, FUNC, 1, 0, seed & 0x7fffffff, 0, 0, 100.0, -100.0)
    P = _lib.PopulationF32(pop.data_ptr(), pfit.data_ptr())
    C = _lib.PopulationF32(cand.data_ptr(), cfit.data_ptr())
    stream = torch.cuda.current_stream()
    L.speo_set_stream(ctypes.c_void_p(stream.cuda_stream))
    h_hist = torch.zeros(steps * n, dtype=torch.float32).pin_memory()  # every generation's fitness

    def run(nsteps):
        _lib.check(L.API_Initilize_f32(C, rng_state.data_ptr(), ii, pi), "API_Initilize_f32")
        pop.copy_(h_pop, non_blocking=True)
        d_rot.copy_(h_rot, non_blocking=True)
        d_sh.copy_(h_sh, non_blocking=True)
        d_info.copy_(h_info, non_blocking=True)
        L.API_evaluateFitness_f32(pfit.data_ptr(), None, None, pop.data_ptr(), d_sh.data_ptr(), d_rot.data_ptr(),
                                  None, None, None, None, n, DIM, 0.0, FUNC)
        g = 0
        for k, mig in chunks(0, nsteps):
            _lib.check(L.speo_de_run_f32(P, C, rng_state.data_ptr(), ii, d_info.data_ptr(), best.data_ptr(), pi,
                                         d_sh.data_ptr(), d_rot.data_ptr(), None, k,
                                         ctypes.c_void_p(h_hist.data_ptr() + 4 * g * n), 1, stream.cuda_stream),
                       "speo_de_run_f32")
            g += k
            if mig:
                _lib.check(L.speo_ring_migrate(d_segs.data_ptr(), N_ISLANDS, MIGRANTS, pop.data_ptr(), pfit.data_ptr(),
                                               staging.data_ptr(), ld, stream.cuda_stream), "speo_ring_migrate")
        stream.synchronize()

    run(20)
    dts = []
    for _ in range(E2E_REPEATS):
        t0 = time.perf_counter()
        run(steps)
        dts.append(time.perf_counter() - t0)
    dt = float(np.median(dts))
    _lib.check(L.API_CheckCUDAError(), "e2e")
    L.speo_set_stream(None)
    h2d = (n * ld + ld * DIM + ld) * 4 + len(bytes(info))
    return {"value": n * steps / dt, "unit": "evals/s", "h2d_bytes_per_step": h2d / steps, "d2h_bytes_per_step": n * 4,
            "steps": steps, "repeats": E2E_REPEATS, "wall_s_each": [round(x, 6) for x in dts], "dtype": "fp32",
            "path": "speo_de_run_f32 over 128 sub-islands of 256 (reference layout, np2=64): the generations of "
                    "API_DE_GenerateNewPopulation_f32 + API_evaluateFitness_f32 + API_DE_SelectSurvival_f32 "
                    "(bit-identical), every generation's fitness read back; speo_ring_migrate every 50 generations"}


def cpu_setup():
    import speo_oracle
    from speo_gb300 import workloads as w

    specs, inst = w.config4_specs(FUNC)
    o, M = inst[0]
    ld = 64
    seed = specs[0].seed
    pop = speo_oracle.init_population(EVALS_PER_STEP, ld, DIM, -100.0, 100.0, seed).astype(np.float64)
    fit = speo_oracle.evaluate_rows(FUNC, pop.astype(np.float32), DIM, o, M)
    return o, M, ld, seed, pop, fit


def cpu_generations(state, gen0: int, gens: int, threads: int) -> int:
    """gens generations of the headline workload on the host cores in FP64: the oracle port of the
    reference's DE generation (kernel_DE_CUDA.cu:172-327) and CEC2014 objective, ring migration
    at the migration points, islands spread over `threads` threads."""
    import speo_oracle

    o, M, ld, seed, pop, fit = state
    return speo_oracle.run_islands_f64(N_ISLANDS, POP, DIM, ld, FUNC, 0.5, 0.9, -100.0, 100.0, o, M, seed, gen0, gens,
                                       INTERVAL, MIGRANTS, pop, fit, threads)


def cpu_baseline(sample_s: float = 10.0) -> dict:
    threads = os.cpu_count() or 1
    state = cpu_setup()
    gens, evals, t_used, chunk = 0, 0, 0.0, 1
    while t_used < sample_s:
        t0 = time.perf_counter()
        evals += cpu_generations(state, gens, chunk, threads)
        t_used += time.perf_counter() - t0
        gens += chunk
        chunk = min(chunk * 2, 50)
    return {"value": evals / t_used, "unit": "evals/s", "cores": threads, "kind": "port",
            "sample": f"{gens} generations of the headline workload (128 x 256, D=50) in FP64, {t_used:.1f} s: the "
                      "oracle restatement of the reference's DE and CEC2014 objective, islands over "
                      f"{threads} threads"}


def bench_reference(args) -> dict | None:
    """The reference's CPU implementation of the path on the host cores: the oracle port (the
    reference's compiled CEC2014.cc is x86-only here), all host threads, exactly --warmup untimed
    and --steps timed generations of the headline workload."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return None
    threads = os.cpu_count() or 1
    state = cpu_setup()
    cpu_generations(state, 0, args.warmup, threads)
    t0 = time.perf_counter()
    evals = cpu_generations(state, args.warmup, args.steps, threads)
    t = time.perf_counter() - t0
    rate = evals / t
    return {"metric": METRIC, "value": rate, "unit": "evals/s", "n_gpus": int(os.environ.get("WORLD_SIZE", "1")),
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp64",
            "data": "synthetic (seeded o ~ U[-80,80]^50, Haar M, uniform init)", "impl": "reference",
            "config": {"workload": WORKLOAD, "islands": N_ISLANDS, "pop_size": POP, "dim": DIM, "func_id": FUNC,
                       "migration_interval": INTERVAL, "migrants": MIGRANTS,
                       "step": f"one generation over all islands ({EVALS_PER_STEP} exact evaluations)"},
            "cpu_baseline": {"value": rate, "unit": "evals/s", "cores": threads, "kind": "port",
                             "sample": f"{args.steps} timed generations after {args.warmup} warm-up, {t:.2f} s, "
                                       f"{threads} threads over islands (oracle port: the reference's compiled "
                                       "CEC2014.cc is x86-only and its sources are absent on the GPU host)"},
            "e2e": {"value": rate, "unit": "evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


# ---- secondary sections (--full): written to --sections-out, not to the record line ----------
C1_ISLANDS, C1_POP, C1_DIM = 64, 100, 30


def c1_seed() -> int:
    from speo_gb300.instances import run_seed as rs

    return rs(1, FUNC, 1)


def bench_config1(L, dev, torch, flush) -> dict:
    """Config 1, the 64 x 100 island ring at D = 30 (rotated Rastrigin, ring best-5 -> worst-5 every
    50 generations): one CUDA graph per 50-generation epoch (one island-resident launch + two
    migration launches), L2 flushed before each timed epoch; the resident kernel alone from a graph
    of back-to-back launches."""
    from speo_gb300 import workloads as w

    specs, inst = w.config1_specs()
    tab = w.table(specs, inst, device=dev, tile_rows=50)
    tab.init_population()

    def epoch():
        tab.epoch(INTERVAL)
        tab.migrate(MIGRANTS)
    g = capture(torch, epoch)
    for _ in range(3):
        g.replay()
    ms = time_graph(torch, g, 20, flush) / INTERVAL
    kg = capture(torch, lambda: tab.epoch(INTERVAL))
    launch_ms = time_graph(torch, kg, 20, flush)
    evals = C1_ISLANDS * C1_POP
    alg = evals * (5 * C1_DIM * 4 + 2 * 4) * INTERVAL
    pk = peaks()
    return {"workload": "64 islands x P=100, D=30, rotated Rastrigin, ring best-5 -> worst-5 every 50 generations",
            "ms_per_generation": ms, "evals_per_s": evals / (ms / 1e3), "gens_per_s": 1e3 / ms,
            "kernel": "k_island_epoch2<1> (two-block cluster per island, 128 blocks)",
            "launch_us_50_generations": launch_ms * 1e3, "hbm_equiv_frac": alg / (launch_ms / 1e3) / 1e9 / pk["hbm_gbs"],
            "fp32_rotation_tflops": evals * INTERVAL * 2 * C1_DIM * C1_DIM / (launch_ms / 1e3) / 1e12}


def bench_operators(L, dev, torch, pk, n_isl: int = 16384) -> dict:
    """Operator kernels on a bandwidth-scale population (measurement-only variant): 16384 islands
    x P = 128, D = 100 = 2^21 rows, 0.84 GB per FP32 buffer (> 6x L2), so every launch streams
    from HBM. Each kernel is timed alone with CUDA events (median of several launches, L2
    flushed before each); achieved = algorithmic bytes / time."""
    from speo_gb300 import _lib
    from speo_gb300.device import SegmentSpec, SegmentTable
    from speo_gb300.instances import make_instance

    P, D = 128, 100
    inst = [make_instance(c1_seed() + 1, D)]
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
    rec("k_evaluate_tc (TMA + tcgen05, two-way FP16 split)", timed(lambda: tab_tc.evaluate(which=0, use_tc=True, out=out_fit)),
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
    tensor cores in two-way split FP16 (trial generation, tensor-core evaluation and selection per generation,
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
                        "two-way split FP16 tcgen05 evaluation (three products, power-of-two row scaling)",
            "ms_per_generation": ms, "gens_per_s": 1e3 / ms, "evals_per_s": tab.rows / (ms / 1e3),
            "launches_per_generation": 3,
            "fitness_rel_err_vs_fp64": {"tcgen05_f16_split2": {"max": float(rel_tc.max()), "median": float(np.median(rel_tc)),
                                                           "p99": float(np.quantile(rel_tc, 0.99))},
                                        "cuda_core_fp32": {"max": float(rel_cc.max()), "median": float(np.median(rel_cc)),
                                                           "p99": float(np.quantile(rel_cc, 0.99))},
                                        "rows_sampled": int(len(sample))},
            "best_error_f64_min_over_islands": float(errs.min().item())}



def bench_config3(L, dev, torch, flush) -> dict:
    """Config 3: 1024 independent runs with D ~ U{10,30,50,100}, P ~ U[50,200], each with its own
    instance and objective; one launch per generation (the mixed-class kernel), 20 generations per
    CUDA graph. The tile height is the library tuner's choice (speo_autotune_tile_rows: each
    candidate timed on this table, the fastest cached for its shape bucket)."""
    from speo_gb300 import _lib
    from speo_gb300 import workloads as w

    specs, inst = w.config3_specs(1024)
    evals = sum(sp.pop_size for sp in specs)
    tab = w.table(specs, inst, device=dev, tile_rows="auto")
    tab.init_population()
    g = capture(torch, lambda: [tab.generation() for _ in range(20)])
    g.replay()
    ms = time_graph(torch, g, 5, flush) / 20
    # the same runs with the rotation on the tensor cores: trials (k = 1), speo_evaluate_tc over
    # 128-row tiles (B rebuilt at every change of instance), selection; three launches per generation
    tab_tc = w.table(specs, inst, device=dev, tile_rows=_lib.TILE_TC)
    tab_tc.init_population()
    trial = torch.zeros_like(tab_tc.pop[0])
    trial_fit = torch.zeros_like(tab_tc.fit[0])
    g_tc = capture(torch, lambda: [tab_tc.tc_generation(trial, trial_fit) for _ in range(20)])
    g_tc.replay()
    ms_tc = time_graph(torch, g_tc, 5, flush) / 20
    return {"workload": f"1024 runs, D in {{10,30,50,100}}, P in [50,200] ({evals} rows), mixed objectives",
            "ms_per_generation": ms, "gens_per_s": 1e3 / ms, "evals_per_s": evals / (ms / 1e3),
            "launches_per_generation": 1, "tile_rows": tab.tile_rows,
            "autotune_ms_per_generation": {str(k): v for k, v in tab.autotune["ms"].items()},
            "autotune_cached": tab.autotune["cached"],
            "tensor_core_form": {"ms_per_generation": ms_tc, "evals_per_s": evals / (ms_tc / 1e3),
                                 "launches_per_generation": 3, "tile_rows": _lib.TILE_TC}}


# DRAM bytes of one 50-generation island-resident launch of this workload (64 x 100, D = 30), from


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



def bench_e2e_config1(L, dev, torch, steps: int, f64: bool = False) -> dict:
    """Config 1 (64 x 100, D = 30) through the reference-shaped C ABI with host buffers: initial population + instance uploaded from
    pinned host memory, then per generation generate / evaluate / select and a read-back of
    the generation's fitness vector; all inside the timed region. f64: the same in the
    reference's shipped precision (`real` = double) through speo_de_run_f64 and the FP64 entry
    points."""
    from speo_gb300 import _lib
    from speo_gb300.instances import make_instance

    n = C1_ISLANDS * C1_POP
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
    o, M = make_instance(c1_seed(), C1_DIM)
    rot = np.zeros((ld, C1_DIM), dtype=npt)
    rot[:C1_DIM] = M.T
    sh = np.zeros(ld, dtype=npt)
    sh[:C1_DIM] = o
    rng = np.random.default_rng(0)
    h_pop = torch.from_numpy(rng.uniform(-100, 100, (n, ld)).astype(npt)).pin_memory()
    h_pop[:, C1_DIM:] = 0
    h_rot = torch.from_numpy(rot).pin_memory()
    h_sh = torch.from_numpy(sh).pin_memory()
    h_fit = torch.zeros(n, dtype=tdt).pin_memory()
    pop, cand = torch.empty(n, ld, dtype=tdt, device=dev), torch.zeros(n, ld, dtype=tdt, device=dev)
    pfit, cfit = torch.empty(n, dtype=tdt, device=dev), torch.empty(n, dtype=tdt, device=dev)
    d_rot, d_sh = torch.empty(ld, C1_DIM, dtype=tdt, device=dev), torch.empty(ld, dtype=tdt, device=dev)
    rng_state = torch.zeros(16, dtype=torch.int32, device=dev)
    perm = torch.arange(n, dtype=torch.int32, device=dev)
    best = torch.zeros(C1_ISLANDS, dtype=torch.int32, device=dev)
    info = (DI * C1_ISLANDS)(*[DI(0.9, 0.5, 4, C1_POP) for _ in range(C1_ISLANDS)])
    h_info = torch.frombuffer(bytearray(bytes(info)), dtype=torch.uint8).pin_memory()
    d_info = torch.empty_like(h_info, device=dev)
    ii = _lib.IslandInfo(n, C1_ISLANDS, perm.data_ptr())
    pi = PI(C1_DIM, FUNC, 1, 0, c1_seed(), 0, 0, 100.0, -100.0)
    P = Pop(pop.data_ptr(), pfit.data_ptr())
    C = Pop(cand.data_ptr(), cfit.data_ptr())
    stream = torch.cuda.current_stream()
    L.speo_set_stream(ctypes.c_void_p(stream.cuda_stream))
    _lib.check(init(C, rng_state.data_ptr(), ii, pi), "API_Initilize" + sfx)
    h_hist = torch.zeros(steps * n, dtype=tdt).pin_memory()  # every generation's fitness

    def upload():
        pop.copy_(h_pop, non_blocking=True)
        d_rot.copy_(h_rot, non_blocking=True)
        d_sh.copy_(h_sh, non_blocking=True)
        d_info.copy_(h_info, non_blocking=True)
        ev(pfit.data_ptr(), None, None, pop.data_ptr(), d_sh.data_ptr(), d_rot.data_ptr(), None, None, None, None, n,
           C1_DIM, 0.0, FUNC)

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
               n, C1_DIM, 0.0, FUNC)
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
    h2d = (n * ld + ld * C1_DIM + ld) * es + len(bytes(info))
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
        o, M, S = make_instance_multi(c1_seed() + fid, D, fid)
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
            pi = PI(D, fid, 1, 0, c1_seed(), 0, 0, 100.0, -100.0)
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



def sections(args) -> dict:
    """The secondary measurements (rank 0, one GPU)."""
    import torch
    from speo_gb300 import _lib

    dev = "cuda:0"
    torch.cuda.set_device(0)
    L = _lib.load()
    flush = torch.empty(128 * 1024 * 1024, dtype=torch.float32, device=dev)
    out = {"config1_island_d30": bench_config1(L, dev, torch, flush),
           "operators_bandwidth_scale": bench_operators(L, dev, torch, peaks(), args.ops_islands),
           "config2_precision": bench_config2(L, dev, torch, flush),
           "config3_batched": bench_config3(L, dev, torch, flush),
           "surrogate_mlp": bench_mlp(L, dev, torch),
           "e2e_config1_fp32": bench_e2e_config1(L, dev, torch, 1000),
           "e2e_config1_fp64": bench_e2e_config1(L, dev, torch, 1000, f64=True),
           "published_config": bench_published(L, dev, torch)}
    return out


def one_section(args) -> dict | None:
    """--ops-only / --e2e-only / --published-only / --mlp-case / --c4-only / --configs-only."""
    import torch
    from speo_gb300 import _lib

    if not (args.ops_only or args.e2e_only or args.published_only or args.mlp_case or args.c4_only
            or args.configs_only or args.surrogate_sweep or args.surrogate_batch_sweep or args.surrogate_uneven
            or args.surrogate_k_sweep):
        return None
    dev = "cuda:0"
    torch.cuda.set_device(0)
    L = _lib.load()
    if args.ops_only:
        return bench_operators(L, dev, torch, peaks(), args.ops_islands)
    if args.e2e_only:
        return {"e2e": bench_e2e(L, dev, torch, max(args.steps, 100)),
                "e2e_dropin": bench_e2e_dropin(L, dev, torch, max(args.steps, 100)),
                "e2e_config1_fp32": bench_e2e_config1(L, dev, torch, 1000),
                "e2e_config1_fp64": bench_e2e_config1(L, dev, torch, 1000, f64=True)}
    if args.published_only:
        a, b = (int(v) for v in args.published_fids.split("-"))
        return {"published_config": bench_published(L, dev, torch, fids=range(a, b + 1),
                                                    fp64=not args.published_fp32_only)}
    if args.mlp_case:
        return {"surrogate_mlp": bench_mlp(L, dev, torch)}
    if args.c4_only:
        return {"surrogate": bench_surrogate(L, dev, torch, args.c4_gens)}
    if args.surrogate_sweep:
        return {"surrogate_sweep": bench_surrogate_sweep(L, dev, torch)}
    if args.surrogate_uneven:
        return {"surrogate_uneven_islands": bench_surrogate(L, dev, torch, args.c4_gens, uneven=True)}
    if args.surrogate_batch_sweep:
        return {"surrogate_batch_sweep": bench_surrogate_sweep(L, dev, torch, grid=SURROGATE_BATCH_GRID)}
    if args.surrogate_k_sweep:
        return {"surrogate_k_sweep": bench_surrogate_sweep(L, dev, torch, grid=SURROGATE_K_GRID)}
    flush = torch.empty(128 * 1024 * 1024, dtype=torch.float32, device=dev)
    return {"config1_island_d30": bench_config1(L, dev, torch, flush),
            "config2_precision": bench_config2(L, dev, torch, flush),
            "config3_batched": bench_config3(L, dev, torch, flush),
            "surrogate": bench_surrogate(L, dev, torch, args.c4_gens)}


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000, help="timed generations")
    ap.add_argument("--warmup", type=int, default=50, help="untimed generations before the timed ones")
    ap.add_argument("--impl", default="speo", choices=["speo", "reference"])
    ap.add_argument("--cpu-sample-s", type=float, default=10.0)
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer C-ABI leg (profiling runs)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-baseline leg (profiling runs)")
    ap.add_argument("--no-surrogate", action="store_true", help="skip the surrogate-vs-plain comparison")
    ap.add_argument("--epoch", default="auto", choices=["auto", "simt", "tc"],
                    help="island-resident kernel: tensor-core rotation where supported (auto), or the CUDA-core one")
    ap.add_argument("--full", action="store_true", help="also measure the secondary sections into --sections-out")
    ap.add_argument("--sections-out", default="gpurun_out/bench_sections.json")
    ap.add_argument("--ops-only", action="store_true", help="only the bandwidth-scale operator measurements")
    ap.add_argument("--ops-islands", type=int, default=16384, help="islands of 128 rows in the operator variant")
    ap.add_argument("--configs-only", action="store_true", help="only the configuration sections")
    ap.add_argument("--c4-gens", type=int, default=200, help="rotated-Rastrigin generations of the surrogate section")
    ap.add_argument("--c4-only", action="store_true", help="only the surrogate-vs-plain section")
    ap.add_argument("--mlp-case", action="store_true", help="only the surrogate network's kernels")
    ap.add_argument("--surrogate-sweep", action="store_true",
                    help="only the surrogate schedule sweep (k, Adam steps, training interval) against plain DE")
    ap.add_argument("--launch-per-interval", action="store_true",
                    help="time the headline as one launch per migration interval with migration launches between")
    ap.add_argument("--surrogate-k-sweep", action="store_true",
                    help="only the surrogate's trials-per-target x Adam-steps sweep against plain DE")
    ap.add_argument("--surrogate-uneven", action="store_true",
                    help="only the surrogate-vs-plain section on 144 islands of uneven size (config 4's instance)")
    ap.add_argument("--surrogate-batch-sweep", action="store_true",
                    help="only the surrogate's training batch / Adam steps / learning rate sweep against plain DE")
    ap.add_argument("--e2e-only", action="store_true", help="only the end-to-end drop-in measurements")
    ap.add_argument("--published-only", action="store_true",
                    help="only the reference's published configuration (F23-F30, D=100, 4096 rows)")
    ap.add_argument("--published-fids", default="23-30", help="function ids a-b of the published configuration")
    ap.add_argument("--published-fp32-only", action="store_true", help="skip the FP64 leg of the published configuration")
    args = ap.parse_args()
    if args.steps < 1 or args.warmup < 0:
        raise SystemExit("--steps must be >= 1 and --warmup >= 0")
    if args.impl == "speo":
        single = one_section(args)
        if single is not None:
            print(json.dumps(single))
            return
    out = bench_reference(args) if args.impl == "reference" else bench_speo(args)
    if out is None or int(os.environ.get("RANK", "0")) != 0:
        return
    if args.full and args.impl == "speo":
        extra = sections(args)
        path = Path(args.sections_out)
        path.parent.mkdir(parents=True, exist_ok=True)
        path.write_text(json.dumps(extra, indent=1))
        out["sections_file"] = str(path)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
