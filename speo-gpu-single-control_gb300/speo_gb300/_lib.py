"""ctypes binding of libspeo_gb300.so (the C ABI declared in include/speo_gb300.h).

The library is loaded from the package's lib/ directory; there is no fallback: if it is
missing, importing the binding raises.
"""
from __future__ import annotations

import ctypes
from ctypes import POINTER, c_char_p, c_double, c_float, c_int, c_int32, c_int64, c_uint32, c_uint64, c_void_p
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent.parent / "lib" / "libspeo_gb300.so"

SPEO_OK = 0
SPEO_ERR_INVALID_ARG = 1
SPEO_ERR_CUDA = 2
SPEO_ERR_UNSUPPORTED = 3
SPEO_ERR_DEVICE_FLAG = 4
SPEO_DEVERR_REDRAW_LIMIT = 0x1
SPEO_DEVERR_BOUND_LIMIT = 0x2
SPEO_DEVERR_WAIT_TIMEOUT = 0x4
SPEO_DEVERR_BAD_SEGMENT = 0x8

FUNC_ROTATED_RASTRIGIN = 9
FUNC_ROTATED_SPHERE = 31
DE_RAND_1 = 4
MAX_DIM = 256
RNG_STATE_BYTES = 64
TILE_SIMT = 64
TILE_TC = 128
NOALLOC_STAGING_FLOATS = 1 << 20


class Segment(ctypes.Structure):
    """speo_segment."""
    _fields_ = [
        ("row0", c_int64), ("pop_size", c_int32), ("dim", c_int32), ("ld", c_int32),
        ("func_id", c_int32), ("strategy", c_int32), ("F", c_float), ("CR", c_float),
        ("lb", c_float), ("ub", c_float), ("shift", c_void_p), ("rot", c_void_p),
        ("ld_rot", c_int32), ("ring_next", c_int32), ("seed", c_uint64), ("shuffle", c_void_p),
    ]


class Archipelago(ctypes.Structure):
    """speo_archipelago: islands of one device and the reference's migration parameters."""
    _fields_ = [
        ("n_islands", c_int32), ("island_size", c_int32), ("dim", c_int32), ("ld", c_int32),
        ("migration_size", c_int32), ("buffer_capacity", c_int32), ("buffer_policy", c_int32),
        ("regroup_option", c_int32), ("migration_rate", c_float), ("reserved", c_int32), ("seed", c_uint64),
    ]


BUFFER_ONLINE_CLUSTER, BUFFER_BEST, BUFFER_RANDOM, BUFFER_FIFO, BUFFER_LIFO = range(5)
REGROUP_STATIC_ORDERED, REGROUP_STATIC_RANDOM, REGROUP_DYNAMIC_ORDERED, REGROUP_DYNAMIC_RANDOM = range(4)


class WorkItem(ctypes.Structure):
    """speo_work_item."""
    _fields_ = [("segment", c_int32), ("first", c_int32), ("count", c_int32), ("pad", c_int32)]


class PopulationF32(ctypes.Structure):
    _fields_ = [("elements", c_void_p), ("fitness_value", c_void_p)]


class PopulationF64(ctypes.Structure):
    _fields_ = [("elements", c_void_p), ("fitness_value", c_void_p)]


class IslandInfo(ctypes.Structure):
    _fields_ = [("island_size", c_int), ("subisland_num", c_int), ("permutated_index", c_void_p)]


class DEInfoF32(ctypes.Structure):
    _fields_ = [("CR", c_float), ("F", c_float), ("strategy_ID", c_int), ("pop_size", c_int)]


class DEInfoF64(ctypes.Structure):
    _fields_ = [("CR", c_double), ("F", c_double), ("strategy_ID", c_int), ("pop_size", c_int)]


class ProblemInfoF32(ctypes.Structure):
    _fields_ = [("dim", c_int), ("function_ID", c_int), ("run_ID", c_int), ("max_base_FEs", c_int),
                ("seed", c_int), ("running_time", c_int), ("computing_time", c_int),
                ("max_bound", c_float), ("min_bound", c_float)]


class ProblemInfoF64(ctypes.Structure):
    _fields_ = [("dim", c_int), ("function_ID", c_int), ("run_ID", c_int), ("max_base_FEs", c_int),
                ("seed", c_int), ("running_time", c_int), ("computing_time", c_int),
                ("max_bound", c_double), ("min_bound", c_double)]


# name -> (restype, argtypes)
SIGNATURES: dict[str, tuple] = {
    "API_Initilize": (c_int, [PopulationF64, c_void_p, IslandInfo, ProblemInfoF64]),
    "API_Initilize_f32": (c_int, [PopulationF32, c_void_p, IslandInfo, ProblemInfoF32]),
    "API_CheckCUDAError": (c_int, []),
    "API_DE_GenerateNewPopulation": (c_int, [PopulationF64, PopulationF64, c_void_p, IslandInfo, c_void_p, c_void_p,
                                             ProblemInfoF64]),
    "API_DE_GenerateNewPopulation_f32": (c_int, [PopulationF32, PopulationF32, c_void_p, IslandInfo, c_void_p,
                                                 c_void_p, ProblemInfoF32]),
    "API_DE_SelectSurvival": (c_int, [PopulationF64, PopulationF64, IslandInfo, ProblemInfoF64]),
    "API_DE_SelectSurvival_f32": (c_int, [PopulationF32, PopulationF32, IslandInfo, ProblemInfoF32]),
    "speo_configure_de_f32": (c_int, [c_void_p, c_int, c_int, c_float, c_float, c_int, c_int, c_uint64]),
    "speo_configure_de_f64": (c_int, [c_void_p, c_int, c_int, c_double, c_double, c_int, c_int, c_uint64]),
    "speo_de_run_f32": (c_int, [PopulationF32, PopulationF32, c_void_p, IslandInfo, c_void_p, c_void_p, ProblemInfoF32,
                                c_void_p, c_void_p, c_void_p, c_int, c_void_p, c_int, c_void_p]),
    "speo_de_run_f64": (c_int, [PopulationF64, PopulationF64, c_void_p, IslandInfo, c_void_p, c_void_p, ProblemInfoF64,
                                c_void_p, c_void_p, c_void_p, c_int, c_void_p, c_int, c_void_p]),
    "API_evaluateFitness": (None, [c_void_p] * 10 + [c_int, c_int, c_double, c_int]),
    "API_evaluateFitness_f32": (None, [c_void_p] * 10 + [c_int, c_int, c_float, c_int]),
    "speo_set_stream": (c_int, [c_void_p]),
    "speo_last_error": (c_char_p, []),
    "speo_device_error_bits": (c_int, [POINTER(c_uint32)]),
    "speo_version": (c_char_p, []),
    "speo_plan_work": (c_int, [c_void_p, c_int, c_int, c_void_p, c_int, POINTER(c_int)]),
    "speo_init_population": (c_int, [c_void_p, c_int, c_void_p, c_int, c_void_p, c_void_p]),
    "speo_evaluate": (c_int, [c_void_p, c_void_p, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p]),
    "speo_evaluate_tc": (c_int, [c_void_p, c_void_p, c_int, c_int, c_int, c_void_p, c_int64, c_int, c_void_p,
                                 c_void_p]),
    "speo_generation": (c_int, [c_void_p, c_void_p, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p,
                                c_void_p, c_int, c_void_p, c_void_p, c_void_p]),
    "speo_epoch_fits": (c_int, [c_int, c_int]),
    "speo_generation_epoch": (c_int, [c_void_p, c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p,
                                      c_void_p, c_int, c_void_p]),
    "speo_generation_epoch_ex": (c_int, [c_void_p, c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p,
                                         c_void_p, c_void_p, c_int, c_int, c_void_p]),
    "speo_epoch_tc_fits": (c_int, [c_int, c_int]),
    "speo_island_run_tc": (c_int, [c_void_p, c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_int64, c_void_p, c_int,
                                   c_int, c_int, c_int, c_void_p, c_int, c_void_p, c_void_p]),
    "speo_island_epochs_tc": (c_int, [c_void_p, c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_int64, c_void_p,
                                      c_int, c_int, c_int, c_int, c_void_p, c_int, c_void_p]),
    "speo_autotune_tile_rows": (c_int, [c_void_p, c_int, c_void_p, c_int, c_int, c_void_p, c_void_p, c_void_p,
                                        c_void_p]),
    "speo_autotune_set_tile_rows": (c_int, [c_void_p, c_int, c_void_p, c_int, c_int]),
    "speo_generation_epoch_tc": (c_int, [c_void_p, c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p,
                                         c_void_p, c_void_p, c_int, c_void_p]),
    "speo_generation_tc": (c_int, [c_void_p, c_void_p, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p,
                                   c_void_p, c_int64, c_int, c_void_p, c_void_p, c_void_p, c_void_p]),
    "speo_ring_migrate": (c_int, [c_void_p, c_int, c_int, c_void_p, c_void_p, c_void_p, c_int, c_void_p]),
    "speo_ring_migrate_noalloc": (c_int, [c_void_p, c_int, c_int, c_void_p, c_void_p, c_int, c_void_p]),
    "speo_archipelago_state_bytes": (ctypes.c_size_t, [c_void_p]),
    "speo_archipelago_init": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_void_p]),
    "speo_migrate_out": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_uint32, c_void_p]),
    "speo_migrate_in": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_uint32, c_void_p]),
    "speo_surrogate_create": (c_int, [c_void_p, c_int, c_int, ctypes.c_longlong, c_int, c_float, c_float, c_uint64]),
    "speo_surrogate_destroy": (c_int, [c_void_p]),
    "speo_surrogate_params": (c_int, [c_void_p, c_void_p, c_void_p, POINTER(c_int)]),
    "speo_surrogate_forward": (c_int, [c_void_p, c_void_p, c_int, c_int, c_void_p, c_void_p]),
    "speo_surrogate_forward_bf16": (c_int, [c_void_p, c_void_p, c_int64, c_int, c_void_p, c_void_p]),
    "speo_surrogate_grad_bf16": (c_int, [c_void_p, c_void_p, c_int, c_int, c_void_p, POINTER(c_float), c_void_p]),
    "speo_surrogate_set_mode": (c_int, [c_void_p, c_int]),
    "speo_surrogate_grad": (c_int, [c_void_p, c_void_p, c_int, c_int, c_void_p, POINTER(c_float), c_void_p]),
    "speo_surrogate_adam_step": (c_int, [c_void_p, c_void_p]),
    "speo_surrogate_standardize": (c_int, [c_void_p, c_void_p, ctypes.c_longlong, c_int, c_void_p]),
    "speo_surrogate_archive_append": (c_int, [c_void_p, c_void_p, c_int, c_int, c_void_p, c_void_p]),
    "speo_surrogate_train": (c_int, [c_void_p, c_int, POINTER(c_float), c_void_p]),
    "speo_make_trials": (c_int, [c_void_p, c_void_p, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p,
                                 c_void_p]),
    "speo_surrogate_generation": (c_int, [c_void_p, c_void_p, c_void_p, c_int, c_int, c_int, ctypes.c_longlong, c_int,
                                          c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_float,
                                          c_void_p]),
    "speo_select_rows": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, ctypes.c_longlong, c_int,
                                 c_void_p]),
    "speo_best_reeval_f64": (c_int, [c_void_p, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
}

_lib = None


def load() -> ctypes.CDLL:
    """Loads libspeo_gb300.so once and declares every entry point's signature."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(f"{LIB_PATH} is missing: run __graft_entry__.build() (no CPU fallback exists)")
    lib = ctypes.CDLL(str(LIB_PATH))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class SpeoError(RuntimeError):
    def __init__(self, status: int, where: str):
        msg = load().speo_last_error().decode(errors="replace")
        super().__init__(f"{where}: status {status}: {msg}")
        self.status = status


def check(status: int, where: str) -> None:
    if status != SPEO_OK:
        raise SpeoError(status, where)
