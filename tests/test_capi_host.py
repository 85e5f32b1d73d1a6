"""CPU tests of the C ABI: the library loads, exports every declared entry point, its
by-value structs have the reference's layouts, and host-side logic (work planning, argument
validation) behaves without a GPU."""
from __future__ import annotations

import ctypes
import re
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parent.parent
HEADER = REPO / "include" / "speo_gb300.h"
sys.path.insert(0, str(Path(__file__).resolve().parent))
from ref_kernels import reference_root  # noqa: E402

_REF_ROOT = reference_root()
REF_LIB_DIR = (_REF_ROOT / "CUDA_EA_library") if _REF_ROOT else Path("/nonexistent")


def declared_functions() -> list[str]:
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:SPEO_API\s+)?(?:const\s+)?(?:int|void|char|size_t|u?int(?:32|64)_t)\s*\*?\s*"
                       r"([A-Za-z_]\w*)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_header_declares_reference_entry_points():
    names = declared_functions()
    for ref_name in ("API_Initilize", "API_CheckCUDAError", "API_DE_GenerateNewPopulation", "API_DE_SelectSurvival",
                     "API_evaluateFitness"):
        assert ref_name in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_bindings_cover_the_header_exactly():
    """Every function the header declares has a ctypes signature, and every signature names a
    declared function."""
    from speo_gb300 import _lib

    declared = set(declared_functions())
    assert "speo_archipelago_state_bytes" in declared
    assert declared == set(_lib.SIGNATURES), (declared ^ set(_lib.SIGNATURES))


def test_version(lib):
    assert b"sm_103a" in lib.speo_version()


def _segments(P_list, D=30):
    from speo_gb300 import _lib

    segs = (_lib.Segment * len(P_list))()
    row = 0
    for i, P in enumerate(P_list):
        segs[i].row0, segs[i].pop_size, segs[i].dim, segs[i].ld = row, P, D, 32
        row += P
    return segs


@pytest.mark.parametrize("tile", [1, 50, 64, 128])
def test_plan_work_covers_rows_once(lib, tile):
    from speo_gb300 import _lib

    P_list = [100, 4, 257, 64, 1000]
    segs = _segments(P_list)
    n = ctypes.c_int()
    assert lib.speo_plan_work(ctypes.addressof(segs), len(P_list), tile, None, 0, ctypes.byref(n)) == 0
    items = (_lib.WorkItem * n.value)()
    assert lib.speo_plan_work(ctypes.addressof(segs), len(P_list), tile, ctypes.addressof(items), n.value,
                              ctypes.byref(n)) == 0
    for s, P in enumerate(P_list):
        mine = sorted((it.first, it.count) for it in items if it.segment == s)
        covered = np.zeros(P, dtype=int)
        for a, c in mine:
            assert 1 <= c <= tile
            covered[a:a + c] += 1
        assert np.all(covered == 1)
        counts = [c for _, c in mine]
        assert max(counts) - min(counts) <= 1          # balanced tiles


def test_plan_work_rejects_bad_input(lib):
    segs = _segments([10])
    n = ctypes.c_int()
    assert lib.speo_plan_work(ctypes.addressof(segs), 1, 0, None, 0, ctypes.byref(n)) == 1
    segs[0].pop_size = 0
    assert lib.speo_plan_work(ctypes.addressof(segs), 1, 8, None, 0, ctypes.byref(n)) == 1
    assert b"pop_size" in lib.speo_last_error()


def test_dropin_validation_happens_before_any_device_work(lib):
    """Invalid shapes are reported as status codes (the reference exits instead)."""
    from speo_gb300 import _lib

    pop = _lib.PopulationF32(1, 1)        # never dereferenced: validation fails first
    ii = _lib.IslandInfo(10, 3, 1)        # 10 not divisible by 3
    pi = _lib.ProblemInfoF32(30, 9, 1, 0, 1, 0, 0, 100.0, -100.0)
    assert lib.API_DE_SelectSurvival_f32(pop, pop, ii, pi) == _lib.SPEO_ERR_INVALID_ARG
    assert b"divisible" in lib.speo_last_error()
    ii = _lib.IslandInfo(10, 1, 1)
    pi.dim = 0
    assert lib.API_Initilize_f32(pop, None, ii, pi) == _lib.SPEO_ERR_INVALID_ARG
    pi.dim = 300
    assert lib.API_Initilize_f32(pop, None, ii, pi) == _lib.SPEO_ERR_INVALID_ARG


def test_noalloc_migration_validation_happens_before_any_device_work(lib):
    """speo_ring_migrate_noalloc rejects k outside [1, 32], no segments and a staging need one
    float past its fixed array, all before it touches the device (pointers never dereferenced)."""
    from speo_gb300 import _lib

    lim = _lib.NOALLOC_STAGING_FLOATS
    for n_segs, k, max_ld, what in ((1, 0, 64, b"outside"), (1, 33, 64, b"outside"), (0, 5, 64, b"bad arguments"),
                                    (1, 5, 0, b"bad arguments"), (1, 1, lim, b"exceed the fixed"),
                                    (2, 1, lim // 2, b"exceed the fixed"), (64, 32, 2 ** 31 - 1, b"exceed the fixed")):
        st = lib.speo_ring_migrate_noalloc(1, n_segs, k, 1, 1, max_ld, None)
        assert st == _lib.SPEO_ERR_INVALID_ARG, (n_segs, k, max_ld)
        assert what in lib.speo_last_error(), (n_segs, k, max_ld, lib.speo_last_error())


def test_autotune_cache_buckets_without_a_device(lib):
    """The tuner's cache: a choice set for one table is returned, without device work, for any
    table of the same shape bucket (column classes, log2 of rows, largest island, segments and the
    candidate list); a table of another bucket is not answered from it."""
    import ctypes as C

    from speo_gb300 import _lib

    def table(P_list, D):
        segs = _segments(P_list, D)
        for sg in segs:
            sg.ld = (D + 3) // 4 * 4
        return segs

    cand = (C.c_int * 3)(32, 48, 64)
    a = table([100] * 64, 30)
    assert lib.speo_autotune_set_tile_rows(C.addressof(a), 64, C.addressof(cand), 3, 48) == 0
    tile, cached, ms = C.c_int(0), C.c_int(0), (C.c_float * 3)()
    b = table([90] * 70, 31)                     # same classes and log2 buckets: answered from the cache
    assert lib.speo_autotune_tile_rows(C.addressof(b), 70, C.addressof(cand), 3, 5, C.byref(tile), C.addressof(ms),
                                       C.byref(cached), None) == 0
    assert tile.value == 48 and cached.value == 1 and list(ms) == [-1.0] * 3
    for other, n in ((table([100] * 64, 50), 64), (table([300] * 64, 30), 64), (table([100] * 8, 30), 8)):
        st = lib.speo_autotune_tile_rows(C.addressof(other), n, C.addressof(cand), 3, 5, C.byref(tile), None,
                                         C.byref(cached), None)
        assert cached.value == 0 and st != 0      # another bucket: it would have to be timed
    cand2 = (C.c_int * 2)(32, 64)                # another candidate list is another bucket
    assert lib.speo_autotune_tile_rows(C.addressof(b), 70, C.addressof(cand2), 2, 5, C.byref(tile), None,
                                       C.byref(cached), None) != 0
    bad = (C.c_int * 1)(0)
    assert lib.speo_autotune_set_tile_rows(C.addressof(a), 64, C.addressof(bad), 1, 8) == _lib.SPEO_ERR_INVALID_ARG


@pytest.mark.parametrize("f64", [False, True])
def test_empty_populations_are_status_codes(lib, f64):
    """Zero-row islands and populations come back as SPEO_ERR_INVALID_ARG from every drop-in
    entry point (the reference would launch empty grids or divide by zero)."""
    from speo_gb300 import _lib

    Pop, PI = (_lib.PopulationF64, _lib.ProblemInfoF64) if f64 else (_lib.PopulationF32, _lib.ProblemInfoF32)
    sfx = "" if f64 else "_f32"
    pop = Pop(16, 16)                      # never dereferenced
    pi = PI(30, 9, 1, 0, 1, 0, 0, 100.0, -100.0)
    for ii in (_lib.IslandInfo(0, 1, 16), _lib.IslandInfo(10, 0, 16)):
        assert getattr(lib, "API_Initilize" + sfx)(pop, None, ii, pi) == _lib.SPEO_ERR_INVALID_ARG
        assert getattr(lib, "API_DE_GenerateNewPopulation" + sfx)(pop, pop, 16, ii, 16, 16, pi) == \
            _lib.SPEO_ERR_INVALID_ARG
        assert getattr(lib, "API_DE_SelectSurvival" + sfx)(pop, pop, ii, pi) == _lib.SPEO_ERR_INVALID_ARG
    # the void evaluation entry point records the failure (API_CheckCUDAError returns it on a GPU)
    getattr(lib, "API_evaluateFitness" + sfx)(16, None, None, 16, 16, 16, None, None, None, None, 0, 30, 0.0, 9)
    assert b"pop_size 0" in lib.speo_last_error()


@pytest.mark.parametrize("f64", [False, True])
def test_de_run_validation_happens_before_any_device_work(lib, f64):
    """speo_de_run_f32 / _f64 report missing buffers and negative generation counts as status
    codes, naming the entry point, before touching the device."""
    from speo_gb300 import _lib

    Pop, PI, run = ((_lib.PopulationF64, _lib.ProblemInfoF64, lib.speo_de_run_f64) if f64 else
                    (_lib.PopulationF32, _lib.ProblemInfoF32, lib.speo_de_run_f32))
    name = b"speo_de_run_f64" if f64 else b"speo_de_run_f32"
    pop = Pop(16, 16)                      # never dereferenced
    ii = _lib.IslandInfo(100, 1, 16)
    pi = PI(30, 9, 1, 0, 1, 0, 0, 100.0, -100.0)
    args = [pop, pop, 16, ii, 16, 16, pi, 16, 16, None, 5, None, 0, None]
    for k in (2, 4, 5, 7, 8):              # rng, DE info, best ids, shift, rotation
        bad = list(args)
        bad[k] = None
        assert run(*bad) == _lib.SPEO_ERR_INVALID_ARG
        assert name in lib.speo_last_error()
    bad = list(args)
    bad[10] = -1                           # generations
    assert run(*bad) == _lib.SPEO_ERR_INVALID_ARG


@pytest.mark.parametrize("fid", [-1, 0, 32, 33])
def test_evaluate_rejects_unimplemented_function_id(lib, fid):
    """Ids 1-30 (CEC2014) and 31 (rotated sphere) are implemented; any other id is refused
    before any device work."""
    lib.API_evaluateFitness_f32(*([ctypes.c_void_p(1)] * 10), 100, 30, 0.0, fid)
    assert f"function_ID {fid} is not implemented".encode() in lib.speo_last_error()


@pytest.mark.parametrize("fid", [17, 22, 29, 30])
def test_evaluate_hybrids_need_shuffle(lib, fid):
    """The hybrid functions and the compositions of hybrids read the shuffle data; without it the
    call is refused before any device work."""
    args = [ctypes.c_void_p(1)] * 10
    args[6] = None
    lib.API_evaluateFitness_f32(*args, 100, 30, 0.0, fid)
    assert f"function_ID {fid} needs the shuffle data".encode() in lib.speo_last_error()


@pytest.mark.parametrize("fid,D", [(17, 2), (21, 3), (22, 4), (29, 2), (30, 3)])
def test_evaluate_hybrids_refuse_dims_without_every_group(lib, fid, D):
    """A hybrid is defined only where each of its groups gets a coordinate (CEC2014.cc:350 excludes
    D = 2); such dimensions are refused."""
    lib.API_evaluateFitness_f32(*([ctypes.c_void_p(1)] * 10), 100, D, 0.0, fid)
    assert f"function_ID {fid} is not defined for dim {D}".encode() in lib.speo_last_error()


def test_struct_layouts_match_c(tmp_path):
    """sizeof/offsetof of the ABI structs from a C compile of the header agree with ctypes."""
    from speo_gb300 import _lib

    src = r'''
#include <stdio.h>
#include <stddef.h>
#include "speo_gb300.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\n", sizeof(speo_segment), offsetof(speo_segment, shift),
         offsetof(speo_segment, seed), sizeof(speo_work_item), sizeof(speo_problem_info_f64),
         offsetof(speo_problem_info_f64, max_bound), sizeof(speo_de_info_f64), sizeof(speo_island_info),
         offsetof(speo_segment, shuffle), sizeof(speo_archipelago), offsetof(speo_archipelago, migration_rate),
         offsetof(speo_archipelago, seed));
  return 0; }
'''
    build = tmp_path
    (build / "abi_probe.c").write_text(src)
    exe = build / "abi_probe"
    subprocess.run(["gcc", "-I", str(REPO / "include"), str(build / "abi_probe.c"), "-o", str(exe)], check=True)
    vals = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    expect = [ctypes.sizeof(_lib.Segment), _lib.Segment.shift.offset, _lib.Segment.seed.offset,
              ctypes.sizeof(_lib.WorkItem), ctypes.sizeof(_lib.ProblemInfoF64), _lib.ProblemInfoF64.max_bound.offset,
              ctypes.sizeof(_lib.DEInfoF64), ctypes.sizeof(_lib.IslandInfo), _lib.Segment.shuffle.offset,
              ctypes.sizeof(_lib.Archipelago), _lib.Archipelago.migration_rate.offset, _lib.Archipelago.seed.offset]
    assert vals == expect


@pytest.mark.skipif(not (REF_LIB_DIR / "config.h").exists(), reason="reference sources not present")
def test_problem_info_layout_matches_reference_config(tmp_path):
    """speo_problem_info_f64 has the layout of the reference's ProblemInfo with real = double
    (CUDA_EA_library/config.h:31-34,48-59), so by-value calls bind unchanged."""
    src = r'''
#include "config.h"
#include "speo_gb300.h"
#include <cstddef>
static_assert(sizeof(ProblemInfo) == sizeof(speo_problem_info_f64), "size");
static_assert(offsetof(ProblemInfo, max_bound) == offsetof(speo_problem_info_f64, max_bound), "max_bound");
static_assert(offsetof(ProblemInfo, min_bound) == offsetof(speo_problem_info_f64, min_bound), "min_bound");
static_assert(offsetof(ProblemInfo, seed) == offsetof(speo_problem_info_f64, seed), "seed");
int main() { return 0; }
'''
    build = tmp_path
    (build / "abi_ref.cc").write_text(src)
    subprocess.run(["g++", "-fsyntax-only", "-I", str(REF_LIB_DIR), "-I", str(REPO / "include"),
                    str(build / "abi_ref.cc")], check=True)


@pytest.mark.parametrize("f64", [False, True])
def test_configure_de_constant_and_dynamic(lib, oracle, f64):
    """DE_CUDA::ConfigureEA (DE_CUDA.cc:89-118): "constant" repeats one setting; "dynamic" picks CR
    in {0.1, 0.9} and strategy in {4, 6} per sub-island, here from Philox({i, 0, 0, 6}, seed)."""
    from speo_gb300 import _lib

    DI = _lib.DEInfoF64 if f64 else _lib.DEInfoF32
    fn = lib.speo_configure_de_f64 if f64 else lib.speo_configure_de_f32
    n = 256
    info = (DI * n)()
    assert fn(ctypes.addressof(info), n, n * 100, 0.5, 0.8, 5, 0, 1) == 0
    assert all((x.CR, x.strategy_ID, x.pop_size) == (pytest.approx(0.8), 5, 100) for x in info)
    assert fn(ctypes.addressof(info), n, n * 100, 0.5, 0.8, 5, 1, 1234) == 0
    crs = np.array([x.CR for x in info])
    sts = np.array([x.strategy_ID for x in info])
    assert set(np.round(crs, 6)) == {0.1, 0.9} and set(sts) == {4, 6}
    assert all(x.F == pytest.approx(0.5) and x.pop_size == 100 for x in info)
    key = oracle.key_of(1234)
    for i in range(n):
        w = oracle.philox([i, 0, 0, 6], key)
        assert (crs[i] > 0.5) == bool(w[0] & 1) and (sts[i] == 6) == bool(w[1] & 1)
    assert 60 < (crs > 0.5).sum() < 196 and 60 < (sts == 6).sum() < 196
    assert fn(ctypes.addressof(info), n, n * 100 + 1, 0.5, 0.8, 5, 0, 1) == _lib.SPEO_ERR_INVALID_ARG

