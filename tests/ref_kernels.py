"""Runs the reference's own DE / EA CUDA kernels (compiled from its sources into
oracle/_ref/*.fatbin) and this project's XORWOW capture kernel through the CUDA driver API.

Test helper only: it lets the tests pin the oracle's DE restatement against the reference's
GPU kernel on identical cuRAND streams.
"""
from __future__ import annotations

import ctypes
from ctypes import byref, c_int, c_uint, c_void_p
from pathlib import Path

REPO = Path(__file__).resolve().parent.parent
REF_DIR = REPO / "oracle" / "_ref"


def reference_root() -> Path | None:
    """The reference project directory the oracle build read its sources from (recorded by
    `make -C oracle ref` in oracle/_ref/REFERENCE_ROOT), or None where it was not built or the
    sources are absent."""
    rec = REF_DIR / "REFERENCE_ROOT"
    if not rec.exists():
        return None
    root = Path(rec.read_text().strip())
    return root if root.is_dir() else None
CAPTURE = REPO / "oracle" / "lib" / "xorwow_capture.fatbin"

# Itanium-mangled names of the reference's kernels (host stub names of the same build).
K_SETUP = b"_Z23global_SetupRandomStateP17curandStateXORWOWi"
K_INIT = b"_Z22global_InitiPopulation14GPU_PopulationP17curandStateXORWOW11ProblemInfo"
K_BEST = b"_Z36global_DE_FindBestIndividualInIslandPi14GPU_Population14GPU_IslandInfo11ProblemInfo"
K_GEN = b"_Z31global_DE_GenerateNewPopulation14GPU_PopulationS_Pi14GPU_IslandInfoP6DEInfoP17curandStateXORWOW11ProblemInfo"
K_SEL = b"_Z24global_DE_SelectSurvival14GPU_PopulationS_11ProblemInfo"
CURAND_STATE_BYTES = 48  # sizeof(curandStateXORWOW)
# kernel_CEC2014_CUDA.cu: global_ShiftAndRotation (:147-181) and global_f8 (:557-587), per precision
K_SR = {"f64": b"_Z23global_ShiftAndRotationPdS_S_S_iiiiiii", "f32": b"_Z23global_ShiftAndRotationPfS_S_S_iiiiiii"}
K_F8 = {"f64": b"_Z9global_f8PdS_iidddd", "f32": b"_Z9global_f8PfS_iiffff"}
# the elementwise bodies global_f1..f4 (:254-387), global_Shift (:183-195), global_CalW (:74-122),
# global_CombineFitness (:197-206): what CompFunc1 (F23, :1416-1451) launches
K_FN = {p: {n: f"_Z9global_f{n}{'PdS_iidddd' if p == 'f64' else 'PfS_iiffff'}".encode() for n in (1, 2, 3, 4)}
        for p in ("f64", "f32")}
K_SHIFT = {"f64": b"_Z12global_ShiftPdS_S_iii", "f32": b"_Z12global_ShiftPfS_S_iii"}
K_CALW = {"f64": b"_Z11global_CalWPdS_S_S_ii", "f32": b"_Z11global_CalWPfS_S_S_ii"}
K_COMBINE = {"f64": b"_Z21global_CombineFitnessPdS_iS_idd", "f32": b"_Z21global_CombineFitnessPfS_iS_iff"}


def available(precision: str, kinds=("de", "ea")) -> bool:
    return all((REF_DIR / f"ref_{k}_{precision}.fatbin").exists() for k in kinds) and CAPTURE.exists()


class Driver:
    def __init__(self):
        self.cu = ctypes.CDLL("libcuda.so.1")
        self._mods = {}

    def check(self, r, what):
        if r != 0:
            raise RuntimeError(f"{what}: CUresult {r}")

    def module(self, path: Path):
        if path not in self._mods:
            data = path.read_bytes()
            buf = ctypes.create_string_buffer(data, len(data))
            mod = c_void_p()
            self.check(self.cu.cuModuleLoadData(byref(mod), buf), f"cuModuleLoadData({path.name})")
            self._mods[path] = (mod, buf)
        return self._mods[path][0]

    def function(self, path: Path, name: bytes):
        fn = c_void_p()
        self.check(self.cu.cuModuleGetFunction(byref(fn), self.module(path), name), f"cuModuleGetFunction({name})")
        return fn

    def launch(self, fn, grid, block, args, smem=0, sync=True):
        """args: ctypes objects (scalars or Structures), passed by value. sync: a context
        synchronisation after the launch (the reference's CudaCheckError does one)."""
        ptrs = (c_void_p * len(args))(*[ctypes.cast(ctypes.pointer(a), c_void_p) for a in args])
        self.check(self.cu.cuLaunchKernel(fn, c_uint(grid[0]), c_uint(grid[1]), c_uint(grid[2]), c_uint(block[0]),
                                          c_uint(block[1]), c_uint(block[2]), c_uint(smem), None, ptrs, None),
                   "cuLaunchKernel")
        if sync:
            self.check(self.cu.cuCtxSynchronize(), "cuCtxSynchronize")


def de_config(pop_size: int):
    """CalConfigurations / CalConfigurationsDE (kernel_EA_CUDA.cu:7-21, kernel_DE_CUDA.cu:48-62)."""
    if pop_size > 16:
        return (pop_size // 16, 1, 1), (32, 16, 1)
    return (1, 1, 1), (32, pop_size, 1)


def c_int_(v):
    return c_int(v)
