"""In-tree build of libspeo_gb300.so (sm_103a) and of the oracle's C library.

The CUDA translation units under csrc/ are compiled in parallel with nvcc for
sm_103a only and linked into ``lib/libspeo_gb300.so`` next to this package. A unit is
rebuilt only when it or a header is newer than its object file.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG_ROOT = Path(__file__).resolve().parent.parent          # speo-gpu-single-control_gb300/
REPO_ROOT = PKG_ROOT.parent
CSRC = PKG_ROOT / "csrc"
BUILD = PKG_ROOT / "_build"
LIB_DIR = PKG_ROOT / "lib"
LIB_PATH = LIB_DIR / "libspeo_gb300.so"
INCLUDE = REPO_ROOT / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-fvisibility=hidden",
              "--expt-relaxed-constexpr", "-Xptxas=-warn-spills", "-I", str(INCLUDE)]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def _headers() -> list[Path]:
    return sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + sorted(INCLUDE.glob("*.h"))


def _compile(src: Path, verbose: bool) -> Path:
    obj = BUILD / (src.stem + ".o")
    newest_dep = max([src.stat().st_mtime] + [h.stat().st_mtime for h in _headers()])
    if obj.exists() and obj.stat().st_mtime >= newest_dep:
        return obj
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{res.stdout}\n{res.stderr}")
    if verbose and res.stderr:
        sys.stderr.write(res.stderr)
    return obj


def build_library(verbose: bool = False, jobs: int | None = None) -> Path:
    """Compiles every csrc/*.cu for sm_103a and links lib/libspeo_gb300.so."""
    BUILD.mkdir(exist_ok=True)
    LIB_DIR.mkdir(exist_ok=True)
    srcs = _sources()
    with ThreadPoolExecutor(max_workers=jobs or min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    if LIB_PATH.exists() and LIB_PATH.stat().st_mtime >= max(o.stat().st_mtime for o in objs):
        return LIB_PATH
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(LIB_PATH), *map(str, objs)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    return LIB_PATH


CLI_SRC = PKG_ROOT / "app" / "speo_gpu.cc"
CLI_PATH = LIB_DIR / "speo_gpu"


def build_cli() -> Path:
    """Builds lib/speo_gpu, the reference driver's command line (src/main.cc flags, Results/SPEO_GPU.csv)
    over libspeo_gb300.so; host C++ compiled and linked by nvcc."""
    lib = build_library()
    deps = [CLI_SRC, lib, INCLUDE / "speo_gb300.h"]
    if CLI_PATH.exists() and CLI_PATH.stat().st_mtime >= max(d.stat().st_mtime for d in deps):
        return CLI_PATH
    cmd = [nvcc(), "-O2", "-std=c++17", "-I", str(INCLUDE), str(CLI_SRC), "-o", str(CLI_PATH), "-L", str(LIB_DIR),
           "-lspeo_gb300", "-Xlinker", "-rpath,$ORIGIN"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"speo_gpu build failed:\n{res.stdout}\n{res.stderr}")
    return CLI_PATH


def build_oracle() -> Path:
    """Builds oracle/lib/libspeo_oracle.so (test infrastructure) with make."""
    res = subprocess.run(["make", "-s", "-C", str(REPO_ROOT / "oracle")], capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{res.stdout}\n{res.stderr}")
    return REPO_ROOT / "oracle" / "lib" / "libspeo_oracle.so"


# Where this build recipe looks for the reference project's sources (read in place, never
# copied): SPEO_REFERENCE_DIR, else the reference's mount point in the build container. The
# resolved directory is recorded in oracle/_ref/REFERENCE_ROOT for the tests that read it.
REFERENCE_MOUNT = "/root/reference/SPEO-GPU-single-control"


def build_reference_objective() -> Path | None:
    """Compiles the reference's own CEC2014.cc, immigrant buffers and kernels into oracle/_ref
    when its sources are present."""
    ref_root = Path(os.environ.get("SPEO_REFERENCE_DIR", REFERENCE_MOUNT))
    if not (ref_root / "CUDA_EA_library" / "CEC2014.cc").exists():
        return None
    res = subprocess.run(["make", "-s", "-C", str(REPO_ROOT / "oracle"), "ref", f"REF_ROOT={ref_root}"],
                         capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"reference objective build failed:\n{res.stdout}\n{res.stderr}")
    return REPO_ROOT / "oracle" / "_ref" / "libref_cec.so"


if __name__ == "__main__":
    print(build_library(verbose="-v" in sys.argv))
