"""Seeded synthetic objective instances and run seeds.

The reference evaluates CEC2014 instances read from its suite data files
(CUDA_EA_library/CEC2014_CUDA.cc:160-289). This library's workloads use seeded synthetic
instances of the same shape instead:
  o ~ U[-80, 80]^D,
  M = Q from the QR factorisation of a seeded N(0,1) D x D matrix, columns' signs fixed by
      sign(diag R) (a Haar-distributed orthogonal matrix).
Both are rounded to float32 and the rounded values *are* the instance: the FP64 oracle and
the FP64 re-evaluation use exactly these numbers, upcast.
"""
from __future__ import annotations

import numpy as np


def run_seed(node_id: int, function_id: int, run_id: int) -> int:
    """seed = (node_ID + function_ID) * (run_ID + function_ID), src/main.cc:138."""
    return (node_id + function_id) * (run_id + function_id)


def make_instance(seed: int, dim: int) -> tuple[np.ndarray, np.ndarray]:
    """(o, M) as float32; M is row-major, z = M (x - o)."""
    rng = np.random.default_rng(seed)
    o = rng.uniform(-80.0, 80.0, size=dim)
    a = rng.standard_normal((dim, dim))
    q, r = np.linalg.qr(a)
    q = q * np.sign(np.diag(r))[None, :]
    return o.astype(np.float32), q.astype(np.float32)


def rot_layout(M: np.ndarray, ld_rot: int | None = None) -> np.ndarray:
    """M^T padded to ld_rot columns: rot[k, j] = M[j, k] (the reference's B operand,
    CUDA_EA_library/CEC2014_CUDA.cc:246-270)."""
    D = M.shape[0]
    ld_rot = ld_rot or ((D + 3) // 4 * 4)
    out = np.zeros((D, ld_rot), dtype=M.dtype)
    out[:, :D] = M.T
    return out


def shift_layout(o: np.ndarray, length: int | None = None) -> np.ndarray:
    D = o.shape[0]
    length = length or ((D + 3) // 4 * 4)
    out = np.zeros(length, dtype=o.dtype)
    out[:D] = o
    return out


def write_reference_data(directory: str, func_id: int, o: np.ndarray, M: np.ndarray) -> None:
    """Writes (o, M) in the reference's text format: input_data/M_<f>_D<d>.txt (D x D, row i
    = row i of M) and input_data/shift_data_<f>.txt (first D values used), as read by
    CEC2014::Initilize (CUDA_EA_library/CEC2014.cc:354-400)."""
    import os

    D = o.shape[0]
    os.makedirs(os.path.join(directory, "input_data"), exist_ok=True)
    with open(os.path.join(directory, "input_data", f"M_{func_id}_D{D}.txt"), "w") as f:
        for i in range(D):
            f.write(" ".join(f"{float(v):.17g}" for v in M[i]) + "\n")
    with open(os.path.join(directory, "input_data", f"shift_data_{func_id}.txt"), "w") as f:
        f.write(" ".join(f"{float(v):.17g}" for v in o) + "\n")


def cec_components(function_id: int) -> int:
    """Components of a composition function (CUDA_EA_library/CEC2014.cc:306-333); 1 otherwise."""
    return {23: 5, 24: 3, 25: 3, 26: 5, 27: 5, 28: 5, 29: 3, 30: 3}.get(function_id, 1)


def uses_shuffle(function_id: int) -> bool:
    """Hybrid functions (17-22) and the compositions of hybrids (29, 30) read a shuffle."""
    return 17 <= function_id <= 22 or function_id in (29, 30)


def make_instance_multi(seed: int, dim: int, function_id: int) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """(o, M, S) for any id: o (nc, D) and M (nc, D, D) as float32, component c drawn like
    make_instance(seed + 1000003 c) (so component 0 is make_instance(seed)); S (nc, D) int32,
    each row a 1-based permutation of 1..D (the reference's shuffle_data convention)."""
    nc = cec_components(function_id)
    o = np.empty((nc, dim), dtype=np.float32)
    M = np.empty((nc, dim, dim), dtype=np.float32)
    for c in range(nc):
        o[c], M[c] = make_instance(seed + 1000003 * c, dim)
    rng = np.random.default_rng(seed + 7919)
    S = np.stack([rng.permutation(dim) + 1 for _ in range(nc)]).astype(np.int32)
    return o, M, S


def write_reference_data_multi(directory: str, func_id: int, o: np.ndarray, M: np.ndarray,
                               S: np.ndarray | None) -> None:
    """Writes (o, M, S) in the reference's text format for any id: M_<f>_D<d>.txt holds the nc
    D x D blocks one after another; shift_data_<f>.txt one line per component, padded to 100
    values (CEC2014.cc:385-418 reads D values and skips the rest of the line;
    CEC2014_CUDA.cc:198-224 reads 100 values per component); shuffle_data_<f>_D<d>.txt one line
    of D 1-based indices per component (CEC2014.cc:423-460)."""
    import os

    o = np.atleast_2d(o)
    nc, D = o.shape
    M = M.reshape(nc, D, D)
    d = os.path.join(directory, "input_data")
    os.makedirs(d, exist_ok=True)
    with open(os.path.join(d, f"M_{func_id}_D{D}.txt"), "w") as f:
        for c in range(nc):
            for i in range(D):
                f.write(" ".join(f"{float(v):.17g}" for v in M[c, i]) + "\n")
    with open(os.path.join(d, f"shift_data_{func_id}.txt"), "w") as f:
        for c in range(nc):
            row = list(o[c]) + [0.0] * max(0, 100 - D)
            f.write(" ".join(f"{float(v):.17g}" for v in row) + "\n")
    if S is not None:
        S = np.atleast_2d(S)
        with open(os.path.join(d, f"shuffle_data_{func_id}_D{D}.txt"), "w") as f:
            for c in range(S.shape[0]):
                f.write(" ".join(str(int(v)) for v in S[c]) + "\n")

