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
