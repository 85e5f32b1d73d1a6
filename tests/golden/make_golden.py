"""Generates tests/golden/objective_f9.npz and tests/golden/objective_cec.npz from the
reference's own CPU objective.

Run where the reference sources exist (it builds oracle/_ref/libref_cec.so from the
reference's CUDA_EA_library/CEC2014.cc with `make -C oracle ref`):

    python tests/golden/make_golden.py

For each D the reference supports (CEC2014.cc:318-321) it makes a seeded synthetic instance
(o, M) in the reference's input_data text format, lets CEC2014::EvaluateFitness (function 9,
rotated Rastrigin, returns f - f*) evaluate a set of points, and stores inputs and outputs.
The tests check the oracle's restatement against these values on any machine.
objective_cec.npz holds the same for functions 1-16 at D = 10 and 30 (keys "<fid>_<D>_<o|M|X|f>"),
objective_multi.npz for the hybrid and composition functions 17-30 at D = 10 and 30 (keys
"<fid>_<D>_<o|M|S|X|f>", o / M / S with one row / block per component).
"""
from __future__ import annotations

import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
sys.path.insert(0, str(REPO / "speo-gpu-single-control_gb300"))
sys.path.insert(0, str(REPO / "oracle"))

from speo_gb300.instances import (make_instance, make_instance_multi, run_seed, uses_shuffle,  # noqa: E402
                                  write_reference_data, write_reference_data_multi)

DIMS = (10, 30, 50, 100)
N_POINTS = 24


def main() -> None:
    subprocess.run(["make", "-s", "-C", str(REPO / "oracle"), "ref"], check=True)
    import speo_oracle

    ref = speo_oracle.ref_lib()
    assert ref is not None, "oracle/_ref/libref_cec.so was not built"
    out = {}
    for D in DIMS:
        seed = run_seed(1, 9, D)
        o, M = make_instance(seed, D)
        rng = np.random.default_rng(seed + 7)
        X = np.empty((N_POINTS, D), dtype=np.float32)
        X[0] = o                                                   # f(o) = 0
        X[1] = np.clip(o + rng.normal(0, 1e-3, D), -100, 100)      # near the optimum
        X[2] = np.clip(o + rng.normal(0, 0.5, D), -100, 100)
        X[3:] = rng.uniform(-100, 100, (N_POINTS - 3, D))
        with tempfile.TemporaryDirectory() as tmp:
            write_reference_data(tmp, 9, o, M)
            assert ref.ref_cec_init(9, D, tmp.encode()) == 0
            Xd = np.ascontiguousarray(X, dtype=np.float64)
            f = np.zeros(N_POINTS, dtype=np.float64)
            ref.ref_cec_eval_batch(Xd.ctypes.data, N_POINTS, D, f.ctypes.data)
        out[f"o_{D}"] = o
        out[f"M_{D}"] = M
        out[f"X_{D}"] = X
        out[f"f_{D}"] = f
    np.savez_compressed(HERE / "objective_f9.npz", **out)
    print("wrote", HERE / "objective_f9.npz")

    cec = {}
    for fid in range(1, 17):
        for D in (10, 30):
            seed = run_seed(1, fid, D)
            o, M = make_instance(seed, D)
            rng = np.random.default_rng(seed + 11)
            n = 12
            X = np.empty((n, D), dtype=np.float32)
            X[0] = o
            X[1] = np.clip(o + rng.normal(0, 1e-2, D), -100, 100)
            X[2] = np.clip(o + rng.normal(0, 1.0, D), -100, 100)
            X[3:] = rng.uniform(-100, 100, (n - 3, D))
            with tempfile.TemporaryDirectory() as tmp:
                write_reference_data(tmp, fid, o, M)
                assert ref.ref_cec_init(fid, D, tmp.encode()) == 0
                Xd = np.ascontiguousarray(X, dtype=np.float64)
                f = np.zeros(n, dtype=np.float64)
                ref.ref_cec_eval_batch(Xd.ctypes.data, n, D, f.ctypes.data)
            cec.update({f"{fid}_{D}_o": o, f"{fid}_{D}_M": M, f"{fid}_{D}_X": X, f"{fid}_{D}_f": f})
    np.savez_compressed(HERE / "objective_cec.npz", **cec)
    print("wrote", HERE / "objective_cec.npz")

    multi = {}
    for fid in range(17, 31):
        for D in (10, 30):
            seed = run_seed(1, fid, D)
            o, M, S = make_instance_multi(seed, D, fid)
            rng = np.random.default_rng(seed + 13)
            n = 12
            X = np.empty((n, D), dtype=np.float32)
            X[0] = o[0]                                                  # optimum (component 0)
            X[1] = np.clip(o[0] + rng.normal(0, 1e-2, D), -100, 100)
            X[2] = np.clip(o[-1] + rng.normal(0, 1.0, D), -100, 100)    # near the last component
            X[3:] = rng.uniform(-100, 100, (n - 3, D))
            with tempfile.TemporaryDirectory() as tmp:
                write_reference_data_multi(tmp, fid, o, M, S if uses_shuffle(fid) else None)
                assert ref.ref_cec_init(fid, D, tmp.encode()) == 0
                Xd = np.ascontiguousarray(X, dtype=np.float64)
                f = np.zeros(n, dtype=np.float64)
                ref.ref_cec_eval_batch(Xd.ctypes.data, n, D, f.ctypes.data)
            multi.update({f"{fid}_{D}_o": o, f"{fid}_{D}_M": M, f"{fid}_{D}_S": S, f"{fid}_{D}_X": X,
                          f"{fid}_{D}_f": f})
    np.savez_compressed(HERE / "objective_multi.npz", **multi)
    print("wrote", HERE / "objective_multi.npz")


if __name__ == "__main__":
    main()
