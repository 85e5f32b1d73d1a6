"""Python binding of the CPU oracle (oracle/lib/libspeo_oracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline leg as the checker; the product library never uses it.
"""
from __future__ import annotations

import ctypes
from ctypes import POINTER, c_double, c_float, c_int, c_int64, c_uint32, c_uint64, c_void_p
from pathlib import Path

import numpy as np

ORACLE_DIR = Path(__file__).resolve().parent
LIB = ORACLE_DIR / "lib" / "libspeo_oracle.so"
REF_LIB = ORACLE_DIR / "_ref" / "libref_cec.so"


class Draws(ctypes.Structure):
    _fields_ = [("kind", c_int), ("key", c_uint32 * 2), ("gen", c_uint32), ("tag_hi", c_uint32),
                ("pos0", c_int64), ("cap", c_void_p), ("cap_len", c_int), ("cap_pos", c_void_p)]


_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            import subprocess
            subprocess.run(["make", "-s", "-C", str(ORACLE_DIR)], check=True)
        L = ctypes.CDLL(str(LIB))
        L.speo_oracle_philox.argtypes = [c_void_p, c_void_p, c_void_p]
        L.speo_oracle_u01.argtypes = [c_uint32]
        L.speo_oracle_u01.restype = c_float
        L.speo_oracle_de_generate_f32.argtypes = [c_void_p, c_void_p, c_int, c_int, c_int, c_int, c_void_p, c_void_p,
                                                  c_void_p, c_void_p, c_void_p, c_float, c_float, POINTER(Draws)]
        L.speo_oracle_de_generate_f64.argtypes = [c_void_p, c_void_p, c_int, c_int, c_int, c_int, c_void_p, c_void_p,
                                                  c_void_p, c_void_p, c_void_p, c_double, c_double, POINTER(Draws)]
        L.speo_oracle_best_per_subisland_f32.argtypes = [c_void_p, c_int, c_int, c_void_p, c_void_p]
        L.speo_oracle_select_f32.argtypes = [c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_int, c_int, c_void_p]
        L.speo_oracle_select_f64.argtypes = [c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_int, c_int, c_void_p]
        L.speo_oracle_init_population_f32.argtypes = [c_void_p, c_int64, c_int, c_int, c_int, c_float, c_float,
                                                      c_void_p]
        L.speo_oracle_objective_f64.argtypes = [c_int, c_void_p, c_void_p, c_void_p, c_int]
        L.speo_oracle_objective_f64.restype = c_double
        L.speo_oracle_evaluate_rows.argtypes = [c_int, c_void_p, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p]
        L.speo_oracle_cec_components.argtypes = [c_int]
        L.speo_oracle_hybrid_groups.argtypes = [c_int, c_int, c_void_p, c_void_p]
        L.speo_oracle_objective_multi_f64.argtypes = [c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_int]
        L.speo_oracle_objective_multi_f64.restype = c_double
        L.speo_oracle_evaluate_rows_multi.argtypes = [c_int, c_void_p, c_int, c_int, c_int, c_void_p, c_void_p,
                                                      c_void_p, c_void_p]
        L.speo_oracle_arch_state_bytes.argtypes = [c_void_p]
        L.speo_oracle_arch_state_bytes.restype = ctypes.c_size_t
        L.speo_oracle_fperm.argtypes = [c_uint32, c_void_p, c_uint32]
        L.speo_oracle_fperm.restype = c_uint32
        L.speo_oracle_arch_init.argtypes = [c_void_p, c_void_p, c_void_p, c_void_p, c_int]
        L.speo_oracle_migrate_out.argtypes = [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_uint32]
        L.speo_oracle_migrate_in.argtypes = [c_void_p, c_void_p, c_void_p, c_void_p, c_uint32]
        L.speo_oracle_generation_f32.argtypes = [c_int] + [c_void_p] * 13 + [c_uint32] + [c_void_p] * 7
        L.speo_oracle_ring_migrate.argtypes = [c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_int,
                                               c_void_p, c_void_p]
        L.speo_oracle_run_islands_f64.argtypes = [c_int, c_int, c_int, c_int, c_int, c_double, c_double, c_double,
                                                  c_double, c_void_p, c_void_p, c_uint64, c_uint32, c_int, c_int,
                                                  c_int, c_void_p, c_void_p, c_int]
        L.speo_oracle_run_islands_f64.restype = c_int64
        L.speo_oracle_mlp_nparams.argtypes = [c_int, c_int]
        L.speo_oracle_mlp_forward.argtypes = [c_void_p, c_int, c_int, c_float, c_void_p, c_int, c_int, c_void_p]
        L.speo_oracle_mlp_loss_grad.argtypes = [c_void_p, c_int, c_int, c_float, c_void_p, c_int, c_int, c_void_p,
                                                c_void_p]
        L.speo_oracle_mlp_loss_grad.restype = c_double
        L.speo_oracle_adam.argtypes = [c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_float, c_float, c_float,
                                       c_float, c_int]
        _lib = L
    return _lib


def _p(a: np.ndarray | None):
    return None if a is None else a.ctypes.data


def philox(ctr, key) -> list[int]:
    c = np.asarray(ctr, dtype=np.uint32)
    k = np.asarray(key, dtype=np.uint32)
    out = np.zeros(4, dtype=np.uint32)
    lib().speo_oracle_philox(_p(c), _p(k), _p(out))
    return [int(v) for v in out]


def key_of(seed: int) -> tuple[int, int]:
    return seed & 0xFFFFFFFF, (seed >> 32) & 0xFFFFFFFF


def philox_draws(seed: int, gen: int, pos0: int = 0, tag_hi: int = 0) -> Draws:
    d = Draws()
    d.kind = 0
    d.key[0], d.key[1] = key_of(seed)
    d.gen = gen
    d.tag_hi = tag_hi
    d.pos0 = pos0
    return d


def captured_draws(cap: np.ndarray, cap_pos: np.ndarray) -> Draws:
    """Reference-layout stream: cap[(p*32+l), i] = i-th uniform of state p*32+l."""
    d = Draws()
    d.kind = 1
    d.cap = cap.ctypes.data
    d.cap_len = cap.shape[1]
    d.cap_pos = cap_pos.ctypes.data
    d._keep = (cap, cap_pos)
    return d


def de_generate(cand, pop, ld, dim, perm, CR, F, strategy, best_id, lb, ub, draws, f64=False) -> int:
    T = np.float64 if f64 else np.float32
    CR = np.ascontiguousarray(CR, dtype=T)
    F = np.ascontiguousarray(F, dtype=T)
    strategy = np.ascontiguousarray(strategy, dtype=np.int32)
    perm = np.ascontiguousarray(perm, dtype=np.int32)
    best = None if best_id is None else np.ascontiguousarray(best_id, dtype=np.int32)
    fn = lib().speo_oracle_de_generate_f64 if f64 else lib().speo_oracle_de_generate_f32
    return fn(_p(cand), _p(pop), ld, dim, len(perm), len(CR), _p(perm), _p(CR), _p(F), _p(strategy), _p(best),
              lb, ub, ctypes.byref(draws))


def best_per_subisland(fit, n_sub, perm) -> np.ndarray:
    out = np.zeros(n_sub, dtype=np.int32)
    perm = np.ascontiguousarray(perm, dtype=np.int32)
    lib().speo_oracle_best_per_subisland_f32(_p(fit), len(perm), n_sub, _p(perm), _p(out))
    return out


def select(pop, pop_fit, cand, cand_fit, ld, dim, f64=False) -> np.ndarray:
    sel = np.zeros(len(pop_fit), dtype=np.uint8)
    fn = lib().speo_oracle_select_f64 if f64 else lib().speo_oracle_select_f32
    fn(_p(pop), _p(pop_fit), _p(cand), _p(cand_fit), len(pop_fit), ld, dim, _p(sel))
    return sel


def init_population(n, ld, dim, lb, ub, seed, row0=0) -> np.ndarray:
    pop = np.zeros((n, ld), dtype=np.float32)
    key = np.asarray(key_of(seed), dtype=np.uint32)
    lib().speo_oracle_init_population_f32(_p(pop), row0, n, ld, dim, lb, ub, _p(key))
    return pop


def objective(func_id, x, o, M) -> float:
    x = np.ascontiguousarray(x, dtype=np.float64)
    o = np.ascontiguousarray(o, dtype=np.float64)
    M = np.ascontiguousarray(M, dtype=np.float64)
    return lib().speo_oracle_objective_f64(func_id, _p(x), _p(o), _p(M), len(o))


def evaluate_rows(func_id, X, dim, o, M) -> np.ndarray:
    X = np.ascontiguousarray(X, dtype=np.float32)
    out = np.zeros(X.shape[0], dtype=np.float64)
    lib().speo_oracle_evaluate_rows(func_id, _p(X), X.shape[0], X.shape[1], dim,
                                    _p(np.ascontiguousarray(o, dtype=np.float32)),
                                    _p(np.ascontiguousarray(M, dtype=np.float32)), _p(out))
    return out


def cec_components(func_id) -> int:
    return lib().speo_oracle_cec_components(func_id)


def hybrid_groups(func_id, dim) -> list[tuple[int, int]]:
    """[(start, length)] of the groups of hybrid func_id (17-22) at dimension dim."""
    G = (ctypes.c_int * 5)()
    n = (ctypes.c_int * 5)()
    k = lib().speo_oracle_hybrid_groups(func_id, dim, G, n)
    return [(G[i], n[i]) for i in range(k)]


def objective_multi(func_id, x, o, M, S=None) -> float:
    """Any id 1-31; o (nc, D), M (nc, D, D), S (nc, D) 1-based (hybrids and 29/30)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    o = np.ascontiguousarray(o, dtype=np.float64)
    M = np.ascontiguousarray(M, dtype=np.float64)
    S = None if S is None else np.ascontiguousarray(S, dtype=np.int32)
    return lib().speo_oracle_objective_multi_f64(func_id, _p(x), _p(o), _p(M), _p(S), x.shape[-1])


def evaluate_rows_multi(func_id, X, dim, o, M, S=None) -> np.ndarray:
    X = np.ascontiguousarray(X, dtype=np.float32)
    S = None if S is None else np.ascontiguousarray(S, dtype=np.int32)
    out = np.zeros(X.shape[0], dtype=np.float64)
    lib().speo_oracle_evaluate_rows_multi(func_id, _p(X), X.shape[0], X.shape[1], dim,
                                          _p(np.ascontiguousarray(o, dtype=np.float32)),
                                          _p(np.ascontiguousarray(M, dtype=np.float32)), _p(S), _p(out))
    return out


class Archipelago:
    """Host restatement of the archipelago migration ops on numpy arrays (same state layout as the
    library). `desc` is a ctypes speo_archipelago (speo_gb300._lib.Archipelago)."""

    def __init__(self, desc, subisland_num: int):
        self.desc = desc
        n = lib().speo_oracle_arch_state_bytes(ctypes.addressof(desc))
        self.state = np.zeros(n, dtype=np.uint8)
        self.perm = np.zeros(desc.n_islands * desc.island_size, dtype=np.int32)
        self.subisland_num = np.zeros(desc.n_islands, dtype=np.int32)
        lib().speo_oracle_arch_init(ctypes.addressof(desc), _p(self.state), _p(self.perm), _p(self.subisland_num),
                                    subisland_num)

    def migrate_out(self, pop, fit, gen):
        lib().speo_oracle_migrate_out(ctypes.addressof(self.desc), _p(self.state), _p(pop), _p(fit), _p(self.perm),
                                      _p(self.subisland_num), gen)

    def migrate_in(self, pop, fit, gen):
        lib().speo_oracle_migrate_in(ctypes.addressof(self.desc), _p(self.state), _p(pop), _p(fit), gen)

    def view(self):
        """(ints, floats) per island: ints (N, istride), floats (N, fstride)."""
        d = self.desc
        istride = (4 + d.n_islands + 3 * d.buffer_capacity + 3) // 4 * 4
        ints = self.state[: 4 * d.n_islands * istride].view(np.int32).reshape(d.n_islands, istride)
        flts = self.state[4 * d.n_islands * istride:].view(np.float32).reshape(d.n_islands, -1)
        return ints, flts


def fperm(n: int, key, x: int) -> int:
    k = np.asarray(key, dtype=np.uint32)
    return lib().speo_oracle_fperm(n, _p(k), x)


def generation(segs: list[dict], gen: int, pop_in, fit_in, trial_fit=None):
    """segs: dicts with row0, P, D, ld, func, strategy, F, CR, lb, ub, o, M, seed.
    Returns (pop_out, fit_out, trials, sel, err)."""
    n = len(segs)
    row0 = np.array([s["row0"] for s in segs], dtype=np.int64)
    P = np.array([s["P"] for s in segs], dtype=np.int32)
    D = np.array([s["D"] for s in segs], dtype=np.int32)
    ld = np.array([s["ld"] for s in segs], dtype=np.int32)
    func = np.array([s["func"] for s in segs], dtype=np.int32)
    st = np.array([s.get("strategy", 4) for s in segs], dtype=np.int32)
    F = np.array([s["F"] for s in segs], dtype=np.float32)
    CR = np.array([s["CR"] for s in segs], dtype=np.float32)
    lb = np.array([s["lb"] for s in segs], dtype=np.float32)
    ub = np.array([s["ub"] for s in segs], dtype=np.float32)
    seed = np.array([s["seed"] for s in segs], dtype=np.uint64)
    os_ = [np.ascontiguousarray(s["o"], dtype=np.float32) for s in segs]
    Ms = [np.ascontiguousarray(s["M"], dtype=np.float32) for s in segs]
    op = (c_void_p * n)(*[a.ctypes.data for a in os_])
    mp = (c_void_p * n)(*[a.ctypes.data for a in Ms])
    pop_out = np.array(pop_in, copy=True)
    fit_out = np.array(fit_in, copy=True)
    trials = np.zeros_like(pop_in)
    sel = np.zeros(len(fit_in), dtype=np.uint8)
    tf = None if trial_fit is None else np.ascontiguousarray(trial_fit, dtype=np.float32)
    err = lib().speo_oracle_generation_f32(n, _p(row0), _p(P), _p(D), _p(ld), _p(func), _p(st), _p(F), _p(CR),
                                           _p(lb), _p(ub), ctypes.cast(op, c_void_p), ctypes.cast(mp, c_void_p),
                                           _p(seed), gen, _p(pop_in), _p(fit_in), _p(pop_out), _p(fit_out),
                                           _p(trials), _p(tf), _p(sel))
    return pop_out, fit_out, trials, sel, err


def ring_migrate(segs: list[dict], k: int, pop: np.ndarray, fit: np.ndarray) -> None:
    n = len(segs)
    row0 = np.array([s["row0"] for s in segs], dtype=np.int64)
    P = np.array([s["P"] for s in segs], dtype=np.int32)
    D = np.array([s["D"] for s in segs], dtype=np.int32)
    ld = np.array([s["ld"] for s in segs], dtype=np.int32)
    nxt = np.array([s["ring_next"] for s in segs], dtype=np.int32)
    lib().speo_oracle_ring_migrate(n, _p(row0), _p(P), _p(D), _p(ld), _p(nxt), k, _p(pop), _p(fit))


def run_islands_f64(n_islands, P, D, ld, func_id, F, CR, lb, ub, o, M, seed, gen0, gens, interval, k, pop, fit,
                    threads) -> int:
    o = np.ascontiguousarray(o, dtype=np.float64)
    M = np.ascontiguousarray(M, dtype=np.float64)
    return lib().speo_oracle_run_islands_f64(n_islands, P, D, ld, func_id, F, CR, lb, ub, _p(o), _p(M), seed, gen0,
                                             gens, interval, k, _p(pop), _p(fit), threads)


# ---- the reference's own CPU objective (oracle/_ref, built where the reference sources are) --
_ref = None


def ref_lib():
    global _ref
    if _ref is None:
        if not REF_LIB.exists():
            return None
        L = ctypes.CDLL(str(REF_LIB))
        L.ref_cec_init.argtypes = [c_int, c_int, ctypes.c_char_p]
        L.ref_cec_init.restype = c_int
        L.ref_cec_eval.argtypes = [c_void_p]
        L.ref_cec_eval.restype = c_double
        L.ref_cec_eval_batch.argtypes = [c_void_p, c_int, c_int, c_void_p]
        _ref = L
    return _ref


# ---- surrogate MLP ------------------------------------------------------------------------------
def mlp_nparams(din, h):
    return lib().speo_oracle_mlp_nparams(din, h)


def mlp_forward(theta, din, h, in_scale, X):
    theta = np.ascontiguousarray(theta, dtype=np.float32)
    X = np.ascontiguousarray(X, dtype=np.float32)
    y = np.zeros(X.shape[0], dtype=np.float64)
    lib().speo_oracle_mlp_forward(_p(theta), din, h, in_scale, _p(X), X.shape[0], X.shape[1], _p(y))
    return y


def mlp_loss_grad(theta, din, h, in_scale, X, t):
    theta = np.ascontiguousarray(theta, dtype=np.float32)
    X = np.ascontiguousarray(X, dtype=np.float32)
    t = np.ascontiguousarray(t, dtype=np.float32)
    g = np.zeros(mlp_nparams(din, h), dtype=np.float64)
    loss = lib().speo_oracle_mlp_loss_grad(_p(theta), din, h, in_scale, _p(X), X.shape[0], X.shape[1], _p(t), _p(g))
    return loss, g


def adam(theta, m, v, g, lr, beta1, beta2, eps, step):
    g = np.ascontiguousarray(g, dtype=np.float32)
    lib().speo_oracle_adam(_p(theta), _p(m), _p(v), _p(g), len(theta), lr, beta1, beta2, eps, step)
