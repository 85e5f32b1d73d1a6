"""CPU tests of the oracle: pinned against published Philox vectors and the reference's own
CPU objective (golden vectors made from CUDA_EA_library/CEC2014.cc), plus the algorithmic
properties of the DE restatement that the reference's kernel implies."""
from __future__ import annotations

import os
import sys
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden" / "objective_f9.npz"
sys.path.insert(0, str(Path(__file__).resolve().parent))
from ref_kernels import reference_root  # noqa: E402

_REF_ROOT = reference_root()
REF_DATA = (_REF_ROOT / "bin" / "input_data") if _REF_ROOT else Path("/nonexistent")


# Random123 v1.09 kat_vectors, philox4x32_10
@pytest.mark.parametrize("ctr,key,expect", [
    ([0, 0, 0, 0], [0, 0], [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]),
    ([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2, [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]),
    ([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0],
     [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]),
])
def test_philox_known_answers(oracle, ctr, key, expect):
    assert oracle.philox(ctr, key) == expect


def test_u01_range(oracle):
    L = oracle.lib()
    assert L.speo_oracle_u01(0) == pytest.approx(2.0 ** -24)
    assert L.speo_oracle_u01(0xFFFFFFFF) == 1.0
    assert L.speo_oracle_u01(0x80000000) == 0.5 + 2.0 ** -24


def _bias_ulps(fid):
    # CEC2014::EvaluateFitness adds f* = 100*fid and subtracts it again (CEC2014.cc:57-62,144)
    return 4 * np.spacing(100.0 * fid)


@pytest.mark.parametrize("D", [10, 30, 50, 100])
def test_objective_matches_reference_golden(oracle, D):
    g = np.load(GOLDEN)
    o, M, X, f_ref = g[f"o_{D}"], g[f"M_{D}"], g[f"X_{D}"], g[f"f_{D}"]
    mine = oracle.evaluate_rows(9, X, D, o, M)
    assert f_ref[0] == 0.0 and mine[0] == 0.0        # f(o) - f* = 0
    np.testing.assert_allclose(mine, f_ref, rtol=0, atol=_bias_ulps(9))


GOLDEN_CEC = Path(__file__).resolve().parent / "golden" / "objective_cec.npz"


@pytest.mark.parametrize("fid", range(1, 17))
@pytest.mark.parametrize("D", [10, 30])
def test_cec_objectives_match_reference_golden(oracle, fid, D):
    """CEC2014 functions 1-16: the oracle against the reference's own CEC2014::EvaluateFitness
    (golden vectors from tests/golden/make_golden.py), at the optimum, near it and at random points."""
    g = np.load(GOLDEN_CEC)
    o, M, X, f_ref = (g[f"{fid}_{D}_{k}"] for k in "oMXf")
    mine = np.array([oracle.objective(fid, x, o, M) for x in X])
    # the reference adds and subtracts f* = 100 fid (CEC2014.cc:144): its values carry that rounding
    np.testing.assert_allclose(mine, f_ref, rtol=1e-12, atol=_bias_ulps(fid))


GOLDEN_MULTI = Path(__file__).resolve().parent / "golden" / "objective_multi.npz"


@pytest.mark.parametrize("fid", range(17, 31))
@pytest.mark.parametrize("D", [10, 30])
def test_hybrid_composition_match_reference_golden(oracle, fid, D):
    """CEC2014 hybrid (17-22) and composition (23-30) functions: the oracle against the reference's
    CEC2014::EvaluateFitness on multi-component instances (one shift / matrix / shuffle per component)."""
    g = np.load(GOLDEN_MULTI)
    o, M, S, X, f_ref = (g[f"{fid}_{D}_{k}"] for k in "oMSXf")
    assert o.shape[0] == oracle.cec_components(fid)
    mine = np.array([oracle.objective_multi(fid, x, o, M, S) for x in X])
    np.testing.assert_allclose(mine, f_ref, rtol=1e-12, atol=_bias_ulps(fid))


def test_hybrid_groups_follow_reference_split(oracle):
    """G_nx[g] = ceil(gp_g * D) in double for all but the last group (CEC2014.cc:961-972)."""
    assert oracle.hybrid_groups(17, 10) == [(0, 3), (3, 3), (6, 4)]
    assert oracle.hybrid_groups(21, 10) == [(0, 1), (1, 2), (3, 2), (5, 2), (7, 3)]
    assert oracle.hybrid_groups(22, 100) == [(0, 10), (10, 20), (30, 20), (50, 20), (70, 30)]
    assert oracle.hybrid_groups(19, 30) == [(0, 6), (6, 6), (12, 9), (21, 9)]


def _suite_instance(fid, D):
    """The reference suite's own (o, M, S) for fid at D, read as CEC2014::Initilize reads them
    (CEC2014.cc:354-460): M = the first nc*D*D values, o = the first D values of each of the first
    nc lines, S = the first nc*D integers."""
    nc = {23: 5, 24: 3, 25: 3, 26: 5, 27: 5, 28: 5, 29: 3, 30: 3}.get(fid, 1)
    M = np.array(open(REF_DATA / f"M_{fid}_D{D}.txt").read().split(), dtype=np.float64)[: nc * D * D]
    lines = open(REF_DATA / f"shift_data_{fid}.txt").read().splitlines()
    if nc == 1:
        o = np.array(" ".join(lines).split(), dtype=np.float64)[:D][None]
    else:
        o = np.stack([np.array(lines[c].split(), dtype=np.float64)[:D] for c in range(nc)])
    S = None
    shuf = REF_DATA / f"shuffle_data_{fid}_D{D}.txt"
    if 17 <= fid <= 22 or fid in (29, 30):
        S = np.array(open(shuf).read().split(), dtype=np.int32)[: nc * D].reshape(nc, D)
    return o, M.reshape(nc, D, D), S


@pytest.mark.skipif(not REF_DATA.exists(), reason="reference suite data not present")
@pytest.mark.parametrize("fid", range(1, 31))
@pytest.mark.parametrize("D", [10, 20, 30, 50, 100])
def test_every_function_on_suite_data(oracle, fid, D):
    """The reference's own instances of every CEC2014 function (read in place), evaluated by the
    reference's CEC2014.cc and by the oracle."""
    ref = oracle.ref_lib()
    if ref is None:
        pytest.skip("oracle/_ref not built")
    o, M, S = _suite_instance(fid, D)
    assert ref.ref_cec_init(fid, D, str(REF_DATA.parent).encode()) == 0
    rng = np.random.default_rng(fid * 100 + D)
    X = np.concatenate([o[:1], o[-1:] + rng.normal(0, 0.5, (1, D)), rng.uniform(-100, 100, (6, D))])
    f_ref = np.zeros(len(X))
    ref.ref_cec_eval_batch(np.ascontiguousarray(X).ctypes.data, len(X), D, f_ref.ctypes.data)
    mine = np.array([oracle.objective_multi(fid, x, o, M, S) for x in X])
    np.testing.assert_allclose(mine, f_ref, rtol=1e-12, atol=_bias_ulps(fid))


@pytest.mark.skipif(not REF_DATA.exists(), reason="reference suite data not present")
@pytest.mark.parametrize("D", [10, 30, 100])
def test_objective_matches_reference_on_suite_data(oracle, D):
    """The reference's own F9 instance (read in place), evaluated by the reference's CEC2014.cc
    and by the oracle."""
    ref = oracle.ref_lib()
    if ref is None:
        pytest.skip("oracle/_ref not built")
    M = np.loadtxt(REF_DATA / f"M_9_D{D}.txt").reshape(-1)[: D * D].reshape(D, D)
    o = np.array(open(REF_DATA / "shift_data_9.txt").read().split(), dtype=np.float64)[:D]
    assert ref.ref_cec_init(9, D, str(REF_DATA.parent).encode()) == 0
    rng = np.random.default_rng(D)
    for x in [o.copy(), rng.uniform(-100, 100, D), o + rng.normal(0, 1, D)]:
        x = np.ascontiguousarray(x)
        f_ref = ref.ref_cec_eval(x.ctypes.data)
        assert oracle.objective(9, x, o, M) == pytest.approx(f_ref, rel=0, abs=_bias_ulps(9))


def test_sphere_is_rotation_invariant_norm(oracle):
    from speo_gb300.instances import make_instance

    o, M = make_instance(11, 30)
    x = np.random.default_rng(0).uniform(-100, 100, 30).astype(np.float32)
    f = oracle.objective(31, x, o, M)
    Md = M.astype(np.float64)
    y = x.astype(np.float64) - o.astype(np.float64)
    assert f == pytest.approx(float((Md @ y) @ (Md @ y)), rel=1e-14)
    assert oracle.objective(31, o, o, M) == 0.0


def _random_pop(rng, n, ld, dim):
    pop = np.zeros((n, ld), dtype=np.float32)
    pop[:, :dim] = rng.uniform(-100, 100, (n, dim)).astype(np.float32)
    return pop


@pytest.mark.parametrize("strategy", range(9))
def test_de_generate_structure(oracle, strategy):
    """Trial rows differ from the target only where the reference's crossover takes the mutant,
    stay inside the bounds, and untouched padding stays zero."""
    rng = np.random.default_rng(strategy)
    n, dim, ld, S = 64, 30, 32, 16
    pop = _random_pop(rng, n, ld, dim)
    perm = rng.permutation(n).astype(np.int32)
    cand = np.zeros_like(pop)
    fit = rng.uniform(0, 1, n).astype(np.float32)
    best = oracle.best_per_subisland(fit, n // S, perm)
    err = oracle.de_generate(cand, pop, ld, dim, perm, [0.9] * (n // S), [0.5] * (n // S), [strategy] * (n // S),
                             best, -100.0, 100.0, oracle.philox_draws(1234, 0))
    assert err == 0
    assert np.all(cand[:, dim:] == 0)
    assert np.all(np.abs(cand[:, :dim]) <= 100)
    changed = (cand[:, :dim] != pop[:, :dim]).mean()
    assert 0.5 < changed <= 1.0      # CR = 0.9


def test_de_generate_cr_zero_changes_one_element(oracle):
    rng = np.random.default_rng(5)
    n, dim, ld = 32, 10, 32
    pop = _random_pop(rng, n, ld, dim)
    cand = np.zeros_like(pop)
    perm = np.arange(n, dtype=np.int32)
    oracle.de_generate(cand, pop, ld, dim, perm, [0.0], [0.5], [4], None, -100.0, 100.0,
                       oracle.philox_draws(9, 3))
    diff = (cand[:, :dim] != pop[:, :dim]).sum(axis=1)
    assert np.all(diff <= 1)           # only jrand (unless jrand == dim, u = 1 exactly)
    assert diff.sum() >= n - 1


def test_de_generate_philox_stream_layout(oracle):
    """Index draws of position p come from philox({k/4, p, gen, TAG_IDX}) in order."""
    seed, gen, p, S = 77, 5, 3, 100
    words = []
    for blk in range(2):
        words += oracle.philox([blk, p, gen, 1], oracle.key_of(seed))
    us = [oracle.lib().speo_oracle_u01(w) for w in words]
    r0 = int(np.float32(us[0]) * np.float32(S))
    # reproduce the first donor through the restatement with a population tagged by row index
    n, dim, ld = S, 4, 32
    pop = np.zeros((n, ld), dtype=np.float32)
    pop[:, 0] = np.arange(n, dtype=np.float32) / 1000.0   # distinct rows, inside bounds
    cand = np.zeros_like(pop)
    oracle.de_generate(cand, pop, ld, dim, np.arange(n, dtype=np.int32), [1.0], [0.0], [4], None, -100.0, 100.0,
                       oracle.philox_draws(seed, gen))
    # with F = 0 and CR = 1 the trial is exactly x_r0
    assert cand[p, 0] == pop[min(r0, S - 1), 0]


def test_captured_stream_consumption(oracle):
    """Reference layout: lane 0 serves the index draws, each lane then one crossover draw per
    32-element chunk (kernel_DE_CUDA.cu:184-237)."""
    n, dim, ld = 8, 40, 64
    rng = np.random.default_rng(1)
    pop = _random_pop(rng, n, ld, dim)
    cand = np.zeros_like(pop)
    cap = rng.uniform(0, 1, (n * 32, 64)).astype(np.float32).astype(np.float64)
    pos = np.zeros(n * 32, dtype=np.int32)
    oracle.de_generate(cand, pop, ld, dim, np.arange(n, dtype=np.int32), [0.9], [0.5], [4], None, -100.0, 100.0,
                       oracle.captured_draws(cap, pos))
    lane_counts = pos.reshape(n, 32)
    assert np.all(lane_counts[:, 1:] == 2)          # np2 = 64 -> two chunks per lane
    assert np.all(lane_counts[:, 0] >= 2 + 6)       # >= 5 donors + jrand + 2 chunks


def test_select_strict_less(oracle):
    pop = np.ones((4, 4), dtype=np.float32)
    cand = np.full((4, 4), 2.0, dtype=np.float32)
    pf = np.array([1.0, 1.0, np.nan, 1.0], dtype=np.float32)
    cf = np.array([0.5, 1.0, 0.0, np.nan], dtype=np.float32)
    sel = oracle.select(pop, pf, cand, cf, 4, 4)
    assert sel.tolist() == [1, 0, 0, 0]          # ties and NaN keep the parent
    assert pop[0, 0] == 2.0 and pop[1, 0] == 1.0


def test_ring_migrate_semantics(oracle):
    rng = np.random.default_rng(3)
    nseg, P, D, ld, k = 4, 20, 6, 8, 3
    pop = np.zeros((nseg * P, ld), dtype=np.float32)
    pop[:, :D] = rng.uniform(-1, 1, (nseg * P, D))
    fit = rng.uniform(0, 10, nseg * P).astype(np.float32)
    fit[5] = fit[6]                                   # a tie
    segs = [dict(row0=s * P, P=P, D=D, ld=ld, ring_next=(s + 1) % nseg) for s in range(nseg)]
    pop0, fit0 = pop.copy(), fit.copy()
    oracle.ring_migrate(segs, k, pop, fit)
    for s in range(nseg):
        src = (s - 1) % nseg
        sf = fit0[src * P:(src + 1) * P]
        best = sorted(range(P), key=lambda i: (sf[i], i))[:k]
        df = fit0[s * P:(s + 1) * P]
        worst = sorted(range(P), key=lambda i: (-df[i], -i))[:k]
        for b, w in zip(best, worst):
            assert fit[s * P + w] == sf[b]
            assert np.array_equal(pop[s * P + w, :D], pop0[src * P + b, :D])
        untouched = [i for i in range(P) if i not in worst]
        assert np.array_equal(fit[s * P + np.array(untouched)], df[untouched])


def test_cpu_baseline_loop_improves(oracle):
    from speo_gb300.instances import make_instance

    D, P, n = 10, 32, 4
    o, M = make_instance(5, D)
    ld = 32
    pop32 = oracle.init_population(n * P, ld, D, -100.0, 100.0, 5)
    pop = pop32.astype(np.float64)
    fit = np.array([oracle.objective(31, pop[i, :D], o, M) for i in range(n * P)])
    f0 = fit.min()
    evals = oracle.run_islands_f64(n, P, D, ld, 31, 0.5, 0.9, -100.0, 100.0, o, M, 5, 0, 60, 20, 2, pop, fit,
                                   threads=2)
    assert evals == 60 * n * P
    assert fit.min() < f0 * 1e-2


def test_mlp_gradient_matches_finite_differences(oracle):
    """The oracle's analytic MLP gradient against central differences (FP64)."""
    din, h, scale = 5, 7, 0.01
    rng = np.random.default_rng(0)
    theta = rng.normal(0, 0.5, oracle.mlp_nparams(din, h)).astype(np.float32)
    X = rng.uniform(-100, 100, (9, din)).astype(np.float32)
    t = rng.normal(0, 1, 9).astype(np.float32)
    loss, g = oracle.mlp_loss_grad(theta, din, h, scale, X, t)
    eps = 1e-3
    for i in rng.choice(len(theta), 25, replace=False):
        tp, tm = theta.copy(), theta.copy()
        tp[i] += eps
        tm[i] -= eps
        lp = np.mean((oracle.mlp_forward(tp, din, h, scale, X) - t) ** 2)
        lm = np.mean((oracle.mlp_forward(tm, din, h, scale, X) - t) ** 2)
        fd = (lp - lm) / (float(tp[i]) - float(tm[i]))
        assert fd == pytest.approx(g[i], rel=2e-3, abs=1e-5)
