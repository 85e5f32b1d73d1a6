"""Archipelago migration policies: the reference's src/migrate.cc (dynamicConnect destinations,
random emigrants, immigrant import into random rows, regroup options) and src/buffer_manage.cc
(OnlineCluster, BestSelect, RandomSelect, FIFO, LIFO) as device ops over many islands.

CPU tests check the oracle's restatement on hand-built cases; GPU tests run the library and the
oracle side by side and compare every state byte, row, fitness and permutation exactly."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest


def _desc(N=3, P=16, D=5, ld=8, k=2, C=3, policy=3, regroup=0, rate=1.0, seed=77):
    from speo_gb300 import _lib

    return _lib.Archipelago(N, P, D, ld, k, C, policy, regroup, rate, 0, seed)


def _pop(N, P, D, ld, seed=0):
    rng = np.random.default_rng(seed)
    pop = np.zeros((N * P, ld), dtype=np.float32)
    pop[:, :D] = rng.uniform(-100, 100, (N * P, D))
    fit = rng.uniform(0, 1000, N * P).astype(np.float32)
    return pop, fit


def _emigrants(oracle, desc, src, gen):
    key = np.array(oracle.philox([src, gen, 0, 8], oracle.key_of(desc.seed)), dtype=np.uint32)
    return [src * desc.island_size + oracle.fperm(desc.island_size, key, q) for q in range(desc.migration_size)]


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 7, 8, 100, 1000, 4096, 4097])
def test_feistel_permutation_is_a_bijection(oracle, n):
    key = [0x12345678, 0x9ABCDEF0, 0x0F1E2D3C, 0x4B5A6978]
    vals = [oracle.fperm(n, key, x) for x in range(n)]
    assert sorted(vals) == list(range(n))


def test_destinations_follow_the_migration_rate(oracle):
    """UpdateDestination (migrate.cc:34-44): rate 1 lists every other island in order, rate 0 none."""
    for rate, expect in ((1.0, lambda s, N: [t for t in range(N) if t != s]), (0.0, lambda s, N: [])):
        d = _desc(N=5, rate=rate)
        a = oracle.Archipelago(d, 1)
        pop, fit = _pop(5, d.island_size, d.dim, d.ld)
        a.migrate_out(pop, fit, 0)
        ints, _ = a.view()
        for s in range(5):
            assert ints[s, 0] == len(expect(s, 5)) and ints[s, 1] == 0
            assert list(ints[s, 4:4 + ints[s, 0]]) == expect(s, 5)


def test_fifo_buffer_receives_emigrants_in_order_and_drops_the_oldest(oracle):
    """Two islands sending to each other every generation (rate 1): FIFO buffer of capacity 3 gets
    2 emigrants per generation; past capacity the oldest goes (BufferManage::UpdateBuffer)."""
    d = _desc(N=2, P=16, k=2, C=3, policy=3)
    a = oracle.Archipelago(d, 1)
    pop, fit = _pop(2, 16, d.dim, d.ld, seed=3)
    a.migrate_out(pop, fit, 0)          # lists [1] and [0]; buffers empty
    a.migrate_in(pop, fit, 0)           # one message each way, heads advance
    ints, flts = a.view()
    rows0 = _emigrants(oracle, d, 0, 0)
    assert ints[1, 2] == 2
    W = d.dim + 1
    for pos, r in enumerate(rows0):
        slot = ints[1, 4 + 2 + 2 * 3 + pos]          # order[pos] of island 1
        e = flts[1, slot * W:(slot + 1) * W]
        assert np.array_equal(e[:d.dim], pop[r, :d.dim]) and e[d.dim] == fit[r]
    a.migrate_out(pop, fit, 1)          # lists used up -> refilled; FIFO selection of 2
    ints, _ = a.view()
    assert ints[1, 2] == 0 and ints[0, 2] == 0
    a.migrate_in(pop, fit, 1)
    a.migrate_in(pop, fit, 2)           # lists used up: nothing sent
    ints, flts = a.view()
    assert ints[1, 2] == 2
    a.migrate_out(pop, fit, 3)
    a.migrate_in(pop, fit, 3)           # 2 more: capacity 3 keeps the 3 newest
    ints, flts = a.view()
    assert ints[1, 2] == 2              # 2 selected at gen 3, then 2 received
    rows3 = _emigrants(oracle, d, 0, 3)
    slot = ints[1, 4 + 2 + 2 * 3 + 1]
    assert np.array_equal(flts[1, slot * W:slot * W + d.dim], pop[rows3[1], :d.dim])


def test_lifo_and_best_selection_order(oracle):
    """LIFO takes the newest entry first; BestSelect takes the largest fitness first
    (buffer_manage.cc:178-191 keeps the first maximum), as the reference does."""
    for policy in (1, 4):
        d = _desc(N=2, P=16, k=3, C=3, policy=policy)
        a = oracle.Archipelago(d, 1)
        pop, fit = _pop(2, 16, d.dim, d.ld, seed=5)
        a.migrate_out(pop, fit, 0)
        a.migrate_in(pop, fit, 0)
        rows = _emigrants(oracle, d, 0, 0)[:3]
        expect = list(reversed(rows)) if policy == 4 else sorted(rows, key=lambda r: -fit[r])
        p2, f2 = pop.copy(), fit.copy()
        a.migrate_out(p2, f2, 1)
        key = np.array(oracle.philox([1, 1, 0, 9], oracle.key_of(d.seed)), dtype=np.uint32)
        dest = [16 + oracle.fperm(16, key, q) for q in range(3)]
        for r_src, r_dst in zip(expect, dest):
            assert np.array_equal(p2[r_dst, :d.dim], pop[r_src, :d.dim]) and f2[r_dst] == fit[r_src]


def test_online_cluster_assigns_to_the_nearest_centre(oracle):
    """OnlineCluster: the first C immigrants found clusters; later ones join the nearest centre,
    whose centre becomes the running mean and whose entry is replaced (buffer_manage.cc:60-131)."""
    d = _desc(N=2, P=16, D=2, ld=4, k=3, C=2, policy=0)
    a = oracle.Archipelago(d, 1)
    pop, fit = _pop(2, 16, 2, 4, seed=9)
    a.migrate_out(pop, fit, 0)
    a.migrate_in(pop, fit, 0)
    rows = _emigrants(oracle, d, 0, 0)
    x0, x1, x2 = (pop[r, :2].astype(np.float64) for r in rows)
    near = 0 if np.linalg.norm(x2 - x0) <= np.linalg.norm(x2 - x1) else 1
    ints, flts = a.view()
    C, D = 2, 2
    centre = flts[1, C * (D + 1) + near * D: C * (D + 1) + (near + 1) * D]
    base = (x0, x1)[near]
    np.testing.assert_allclose(centre, (base + x2) / 2, rtol=1e-6)
    member = ints[1, 4 + 2: 4 + 2 + C]
    assert member[near] == 2 and member[1 - near] == 1
    entry = flts[1, near * (D + 1): near * (D + 1) + D]
    assert np.array_equal(entry, pop[rows[2], :2])


@pytest.mark.parametrize("regroup", [1, 2, 3])
def test_regroup_options(oracle, regroup):
    d = _desc(N=3, P=64, regroup=regroup, rate=0.0)
    a = oracle.Archipelago(d, 2)
    pop, fit = _pop(3, 64, d.dim, d.ld)
    for g in range(4):
        a.migrate_out(pop, fit, g)
        for s in range(3):
            perm = a.perm[s * 64:(s + 1) * 64]
            assert sorted(perm) == list(range(64))
            if regroup == 2:
                assert list(perm) == list(range(64))
            if regroup in (2, 3):
                assert a.subisland_num[s] in (16, 8, 4, 2, 1)
            else:
                assert a.subisland_num[s] == 2


# ---------------------------------------------------------------------------------------------
# the library against the oracle, bit for bit
# ---------------------------------------------------------------------------------------------
@pytest.mark.gpu
@pytest.mark.parametrize("policy", [0, 1, 2, 3, 4])
@pytest.mark.parametrize("regroup", [0, 3, 1, 2])
@pytest.mark.parametrize("N,P,D,k,C,rate,interval", [(6, 64, 30, 8, 16, 0.5, 3), (3, 100, 10, 32, 32, 1.0, 2),
                                                     (17, 40, 50, 5, 7, 0.3, 1),
                                                     (1, 16, 1, 16, 1, 1.0, 1),      # one island: nobody to send to
                                                     (2, 4, 3, 4, 4, 1.0, 1),        # the smallest islands, k = P
                                                     (4, 33, 100, 1, 32, 0.0, 1),    # rate 0: lists stay empty
                                                     (2, 128, 20, 64, 64, 1.0, 1)])  # capacity 64, the largest
def test_archipelago_matches_oracle(lib, oracle, cuda, policy, regroup, N, P, D, k, C, rate, interval):
    import torch
    from speo_gb300 import _lib

    ld = (D + 3) // 4 * 4
    d = _desc(N=N, P=P, D=D, ld=ld, k=k, C=C, policy=policy, regroup=regroup, rate=rate, seed=1000 + N)
    ref = oracle.Archipelago(d, 2)
    nbytes = lib.speo_archipelago_state_bytes(ctypes.addressof(d))
    assert nbytes == ref.state.size
    state = torch.full((nbytes // 4,), -7, dtype=torch.int32, device=cuda)
    perm = torch.zeros(N * P, dtype=torch.int32, device=cuda)
    nsub = torch.zeros(N, dtype=torch.int32, device=cuda)
    _lib.check(lib.speo_archipelago_init(ctypes.addressof(d), state.data_ptr(), perm.data_ptr(), nsub.data_ptr(), 2,
                                         None), "init")
    pop, fit = _pop(N, P, D, ld, seed=N * 13)
    tpop, tfit = torch.from_numpy(pop).to(cuda), torch.from_numpy(fit).to(cuda)
    rng = np.random.default_rng(4)

    def same(tag):
        torch.cuda.synchronize()
        assert np.array_equal(state.cpu().numpy().view(np.uint8), ref.state), tag
        assert np.array_equal(tpop.cpu().numpy(), pop), tag
        assert np.array_equal(tfit.cpu().numpy(), fit), tag
        assert np.array_equal(perm.cpu().numpy(), ref.perm), tag
        assert np.array_equal(nsub.cpu().numpy(), ref.subisland_num), tag

    same("init")
    for g in range(9):
        # stand-in for a generation: perturb some rows on both sides identically
        rows = rng.choice(N * P, size=N * P // 3, replace=False)
        pop[rows, :D] += rng.normal(0, 1, (len(rows), D)).astype(np.float32)
        fit[rows] = rng.uniform(0, 1000, len(rows)).astype(np.float32)
        tpop.copy_(torch.from_numpy(pop))
        tfit.copy_(torch.from_numpy(fit))
        if g % interval == 0:
            _lib.check(lib.speo_migrate_out(ctypes.addressof(d), state.data_ptr(), tpop.data_ptr(), tfit.data_ptr(),
                                            perm.data_ptr(), nsub.data_ptr(), g, None), "migrate_out")
            ref.migrate_out(pop, fit, g)
            same(f"out {g}")
        _lib.check(lib.speo_migrate_in(ctypes.addressof(d), state.data_ptr(), tpop.data_ptr(), tfit.data_ptr(), g,
                                       None), "migrate_in")
        ref.migrate_in(pop, fit, g)
        same(f"in {g}")
    _lib.check(lib.API_CheckCUDAError(), "archipelago")


def test_archipelago_rejects_bad_descriptions(lib):
    """Checked on the host before any device work."""
    from speo_gb300 import _lib

    state = ctypes.c_void_p(16)
    for bad in (dict(C=65), dict(C=0), dict(k=0), dict(P=3, C=2, k=2), dict(policy=5), dict(regroup=4),
                dict(rate=1.5), dict(N=0), dict(D=0)):
        args = dict(N=3, P=16, D=5, ld=8, k=2, C=3, policy=3, regroup=0, rate=1.0)
        args.update(bad)
        d = _desc(**args)
        assert lib.speo_migrate_in(ctypes.addressof(d), state, ctypes.c_void_p(16), ctypes.c_void_p(16), 0,
                                   None) == _lib.SPEO_ERR_INVALID_ARG
