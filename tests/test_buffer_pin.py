"""The oracle's immigrant-buffer policies pinned to the reference's own classes.

oracle/_ref/libref_buffer.so is the reference's src/buffer_manage.cc (+ src/random.cc),
compiled in place with `real = float` behind a small C wrapper (oracle/ref_buffer_wrap.cc).
The oracle's archipelago (speo_oracle_migrate_out / _in) runs several islands for many
generations; every message it delivers to an island is also fed, in the same order, to that
island's reference buffer object (UpdateBuffer, as src/migrate.cc:71-103 calls it), and every
selection it makes is replayed with SelectFromBuffer (src/migrate.cc:46-62). The buffers must
hold the same individuals in the same order, with the same cluster centres, member counts and
update flags (OnlineCluster), and selections must return the same individuals in the same order.

Replayable: UpdateBuffer of all five policies (deterministic); SelectFromBuffer of OnlineCluster,
BestSelect and FIFO. RandomSelect's selection draws from the host rand() (the library draws from
Philox instead) and LIFO's erases end() (undefined behaviour, buffer_manage.cc:309), so their
selections are not replayed: after each of them the reference object is given the oracle's
remaining buffer, and UpdateBuffer is compared from there. The oracle's LIFO takes the newest
entry.
"""
from __future__ import annotations

import ctypes
import sys
from pathlib import Path

import numpy as np
import pytest

sys.path.insert(0, str(Path(__file__).resolve().parent))
from ref_kernels import REF_DIR  # noqa: E402

REF_BUF = REF_DIR / "libref_buffer.so"
pytestmark = pytest.mark.skipif(not REF_BUF.exists(), reason="reference buffer library not built (needs its sources)")


def _ref():
    L = ctypes.CDLL(str(REF_BUF))
    vp, i, fp, ip = ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p
    L.ref_buf_create.argtypes, L.ref_buf_create.restype = [i, i], vp
    L.ref_buf_destroy.argtypes = [vp]
    L.ref_buf_update.argtypes, L.ref_buf_update.restype = [vp, i, i, fp, fp], i
    L.ref_buf_select.argtypes, L.ref_buf_select.restype = [vp, i, i, fp, fp], i
    L.ref_buf_size.argtypes, L.ref_buf_size.restype = [vp], i
    L.ref_buf_assign.argtypes, L.ref_buf_assign.restype = [vp, i, i, fp, fp], i
    L.ref_buf_entries.argtypes = [vp, i, fp, fp]
    L.ref_buf_clusters.argtypes, L.ref_buf_clusters.restype = [vp, i, fp, ip, ip], i
    return L


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class RefIsland:
    def __init__(self, L, policy, cap, dim):
        self.L, self.policy, self.cap, self.dim = L, policy, cap, dim
        self.h = L.ref_buf_create(policy, cap)
        assert self.h

    def update(self, X, f):
        X = np.ascontiguousarray(X, dtype=np.float32)
        f = np.ascontiguousarray(f, dtype=np.float32)
        assert self.L.ref_buf_update(self.h, len(f), self.dim, _p(X), _p(f)) == 0

    def select(self, k):
        n = self.L.ref_buf_size(self.h)
        X = np.zeros((max(n, 1), self.dim), dtype=np.float32)
        f = np.zeros(max(n, 1), dtype=np.float32)
        got = self.L.ref_buf_select(self.h, k, self.dim, _p(X), _p(f))
        return X[:got], f[:got]

    def assign(self, X, f):
        X = np.ascontiguousarray(X, dtype=np.float32)
        f = np.ascontiguousarray(f, dtype=np.float32)
        assert self.L.ref_buf_assign(self.h, len(f), self.dim, _p(X), _p(f)) == 0

    def entries(self):
        n = self.L.ref_buf_size(self.h)
        X = np.zeros((max(n, 1), self.dim), dtype=np.float32)
        f = np.zeros(max(n, 1), dtype=np.float32)
        self.L.ref_buf_entries(self.h, self.dim, _p(X), _p(f))
        return X[:n], f[:n]

    def clusters(self):
        n = self.L.ref_buf_size(self.h)
        c = np.zeros((max(n, 1), self.dim), dtype=np.float32)
        m = np.zeros(max(n, 1), dtype=np.int32)
        fl = np.zeros(max(n, 1), dtype=np.int32)
        got = self.L.ref_buf_clusters(self.h, self.dim, _p(c), _p(m), _p(fl))
        return c[:got], m[:got], fl[:got]

    def close(self):
        self.L.ref_buf_destroy(self.h)


def _state(a, d):
    """Per island: (size, list length, head, list, member, flag, order, entries[C][D+1], centres[C][D])."""
    ints, flts = a.view()
    N, C, D = d.n_islands, d.buffer_capacity, d.dim
    out = []
    for s in range(N):
        row = ints[s]
        lst = row[4:4 + N]
        member = row[4 + N:4 + N + C]
        flag = row[4 + N + C:4 + N + 2 * C]
        order = row[4 + N + 2 * C:4 + N + 3 * C]
        ent = flts[s, :C * (D + 1)].reshape(C, D + 1)
        cen = flts[s, C * (D + 1):C * (D + 1) + C * D].reshape(C, D)
        out.append(dict(length=int(row[0]), head=int(row[1]), size=int(row[2]), list=lst.copy(), member=member.copy(),
                        flag=flag.copy(), order=order.copy(), entries=ent.copy(), centres=cen.copy()))
    return out


def _messages(oracle, d, st, g):
    """The messages migrate_in(g) delivers, per destination island in source order: rows of the
    source island (SendEmigrations, src/migrate.cc:105-136, with the library's draws)."""
    P = d.island_size
    msgs = {i: [] for i in range(d.n_islands)}
    for src in range(d.n_islands):
        h = st[src]
        if h["head"] >= h["length"]:
            continue
        dst = int(h["list"][h["head"]])
        key = np.array(oracle.philox([src, g, 0, 8], oracle.key_of(d.seed)), dtype=np.uint32)
        rows = [src * P + oracle.fperm(P, key, q) for q in range(d.migration_size)]
        msgs[dst].append(rows)
    return msgs


def _check_buffer(ref_isl, st_isl, policy, D):
    X, f = ref_isl.entries()
    size = st_isl["size"]
    assert len(f) == size
    ent = st_isl["entries"]
    if policy == 0:          # OnlineCluster: slot c is the vector's position c
        slots = list(range(size))
        c, m, fl = ref_isl.clusters()
        assert np.array_equal(c, st_isl["centres"][:size])
        assert np.array_equal(m, st_isl["member"][:size])
        assert np.array_equal(fl, st_isl["flag"][:size])
    else:                    # the live order gives the vector's positions
        slots = [int(s) for s in st_isl["order"][:size]]
    for pos, slot in enumerate(slots):
        assert np.array_equal(X[pos], ent[slot, :D]), (pos, slot)
        assert f[pos] == ent[slot, D]


@pytest.mark.parametrize("policy", [0, 1, 2, 3, 4])
@pytest.mark.parametrize("N,P,D,k,C,rate", [(4, 32, 6, 3, 5, 1.0), (6, 40, 10, 4, 8, 0.5), (3, 16, 3, 2, 2, 1.0)])
def test_buffers_match_the_reference_classes(oracle, policy, N, P, D, k, C, rate):
    from speo_gb300 import _lib

    L = _ref()
    ld = (D + 3) // 4 * 4
    d = _lib.Archipelago(N, P, D, ld, k, C, policy, 0, rate, 0, 4242 + policy)
    a = oracle.Archipelago(d, 1)
    refs = [RefIsland(L, policy, C, D) for _ in range(N)]
    rng = np.random.default_rng(policy * 100 + N)
    replay_select = policy in (0, 1, 3)
    selections = 0
    try:
        for g in range(40):
            # fresh rows every generation, with repeated fitness values so that ties occur
            pop = np.zeros((N * P, ld), dtype=np.float32)
            pop[:, :D] = rng.uniform(-100, 100, (N * P, D)).astype(np.float32)
            fit = rng.integers(0, 50, N * P).astype(np.float32)
            if g % 3 == 0:                                   # MigrateOut every third generation
                before = _state(a, d)
                a.migrate_out(pop, fit, g)
                after = _state(a, d)
                for s in range(N):
                    taken = before[s]["size"] - after[s]["size"] if policy != 0 else int(before[s]["flag"].sum())
                    if not replay_select:
                        # carry the oracle's selection over to the reference object, so that the
                        # next UpdateBuffer calls start from the same buffer
                        slots = [int(c) for c in after[s]["order"][:after[s]["size"]]]
                        ent = after[s]["entries"]
                        refs[s].assign(ent[slots, :D].reshape(len(slots), D), ent[slots, D])
                        continue
                    X, f = refs[s].select(k)
                    assert len(f) == taken
                    key = np.array(oracle.philox([s, g, 0, 9], oracle.key_of(d.seed)), dtype=np.uint32)
                    for q in range(len(f)):
                        row = s * P + oracle.fperm(P, key, q)
                        assert np.array_equal(pop[row, :D], X[q]) and fit[row] == f[q], (g, s, q)
                        selections += 1
            st = _state(a, d)
            msgs = _messages(oracle, d, st, g)
            a.migrate_in(pop, fit, g)
            st = _state(a, d)
            for dst in range(N):
                for rows in msgs[dst]:
                    refs[dst].update(pop[rows, :D], fit[rows])
                _check_buffer(refs[dst], st[dst], policy, D)
        if replay_select and rate == 1.0:
            assert selections > 0
    finally:
        for r in refs:
            r.close()
