"""Ring migration across ranks: the island ring of one run partitioned over ranks in contiguous
blocks.

The reference migrates between MPI ranks through host buffers (src/migrate.cc:71-136: D2H copies
of the whole population, MPI_Isend / MPI_Iprobe / MPI_Recv). Here rank r holds islands
[r n, (r + 1) n) of the global ring i -> i + 1 (mod N = n x world) in one local population buffer,
followed by 2 k "ghost" rows, and one migration (each island's best k rows replace the next
island's worst k rows, every emigrant chosen before any row is replaced) is:

  1. out:   the block's last island's k best rows are copied to the outgoing ghost rows
            (the ring kernel on the two-segment ring last island -> ghost);
  2. local: the ring kernel on the block's islands, the last one with no local successor;
  3. trade: the outgoing ghost rows go to rank r + 1 and rank r - 1's arrive in the incoming ghost
            rows (point-to-point send / receive of k (ld + 1) floats; nothing else crosses ranks);
  4. in:    the ring kernel on the two-segment ring ghost -> the block's first island.

Every kernel reads local memory only. The ring kernel picks emigrants best first by (fitness,
row) and replaces the worst rows worst first; the outgoing ghost rows are filled worst row
first, so they are sent in reverse, which makes the incoming rows best first with ties in the
sender's row order: the result is row for row that of the single-buffer ring over all N islands.
The host side is the same for the device (library kernels, NCCL or gloo) and for the oracle
(numpy arrays), which the CPU tests run under gloo.
"""
from __future__ import annotations

import ctypes

import numpy as np


class RingBlock:
    """Rank `rank` of `world`: n_local islands of P rows (dimension D, row stride ld), k migrants.
    Rows [0, n_local P) of the local buffer are the islands, then k outgoing and k incoming ghost
    rows."""

    def __init__(self, n_local: int, P: int, D: int, ld: int, k: int, rank: int, world: int):
        if n_local < 1 or P < k or k < 1:
            raise ValueError("a block needs at least one island of at least k rows")
        self.n, self.P, self.D, self.ld, self.k = n_local, P, D, ld, k
        self.rank, self.world = rank, world
        self.ghost_out = n_local * P
        self.ghost_in = n_local * P + k
        self.rows = n_local * P + 2 * k

    # the three rings, as (row0, pop_size, ring_next) per segment
    def ring_out(self):
        return [((self.n - 1) * self.P, self.P, 1), (self.ghost_out, self.k, -1)]

    def ring_local(self):
        nxt = lambda j: j + 1 if j + 1 < self.n else -1  # noqa: E731
        if self.world == 1:
            nxt = lambda j: (j + 1) % self.n  # noqa: E731  (the whole ring is local)
        return [(j * self.P, self.P, nxt(j)) for j in range(self.n)]

    def ring_in(self):
        return [(self.ghost_in, self.k, 1), (0, self.P, -1)]

    def migrate(self, ops, pop, fit) -> None:
        """One migration on this rank's buffer through `ops` (DeviceRingOps or HostRingOps)."""
        if self.world == 1:
            ops.ring(self, self.ring_local(), pop, fit)
            return
        ops.fill_worst(fit, self.ghost_out, self.k)
        ops.ring(self, self.ring_out(), pop, fit)
        ops.ring(self, self.ring_local(), pop, fit)
        ops.trade(self, pop, fit)
        ops.ring(self, self.ring_in(), pop, fit)


class HostRingOps:
    """The oracle's ring (numpy buffers), with torch.distributed point-to-point messages."""

    def __init__(self, oracle):
        self.oracle = oracle

    def fill_worst(self, fit, row0, k):
        fit[row0:row0 + k] = np.inf

    def ring(self, blk, segs, pop, fit):
        self.oracle.ring_migrate([dict(row0=r, P=p, D=blk.D, ld=blk.ld, ring_next=n) for r, p, n in segs], blk.k,
                                 pop, fit)

    def trade(self, blk, pop, fit):
        import torch
        import torch.distributed as dist

        k, ld = blk.k, blk.ld
        msg = np.concatenate([pop[blk.ghost_out:blk.ghost_out + k][::-1].reshape(-1),
                              fit[blk.ghost_out:blk.ghost_out + k][::-1]]).astype(np.float32)
        got = torch.empty(k * ld + k, dtype=torch.float32)
        reqs = [dist.isend(torch.from_numpy(np.ascontiguousarray(msg)), (blk.rank + 1) % blk.world),
                dist.irecv(got, (blk.rank - 1) % blk.world)]
        for r in reqs:
            r.wait()
        g = got.numpy()
        pop[blk.ghost_in:blk.ghost_in + k] = g[:k * ld].reshape(k, ld)
        fit[blk.ghost_in:blk.ghost_in + k] = g[k * ld:]


class DeviceRingOps:
    """The library's ring kernel (speo_ring_migrate) on torch device buffers, with
    torch.distributed point-to-point messages (NCCL between GPUs)."""

    def __init__(self, device):
        import torch

        from . import _lib

        self.torch, self._lib, self.L = torch, _lib, _lib.load()
        self.device = device
        self._tables = {}
        self._staging = None

    def _table(self, blk, segs):
        key = (id(blk), tuple(segs))
        if key not in self._tables:
            arr = (self._lib.Segment * len(segs))()
            for i, (r, p, n) in enumerate(segs):
                arr[i].row0, arr[i].pop_size, arr[i].dim, arr[i].ld, arr[i].ring_next = r, p, blk.D, blk.ld, n
            host = self.torch.frombuffer(bytearray(bytes(arr)), dtype=self.torch.uint8)
            self._tables[key] = host.to(self.device)
        return self._tables[key]

    def fill_worst(self, fit, row0, k):
        fit[row0:row0 + k] = float("inf")

    def ring(self, blk, segs, pop, fit):
        need = len(segs) * blk.k * (blk.ld + 1)
        if self._staging is None or self._staging.numel() < need:
            self._staging = self.torch.zeros(need, device=self.device)
        stream = ctypes.c_void_p(self.torch.cuda.current_stream().cuda_stream)
        self._lib.check(self.L.speo_ring_migrate(self._table(blk, segs).data_ptr(), len(segs), blk.k, pop.data_ptr(),
                                                 fit.data_ptr(), self._staging.data_ptr(), blk.ld, stream),
                        "speo_ring_migrate")

    def trade(self, blk, pop, fit):
        import torch.distributed as dist

        torch = self.torch
        k = blk.k
        out = torch.cat([pop[blk.ghost_out:blk.ghost_out + k].flip(0).reshape(-1),
                         fit[blk.ghost_out:blk.ghost_out + k].flip(0)])
        got = torch.empty_like(out)
        reqs = [dist.isend(out, (blk.rank + 1) % blk.world), dist.irecv(got, (blk.rank - 1) % blk.world)]
        for r in reqs:
            r.wait()
        pop[blk.ghost_in:blk.ghost_in + k] = got[:k * blk.ld].view(k, blk.ld)
        fit[blk.ghost_in:blk.ghost_in + k] = got[k * blk.ld:]
