"""Device-side tables for the extended C ABI, built with torch for device memory.

`SegmentTable` holds the population double buffers, the segment descriptors, the planned
work items and the per-instance (shift, M^T) data in HBM, and calls the library's entry
points on them. It is the thin host layer the tests and the benchmark drive; the generation
loop itself (graph capture, migration cadence, best tracking) is in the library's C++
island driver.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib
from .instances import rot_layout, shift_layout


@dataclass
class SegmentSpec:
    pop_size: int
    dim: int
    func_id: int
    instance: int                 # index into the instance list
    seed: int
    F: float = 0.5
    CR: float = 0.9
    lb: float = -100.0
    ub: float = 100.0
    strategy: int = _lib.DE_RAND_1
    ring_next: int = -1
    ld: int | None = None


AUTOTUNE_CANDIDATES = (32, 48, 64)


def tune_tile_rows(host_segs: ctypes.Array, n_segs: int, candidates=AUTOTUNE_CANDIDATES, reps: int = 5):
    """The library's tuner (speo_autotune_tile_rows) on a host segment table: (tile rows,
    {"ms": {tile: ms per generation}, "cached": bool})."""
    L = _lib.load()
    cand = (ctypes.c_int * len(candidates))(*candidates)
    tile = ctypes.c_int(0)
    cached = ctypes.c_int(0)
    ms = (ctypes.c_float * len(candidates))()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.check(L.speo_autotune_tile_rows(ctypes.addressof(host_segs), n_segs, ctypes.addressof(cand), len(candidates),
                                         reps, ctypes.byref(tile), ctypes.addressof(ms), ctypes.byref(cached), stream),
               "speo_autotune_tile_rows")
    return tile.value, {"ms": {c: ms[i] for i, c in enumerate(candidates)}, "cached": bool(cached.value)}


def _bytes_to_device(buf: ctypes.Array, device) -> torch.Tensor:
    host = torch.frombuffer(bytearray(bytes(buf)), dtype=torch.uint8)
    return host.to(device)


@dataclass
class SegmentTable:
    specs: list[SegmentSpec]
    # (o, M) float32, or (o, M, S) for ids 17-30: o (nc, D), M (nc, D, D), S (nc, D) 1-based int32
    instances: list[tuple]
    tile_rows: int | str = _lib.TILE_SIMT  # rows per work item, or "auto": the library's tuner picks it
    device: str = "cuda"
    extra_rows: int = 0           # rows past the segments' rows in the population buffers (ring ghost rows)
    rows: int = field(init=False)

    def __post_init__(self):
        L = _lib.load()
        dev = torch.device(self.device)
        self.inst_shift = []
        self.inst_rot = []
        self.inst_shuf = []
        for inst in self.instances:
            # component c: shift at c*ldr, D rows of M^T at c*D*ldr, shuffle at c*ldr
            o = np.atleast_2d(inst[0])
            nc, D = o.shape
            M = np.asarray(inst[1]).reshape(nc, D, D)
            ldr = (D + 3) // 4 * 4
            self.inst_shift.append(torch.from_numpy(np.concatenate([shift_layout(o[c], ldr) for c in range(nc)])).to(dev))
            self.inst_rot.append(torch.from_numpy(np.concatenate([rot_layout(M[c], ldr) for c in range(nc)])).to(dev))
            shuf = None
            if len(inst) > 2 and inst[2] is not None:
                S = np.atleast_2d(inst[2]).astype(np.int32)
                pad = np.zeros((nc, ldr), dtype=np.int32)
                pad[:, :D] = S
                shuf = torch.from_numpy(pad.reshape(-1)).to(dev)
            self.inst_shuf.append(shuf)
        segs = (_lib.Segment * len(self.specs))()
        row = 0
        self.max_ld = 0
        # rows of every segment share one stride so a flat [rows, ld] buffer can hold them
        self.ld = max((sp.ld or (sp.dim + 3) // 4 * 4) for sp in self.specs)
        for i, sp in enumerate(self.specs):
            s = segs[i]
            s.row0 = row
            s.pop_size = sp.pop_size
            s.dim = sp.dim
            s.ld = self.ld
            s.func_id = sp.func_id
            s.strategy = sp.strategy
            s.F, s.CR, s.lb, s.ub = sp.F, sp.CR, sp.lb, sp.ub
            s.shift = self.inst_shift[sp.instance].data_ptr()
            s.rot = self.inst_rot[sp.instance].data_ptr()
            s.ld_rot = self.inst_rot[sp.instance].shape[1]
            shuf = self.inst_shuf[sp.instance]
            s.shuffle = shuf.data_ptr() if shuf is not None else None
            s.ring_next = sp.ring_next
            s.seed = sp.seed
            row += sp.pop_size
        self.rows = row
        self.max_ld = self.ld
        self.host_segs = segs
        self.d_segs = _bytes_to_device(segs, dev)
        self.autotune = None
        if self.tile_rows == "auto":
            self.tile_rows, self.autotune = tune_tile_rows(segs, len(self.specs))
        n = ctypes.c_int(0)
        _lib.check(L.speo_plan_work(ctypes.addressof(segs), len(self.specs), self.tile_rows, None, 0, ctypes.byref(n)),
                   "speo_plan_work")
        items = (_lib.WorkItem * n.value)()
        _lib.check(L.speo_plan_work(ctypes.addressof(segs), len(self.specs), self.tile_rows, ctypes.addressof(items),
                                    n.value, ctypes.byref(n)), "speo_plan_work")
        self.host_items = items
        self.n_items = n.value
        self.d_items = _bytes_to_device(items, dev)
        self.dim_lo = min(sp.dim for sp in self.specs)
        self.dim_hi = max(sp.dim for sp in self.specs)
        n = self.rows + self.extra_rows
        self.pop = [torch.zeros(n, self.ld, device=dev), torch.zeros(n, self.ld, device=dev)]
        self.fit = [torch.zeros(n, device=dev), torch.zeros(n, device=dev)]
        self.gen = torch.zeros(2, dtype=torch.int32, device=dev)
        self.cur = 0
        self.staging = torch.zeros(len(self.specs) * 32 * (self.max_ld + 1), device=dev)

    # -- entry points ------------------------------------------------------------------------
    @staticmethod
    def _stream():
        return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    def init_population(self):
        L = _lib.load()
        _lib.check(L.speo_init_population(self.d_segs.data_ptr(), len(self.specs), self.d_items.data_ptr(),
                                          self.n_items, self.pop[self.cur].data_ptr(), self._stream()),
                   "speo_init_population")
        self.evaluate()

    def evaluate(self, which: int | None = None, use_tc: bool = False, out: torch.Tensor | None = None):
        """Fitness of population buffer `which` (default: current) into `out` (default: its own
        fitness buffer). use_tc selects the tcgen05 split-FP16 kernel (tiles of 128 rows)."""
        L = _lib.load()
        w = self.cur if which is None else which
        fit = self.fit[w] if out is None else out
        if use_tc:
            _lib.check(L.speo_evaluate_tc(self.d_segs.data_ptr(), self.d_items.data_ptr(), self.n_items, self.dim_lo,
                                          self.dim_hi, self.pop[w].data_ptr(), self.rows, self.ld, fit.data_ptr(),
                                          self._stream()), "speo_evaluate_tc")
        else:
            _lib.check(L.speo_evaluate(self.d_segs.data_ptr(), self.d_items.data_ptr(), self.n_items, self.dim_lo,
                                       self.dim_hi, self.pop[w].data_ptr(), fit.data_ptr(), self._stream()),
                       "speo_evaluate")

    def generation(self, trial_out: torch.Tensor | None = None, trial_fit_out: torch.Tensor | None = None):
        """One fused generation on the CUDA cores (speo_generation); tc_generation is the
        tensor-core form."""
        L = _lib.load()
        a, b = self.cur, 1 - self.cur
        _lib.check(L.speo_generation(self.d_segs.data_ptr(), self.d_items.data_ptr(), self.n_items, self.dim_lo,
                                     self.dim_hi, self.pop[a].data_ptr(), self.fit[a].data_ptr(),
                                     self.pop[b].data_ptr(), self.fit[b].data_ptr(), self.gen.data_ptr(),
                                     0, None if trial_out is None else trial_out.data_ptr(),
                                     None if trial_fit_out is None else trial_fit_out.data_ptr(), self._stream()),
                   "speo_generation")
        self.cur = b

    def epoch_fits(self) -> bool:
        L = _lib.load()
        return bool(L.speo_epoch_fits(max(sp.pop_size for sp in self.specs), self.dim_hi))

    def epoch(self, generations: int, cluster: int = 0):
        """`generations` generations with every island resident in shared memory (in place);
        cluster: 0 = library's choice, 1 = one block per island, 2 = two-block clusters."""
        L = _lib.load()
        w = self.cur
        _lib.check(L.speo_generation_epoch_ex(self.d_segs.data_ptr(), len(self.specs), self.dim_lo, self.dim_hi,
                                              max(sp.pop_size for sp in self.specs), self.pop[w].data_ptr(),
                                              self.fit[w].data_ptr(), self.pop[w].data_ptr(), self.fit[w].data_ptr(),
                                              self.gen.data_ptr(), generations, cluster, self._stream()),
                   "speo_generation_epoch_ex")

    def epoch_tc_fits(self) -> bool:
        L = _lib.load()
        return bool(L.speo_epoch_tc_fits(max(sp.pop_size for sp in self.specs), self.dim_hi))

    def epoch_tc(self, generations: int):
        """`generations` generations with every island resident in shared memory and the rotation
        on the tensor cores (speo_generation_epoch_tc; in place)."""
        L = _lib.load()
        w = self.cur
        _lib.check(L.speo_generation_epoch_tc(self.d_segs.data_ptr(), len(self.specs), self.dim_lo, self.dim_hi,
                                              max(sp.pop_size for sp in self.specs), self.pop[w].data_ptr(),
                                              self.fit[w].data_ptr(), self.pop[w].data_ptr(), self.fit[w].data_ptr(),
                                              self.gen.data_ptr(), generations, self._stream()),
                   "speo_generation_epoch_tc")

    def tc_generation(self, trial: torch.Tensor, trial_fit: torch.Tensor):
        """One generation with the rotation on the tensor cores: one DE trial per target
        (speo_make_trials, k = 1), tcgen05 split-FP16 evaluation, strict-`<` selection. The table must
        be planned with tiles of at most 128 rows."""
        L = _lib.load()
        a, b = self.cur, 1 - self.cur
        _lib.check(L.speo_generation_tc(self.d_segs.data_ptr(), self.d_items.data_ptr(), self.n_items, self.dim_lo,
                                        self.dim_hi, self.pop[a].data_ptr(), self.fit[a].data_ptr(),
                                        self.pop[b].data_ptr(), self.fit[b].data_ptr(), self.rows, self.ld,
                                        self.gen.data_ptr(), trial.data_ptr(), trial_fit.data_ptr(), self._stream()),
                   "speo_generation_tc")
        self.cur = b

    def surrogate_generation(self, surrogate, k: int = 8, train_steps: int = 16, explore: float = 0.25):
        """One surrogate-screened generation (speo_surrogate_generation); `surrogate` is an
        speo_surrogate handle (ctypes.c_void_p)."""
        L = _lib.load()
        a, b = self.cur, 1 - self.cur
        _lib.check(L.speo_surrogate_generation(surrogate, self.d_segs.data_ptr(), self.d_items.data_ptr(),
                                               self.n_items, self.dim_lo, self.dim_hi, self.rows, self.ld, k,
                                               self.pop[a].data_ptr(), self.fit[a].data_ptr(), self.pop[b].data_ptr(),
                                               self.fit[b].data_ptr(), self.gen.data_ptr(), train_steps, explore,
                                               self._stream()), "speo_surrogate_generation")
        self.cur = b

    def island_epochs_tc(self, generations: int, first: int, interval: int, migrants: int):
        """`generations` tensor-core generations with the ring migration of `migrants` rows after
        every multiple of `interval` generations of the run (`first` already done), in place and
        asynchronous (speo_island_epochs_tc: the migrations inside the launch when every island
        is resident at once)."""
        L = _lib.load()
        w = self.cur
        _lib.check(L.speo_island_epochs_tc(self.d_segs.data_ptr(), len(self.specs), self.dim_lo, self.dim_hi,
                                           max(sp.pop_size for sp in self.specs), self.pop[w].data_ptr(),
                                           self.fit[w].data_ptr(), self.rows, self.gen.data_ptr(), first,
                                           generations, interval, migrants, self.staging.data_ptr(), self.max_ld,
                                           self._stream()), "speo_island_epochs_tc")

    def migrate(self, k: int):
        L = _lib.load()
        _lib.check(L.speo_ring_migrate(self.d_segs.data_ptr(), len(self.specs), k, self.pop[self.cur].data_ptr(),
                                       self.fit[self.cur].data_ptr(), self.staging.data_ptr(), self.max_ld,
                                       self._stream()), "speo_ring_migrate")

    def best_f64(self):
        L = _lib.load()
        n = len(self.specs)
        rows = torch.zeros(n, dtype=torch.int64, device=self.pop[0].device)
        errs = torch.zeros(n, dtype=torch.float64, device=self.pop[0].device)
        _lib.check(L.speo_best_reeval_f64(self.d_segs.data_ptr(), n, self.pop[self.cur].data_ptr(),
                                          self.fit[self.cur].data_ptr(), rows.data_ptr(), errs.data_ptr(),
                                          self._stream()), "speo_best_reeval_f64")
        return rows, errs

    def oracle_segments(self) -> list[dict]:
        """The segment table as the oracle's dicts (host copies of o and M)."""
        out = []
        for i, sp in enumerate(self.specs):
            inst = self.instances[sp.instance]
            o, M = inst[0], inst[1]
            S = inst[2] if len(inst) > 2 else None
            out.append(dict(row0=int(self.host_segs[i].row0), P=sp.pop_size, D=sp.dim, ld=self.ld, func=sp.func_id,
                            strategy=sp.strategy, F=sp.F, CR=sp.CR, lb=sp.lb, ub=sp.ub, o=o, M=M, S=S, seed=sp.seed,
                            ring_next=sp.ring_next))
        return out
