"""GPU tests of the online MLP surrogate: forward, gradients and Adam against the FP64 oracle,
the k-trial generation bit-exact against the oracle's DE restatement, training on the archive,
and the ablation against plain DE at equal numbers of exact evaluations."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DIN, H, SCALE = 50, 256, 0.01


def _cu():
    return ctypes.CDLL("libcuda.so.1")


def dev_to_np(ptr, n):
    """float32[n] from a device pointer owned by the library (driver API copy, synchronous)."""
    out = np.empty(n, dtype=np.float32)
    cu = _cu()
    assert cu.cuCtxSynchronize() == 0
    assert cu.cuMemcpyDtoH_v2(ctypes.c_void_p(out.ctypes.data), ctypes.c_uint64(ptr), ctypes.c_size_t(4 * n)) == 0
    return out


def np_to_dev(ptr, arr):
    arr = np.ascontiguousarray(arr, dtype=np.float32)
    cu = _cu()
    assert cu.cuCtxSynchronize() == 0
    assert cu.cuMemcpyHtoD_v2(ctypes.c_uint64(ptr), ctypes.c_void_p(arr.ctypes.data), ctypes.c_size_t(4 * arr.size)) == 0


class Surr:
    """An speo_surrogate object and raw views of its parameter and gradient buffers."""

    def __init__(self, lib, din=DIN, h=H, cap=1 << 16, batch=4096, lr=1e-3, seed=5):
        from speo_gb300 import _lib

        self.lib = lib
        self.p = ctypes.c_void_p()
        _lib.check(lib.speo_surrogate_create(ctypes.byref(self.p), din, h, cap, batch, lr, SCALE, seed),
                   "speo_surrogate_create")
        th, gr, n = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_int()
        _lib.check(lib.speo_surrogate_params(self.p, ctypes.byref(th), ctypes.byref(gr), ctypes.byref(n)), "params")
        self.theta_ptr, self.grad_ptr, self.n = th.value, gr.value, n.value
        self.din, self.h = din, h

    def theta(self):
        return dev_to_np(self.theta_ptr, self.n)

    def grad(self):
        return dev_to_np(self.grad_ptr, self.n)

    def close(self):
        self.lib.speo_surrogate_destroy(self.p)


def _bf16(x):
    """Round float32 to the nearest BF16, ties to even, returned as float32."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def _forward_bf16_emulated(theta, din, h, X, scale):
    """The tensor-core forward pass with its roundings made explicit: standardise in FP32, round
    inputs, weights and hidden activations to BF16, accumulate exactly (FP64) and round the sums
    to FP32 before each bias add."""
    f32 = np.float32
    W1 = theta[: h * din].reshape(h, din)
    o = h * din
    b1 = theta[o:o + h]; o += h
    W2 = theta[o:o + h * h].reshape(h, h); o += h * h
    b2 = theta[o:o + h]; o += h
    w3 = theta[o:o + h]; b3 = theta[o + h]
    xn = _bf16((X[:, :din] - f32(0)) * f32(scale)).astype(np.float64)
    a1 = (xn @ _bf16(W1).astype(np.float64).T).astype(f32)
    h1 = _bf16(np.maximum(a1 + b1, f32(0))).astype(np.float64)
    a2 = (h1 @ _bf16(W2).astype(np.float64).T).astype(f32)
    h2 = np.maximum(a2 + b2, f32(0)).astype(np.float64)
    return h2 @ w3.astype(np.float64) + float(b3)


@pytest.mark.parametrize("din,h,n,ldx", [(50, 256, 1000, 52), (50, 256, 128, 50), (10, 64, 777, 12),
                                         (64, 128, 300, 64)])
def test_forward_bf16_matches_emulation(lib, cuda, din, h, n, ldx):
    """tcgen05 forward (BF16 operands, FP32 accumulation) against the same roundings in numpy:
    only the order of the FP32 accumulation differs."""
    import torch
    from speo_gb300 import _lib

    s = Surr(lib, din=din, h=h)
    try:
        rng = np.random.default_rng(din + h)
        theta = (rng.normal(0, 1, s.n) * np.sqrt(2.0 / np.where(np.arange(s.n) < h * din, din, h))).astype(np.float32)
        np_to_dev(s.theta_ptr, theta)
        X = np.zeros((n, ldx), dtype=np.float32)
        X[:, :din] = rng.uniform(-100, 100, (n, din))
        if ldx > din:
            X[:, din:] = 1e30        # padding must never reach the network
        tX = torch.from_numpy(X).cuda()
        y = torch.full((n + 1,), -7.0, device="cuda")
        _lib.check(lib.speo_surrogate_forward_bf16(s.p, tX.data_ptr(), n, ldx, y.data_ptr(), None), "forward_bf16")
        torch.cuda.synchronize()
        got = y.cpu().numpy()
        assert got[n] == -7.0        # nothing written past n rows
        ref = _forward_bf16_emulated(theta, din, h, X, SCALE)
        scale = np.abs(ref).max() + 1.0
        np.testing.assert_allclose(got[:n], ref, rtol=0, atol=2e-4 * scale)
        # and close to the FP32 network: BF16 rounding only
        y32 = torch.zeros(n, device="cuda")
        _lib.check(lib.speo_surrogate_forward(s.p, tX.data_ptr(), n, ldx, y32.data_ptr(), None), "forward")
        torch.cuda.synchronize()
        assert np.corrcoef(got[:n], y32.cpu().numpy())[0, 1] > 0.999
    finally:
        s.close()


def test_forward_bf16_rejects_unsupported_shapes(lib, cuda):
    from speo_gb300 import _lib

    s = Surr(lib, din=100, h=256)
    try:
        import torch
        X = torch.zeros(4, 100, device="cuda")
        y = torch.zeros(4, device="cuda")
        assert lib.speo_surrogate_forward_bf16(s.p, X.data_ptr(), 4, 100, y.data_ptr(), None) == _lib.SPEO_ERR_UNSUPPORTED
    finally:
        s.close()


def test_forward_matches_oracle(lib, oracle, cuda):
    import torch

    s = Surr(lib)
    try:
        theta = s.theta()
        rng = np.random.default_rng(1)
        X = np.zeros((300, 52), dtype=np.float32)
        X[:, :DIN] = rng.uniform(-100, 100, (300, DIN))
        tX = torch.from_numpy(X).cuda()
        y = torch.zeros(300, device="cuda")
        from speo_gb300 import _lib
        _lib.check(lib.speo_surrogate_forward(s.p, tX.data_ptr(), 300, 52, y.data_ptr(), None), "forward")
        torch.cuda.synchronize()
        ref = oracle.mlp_forward(theta, DIN, H, SCALE, X[:, :DIN])
        np.testing.assert_allclose(y.cpu().numpy(), ref, rtol=1e-4, atol=1e-4 * np.abs(ref).max())
    finally:
        s.close()


def test_gradients_match_oracle(lib, oracle, cuda):
    import torch
    from speo_gb300 import _lib

    s = Surr(lib, batch=128)
    try:
        theta = s.theta()
        rng = np.random.default_rng(2)
        n = 96
        X = np.zeros((n, 52), dtype=np.float32)
        X[:, :DIN] = rng.uniform(-100, 100, (n, DIN))
        t = rng.normal(2.0, 1.0, n).astype(np.float32)
        tX, tt = torch.from_numpy(X).cuda(), torch.from_numpy(t).cuda()
        loss = ctypes.c_float()
        _lib.check(lib.speo_surrogate_grad(s.p, tX.data_ptr(), n, 52, tt.data_ptr(), ctypes.byref(loss), None), "grad")
        g = s.grad()
        ref_loss, ref = oracle.mlp_loss_grad(theta, DIN, H, SCALE, X[:, :DIN], t)
        assert loss.value == pytest.approx(ref_loss, rel=1e-4)
        # per parameter block: |g - ref| <= 1e-3 * max|ref in block| + 1e-7
        o = 0
        for name, size in [("W1", H * DIN), ("b1", H), ("W2", H * H), ("b2", H), ("w3", H), ("b3", 1)]:
            gb, rb = g[o:o + size], ref[o:o + size]
            tol = 1e-3 * np.abs(rb).max() + 1e-7
            assert np.abs(gb - rb).max() <= tol, (name, np.abs(gb - rb).max(), tol)
            o += size
    finally:
        s.close()


def _grad_bf16_emulated(theta, din, h, X, t, scale):
    """The tensor-core gradient with its roundings made explicit (BF16 at every tensor-core operand,
    exact sums rounded to FP32 before each bias add); returns (mean loss, gradient)."""
    f32, f64 = np.float32, np.float64
    n = X.shape[0]
    W1 = theta[: h * din].reshape(h, din)
    o = h * din
    b1 = theta[o:o + h]; o += h
    W2 = theta[o:o + h * h].reshape(h, h); o += h * h
    b2 = theta[o:o + h]; o += h
    w3 = theta[o:o + h]; b3 = theta[o + h]
    W1b, W2b = _bf16(W1).astype(f64), _bf16(W2).astype(f64)
    xn = _bf16((X[:, :din] - f32(0)) * f32(scale)).astype(f64)
    z1 = (xn @ W1b.T).astype(f32) + b1
    h1f = np.maximum(z1, f32(0))
    h1 = _bf16(h1f).astype(f64)
    z2 = (h1 @ W2b.T).astype(f32) + b2
    h2 = np.maximum(z2, f32(0))
    y = h2.astype(f64) @ w3.astype(f64) + float(b3)
    e = (y - t.astype(f64)).astype(f32)
    dy = (e * f32(2.0 / n)).astype(f32)
    dz2 = _bf16(np.where(z2 > 0, dy[:, None] * w3[None, :], f32(0)).astype(f32)).astype(f64)
    dz1 = _bf16(np.where(h1f > 0, (dz2 @ W2b).astype(f32), f32(0))).astype(f64)
    h2b = _bf16(h2).astype(f64)
    g = np.concatenate([(dz1.T @ xn).ravel(), dz1.sum(0), (dz2.T @ h1).ravel(), dz2.sum(0),
                        (dy.astype(f64)[:, None] * h2b).sum(0), [dy.astype(f64).sum()]])
    return float(np.mean(e.astype(f64) ** 2)), g


@pytest.mark.parametrize("din,h,n", [(50, 256, 1000), (50, 256, 4096), (10, 64, 300), (64, 128, 128)])
def test_gradients_bf16_match_emulation(lib, oracle, cuda, din, h, n):
    """tcgen05 gradient (BF16 operands, FP32 accumulation) against the same roundings in numpy,
    and close to the FP64 oracle's exact gradient."""
    import torch
    from speo_gb300 import _lib

    s = Surr(lib, din=din, h=h, batch=4096)
    try:
        rng = np.random.default_rng(n + h)
        theta = (rng.normal(0, 1, s.n) * np.sqrt(2.0 / np.where(np.arange(s.n) < h * din, din, h))).astype(np.float32)
        np_to_dev(s.theta_ptr, theta)
        ldx = (din + 3) // 4 * 4
        X = np.zeros((n, ldx), dtype=np.float32)
        X[:, :din] = rng.uniform(-100, 100, (n, din))
        t = rng.normal(2.0, 1.0, n).astype(np.float32)
        tX, tt = torch.from_numpy(X).cuda(), torch.from_numpy(t).cuda()
        loss = ctypes.c_float()
        _lib.check(lib.speo_surrogate_grad_bf16(s.p, tX.data_ptr(), n, ldx, tt.data_ptr(), ctypes.byref(loss), None),
                   "grad_bf16")
        g = s.grad()
        ref_loss, ref = _grad_bf16_emulated(theta, din, h, X, t, SCALE)
        exact_loss, exact = oracle.mlp_loss_grad(theta, din, h, SCALE, X[:, :din], t)
        assert loss.value == pytest.approx(ref_loss, rel=1e-4)
        o = 0
        for name, size in [("W1", h * din), ("b1", h), ("W2", h * h), ("b2", h), ("w3", h), ("b3", 1)]:
            gb, rb, xb = g[o:o + size], ref[o:o + size], exact[o:o + size]
            tol = 5e-3 * np.abs(rb).max() + 1e-7
            assert np.abs(gb - rb).max() <= tol, (name, np.abs(gb - rb).max(), tol)
            # BF16 rounding only: the direction of each block agrees with the exact gradient
            cos = float(np.dot(gb, xb) / (np.linalg.norm(gb) * np.linalg.norm(xb) + 1e-30))
            assert cos > 0.99, (name, cos)
            o += size
    finally:
        s.close()


def test_adam_matches_oracle(lib, oracle, cuda):
    from speo_gb300 import _lib

    s = Surr(lib, din=8, h=16, lr=1e-3)
    try:
        rng = np.random.default_rng(3)
        theta = s.theta()
        m = np.zeros_like(theta)
        v = np.zeros_like(theta)
        for step in range(1, 4):
            g = rng.normal(0, 1, s.n).astype(np.float32)
            np_to_dev(s.grad_ptr, g)
            _lib.check(lib.speo_surrogate_adam_step(s.p, None), "adam")
            oracle.adam(theta, m, v, g, 1e-3, 0.9, 0.999, 1e-8, step)
        got = s.theta()
        np.testing.assert_allclose(got, theta, rtol=2e-6, atol=1e-7)
    finally:
        s.close()


def _islands(cuda, n_isl, P, D, func=31, seed=11):
    """n_isl islands of one instance; P an int, or a list of per-island sizes (uneven islands)."""
    from speo_gb300.device import SegmentSpec, SegmentTable
    from speo_gb300.instances import make_instance

    inst = [make_instance(seed, D)]
    sizes = P if isinstance(P, (list, tuple)) else [P] * n_isl
    specs = [SegmentSpec(pop_size=sizes[i], dim=D, func_id=func, instance=0, seed=seed * 100 + i,
                         ring_next=(i + 1) % n_isl) for i in range(n_isl)]
    return SegmentTable(specs, inst, device=str(cuda))


@pytest.mark.parametrize("strategy", [4, 6])
def test_make_trials_match_oracle(lib, oracle, cuda, strategy):
    import torch
    from speo_gb300 import _lib

    tab = _islands(cuda, 3, 40, 50)
    for sp in tab.specs:
        sp.strategy = strategy
    tab = type(tab)(tab.specs, tab.instances, device=str(cuda))
    tab.init_population()
    k = 8
    T = torch.zeros(tab.rows * k, tab.ld, device=cuda)
    _lib.check(lib.speo_make_trials(tab.d_segs.data_ptr(), tab.d_items.data_ptr(), tab.n_items, tab.dim_hi, k,
                                    tab.pop[0].data_ptr(), tab.fit[0].data_ptr(), T.data_ptr(), tab.gen.data_ptr(),
                                    None), "speo_make_trials")
    torch.cuda.synchronize()
    got = T.cpu().numpy().reshape(tab.rows, k, tab.ld)
    pop = tab.pop[0].cpu().numpy()
    fit = tab.fit[0].cpu().numpy()
    for s in tab.oracle_segments():
        P, D = s["P"], s["D"]
        seg_pop = pop[s["row0"]:s["row0"] + P]
        best = int(np.argmin(fit[s["row0"]:s["row0"] + P]))
        for t in range(k):
            cand = np.zeros_like(seg_pop)
            d = oracle.philox_draws(s["seed"], 0, pos0=s["row0"], tag_hi=(t + 1) << 8)
            assert oracle.de_generate(cand, seg_pop, tab.ld, D, np.arange(P), [0.9], [0.5], [strategy], [best],
                                      -100.0, 100.0, d) == 0
            assert np.array_equal(got[s["row0"]:s["row0"] + P, t, :D], cand[:, :D]), f"trial {t}"


def test_training_reduces_loss(lib, cuda):
    import torch
    from speo_gb300 import _lib
    from speo_gb300.instances import make_instance
    import speo_oracle

    s = Surr(lib, cap=1 << 15, batch=1024, lr=1e-3)
    try:
        o, M = make_instance(4, DIN)
        rng = np.random.default_rng(4)
        X = np.zeros((1 << 15, 52), dtype=np.float32)
        X[:, :DIN] = rng.uniform(-100, 100, (1 << 15, DIN))
        f = speo_oracle.evaluate_rows(31, X, DIN, o, M).astype(np.float32)
        tX, tf = torch.from_numpy(X).cuda(), torch.from_numpy(f).cuda()
        _lib.check(lib.speo_surrogate_archive_append(s.p, tX.data_ptr(), X.shape[0], 52, tf.data_ptr(), None), "append")
        l0, l1 = ctypes.c_float(), ctypes.c_float()
        _lib.check(lib.speo_surrogate_train(s.p, 1, ctypes.byref(l0), None), "train")
        _lib.check(lib.speo_surrogate_train(s.p, 300, ctypes.byref(l1), None), "train")
        assert l1.value < 0.2 * l0.value, (l0.value, l1.value)
    finally:
        s.close()


def _run(lib, cuda, use_surrogate, gens, seed, D=10, n_isl=8, P=64, k=8, func=31):
    """Best FP64 error after `gens` generations of n_isl x P islands (ring migration every 25).
    Screened runs: MLP D -> 64 -> 64 -> 1, archive of the last 8 generations, 32 Adam steps
    (lr 3e-3, batch 1024) per generation, 25 % of targets take a random trial."""
    import torch
    from speo_gb300 import _lib

    tab = _islands(cuda, n_isl, P, D, func=func, seed=seed)
    tab.init_population()
    s = Surr(lib, din=D, h=64, cap=8 * n_isl * P, batch=1024, lr=3e-3, seed=seed) if use_surrogate else None
    try:
        for g in range(gens):
            if use_surrogate:
                a, b = tab.cur, 1 - tab.cur
                _lib.check(lib.speo_surrogate_generation(s.p, tab.d_segs.data_ptr(), tab.d_items.data_ptr(),
                                                         tab.n_items, tab.dim_lo, tab.dim_hi, tab.rows, tab.ld, k,
                                                         tab.pop[a].data_ptr(), tab.fit[a].data_ptr(),
                                                         tab.pop[b].data_ptr(), tab.fit[b].data_ptr(),
                                                         tab.gen.data_ptr(), 32, 0.25, None), "surrogate generation")
                tab.cur = b
            else:
                tab.generation()
            if (g + 1) % 25 == 0:
                tab.migrate(3)
        rows, errs = tab.best_f64()
        torch.cuda.synchronize()
        return float(errs.min().item())
    finally:
        if s is not None:
            s.close()


def test_surrogate_beats_plain_de_at_equal_exact_evaluations(lib, cuda):
    """Rotated sphere, D = 10, 8 islands x 64: both variants spend exactly 512 exact evaluations
    per generation; after the same number of generations the screened run must be far ahead
    (median over seeds). The rotated Rastrigin figures are printed for information."""
    gens = 100
    ratios = []
    for seed in (21, 22, 23):
        plain = _run(lib, cuda, False, gens, seed)
        screened = _run(lib, cuda, True, gens, seed)
        ratios.append(plain / max(screened, 1e-300))
        print(f"sphere seed {seed}: plain DE best error {plain:.3e}, surrogate-screened {screened:.3e}")
    for seed in (21,):
        print(f"rastrigin seed {seed}: plain {_run(lib, cuda, False, gens, seed, func=9):.3e}, "
              f"screened {_run(lib, cuda, True, gens, seed, func=9):.3e}")
    assert np.median(ratios) > 10.0, ratios


def test_surrogate_on_uneven_islands(lib, cuda):
    """The screened generation over islands of uneven size in one table (one launch per stage):
    every island keeps exactly its own rows, the kept fitness is the exact fitness of the kept rows
    (re-evaluated), and at equal exact evaluations the screened run is ahead of plain DE."""
    import torch

    sizes = [40, 64, 100, 33, 77, 128, 52, 90]
    errs = {}
    for use in (False, True):
        tab = _islands(cuda, len(sizes), sizes, 10, func=31, seed=31)
        tab.init_population()
        s = Surr(lib, din=10, h=64, cap=8 * sum(sizes), batch=1024, lr=3e-3, seed=31) if use else None
        try:
            for g in range(80):
                if use:
                    tab.surrogate_generation(s.p, k=8, train_steps=32, explore=0.25)
                else:
                    tab.generation()
                if (g + 1) % 20 == 0:
                    tab.migrate(2)
            torch.cuda.synchronize()
            assert tab.rows == sum(sizes)
            fit = tab.fit[tab.cur].clone()
            again = torch.full_like(fit, float("nan"))
            tab.evaluate(out=again)
            torch.cuda.synchronize()
            assert torch.equal(fit[:tab.rows], again[:tab.rows])
            rows, e = tab.best_f64()
            errs[use] = float(e.min().item())
        finally:
            if s is not None:
                s.close()
    print(f"uneven islands, sphere D=10: plain {errs[False]:.3e}, screened {errs[True]:.3e}")
    assert errs[True] < errs[False] / 10.0


def test_surrogate_generation_replays_from_a_cuda_graph(lib, cuda):
    """The archive ring head and fill and the Adam step counter live on the device, so generations
    captured once in a CUDA graph and replayed give bit-identical populations, fitness and network
    parameters to the same generations run eagerly (the archive wraps during the run)."""
    import torch

    tabs, surrs = [], []
    for _ in range(2):
        tab = _islands(cuda, 8, 64, 10, func=31, seed=5)
        tab.init_population()
        tabs.append(tab)
        surrs.append(Surr(lib, din=10, h=64, cap=4096, batch=1024, lr=3e-3, seed=5))
    try:
        def gen(i):
            tabs[i].surrogate_generation(surrs[i].p, k=8, train_steps=4, explore=0.25)

        for i in range(2):       # eager: scratch sizing and archive seeding
            gen(i)
            gen(i)
        for _ in range(6):
            gen(0)
        g = torch.cuda.CUDAGraph()
        cs = torch.cuda.Stream()
        cs.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(cs), torch.cuda.graph(g, stream=cs):
            gen(1)
            gen(1)
        torch.cuda.current_stream().wait_stream(cs)
        for _ in range(3):
            g.replay()
        torch.cuda.synchronize()
        a, b = tabs[0], tabs[1]
        assert a.cur == b.cur
        assert torch.equal(a.pop[a.cur], b.pop[b.cur])
        assert torch.equal(a.fit[a.cur], b.fit[b.cur])
        assert np.array_equal(surrs[0].theta(), surrs[1].theta())
        assert int(a.gen[0].item()) == int(b.gen[0].item())
    finally:
        for s_ in surrs:
            s_.close()

