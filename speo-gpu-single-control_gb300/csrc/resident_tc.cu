// resident_tc.cu -- island-resident DE epochs with the rotation on the tcgen05 tensor cores.
//
// The reference runs each generation as separate launches over HBM-resident buffers, with the
// rotation of every trial as an FP64 16x16 shared-memory GEMM (CUDA_EA_library/DE_CUDA.cc:200-216,
// kernel_CEC2014_CUDA.cu:147-181) followed by the objective kernel (:557-587). Here one block
// keeps an island (P <= 256 rows, D <= 64) in shared memory for up to `interval` generations,
// as k_island_epoch does, and each generation
//   (1) draws donors and builds the trial rows on the CUDA cores (the same Philox counters and
//       arithmetic as speo_generation: the trials are bit-identical);
//   (2) scales y = x - o of every trial by the row's power of two (its largest |y_j| into
//       [2^14, 2^15)), splits it two ways into FP16 and stores it into tensor memory as the A
//       operand (one thread per row and K half);
//   (3) one thread issues the three split products per 16-wide K step for each 128-row tile
//       (tcgen05.mma, the scaled M^T's two-way split resident in shared memory as the B operand)
//       into an FP32 accumulator in tensor memory;
//   (4) two threads per row read its z row back (tcgen05.ld, the column split of tcs::epi_split)
//       and reduce the objective with the same packed arithmetic as speo_evaluate_tc, so the
//       fitness of a row is bit-identical to that kernel's;
//   (5) greedy selection (strict `<`, kernel_DE_CUDA.cu:312) in place.
// The rotated Rastrigin (9) and sphere (31) only.
#include <mutex>

#include "dropin.cuh"
#include "host.h"
#include "tc_split.cuh"

SPEO_DEFINE_DEVERR(speo_deverr_resident_tc)

namespace speo {
namespace {

constexpr int kThreadsE = 512;
constexpr int kWarpsE = kThreadsE / 32;
constexpr int kMaxPopE = 2 * tcs::kTileM;  // two 128-row MMA tiles
constexpr int kMaxDimE = 64;               // K = N = round16(D) <= 64
constexpr int kTmemAllocE = 512;           // whole SM: one block per SM
constexpr int kAccColsE = 64;              // accumulator of tile t at columns 64 t
constexpr int kAcolE = 128;                // A operand of tile t at 128 + 64 t (hi, lo 32 apart)
constexpr int kApartE = 32;                // columns of one A part (K <= 64: 32 FP16 pairs)
constexpr long long kWaitBudgetE = 2000000000LL;  // ~1 s at 2 GHz: a longer wait is a failure

__device__ __forceinline__ float4 ld4e(const float *p) { return *reinterpret_cast<const float4 *>(p); }
__device__ __forceinline__ void st4e(float *p, float4 v) { *reinterpret_cast<float4 *>(p) = v; }
__device__ __forceinline__ float f4ge(const float4 &v, int q) { return q == 0 ? v.x : q == 1 ? v.y : q == 2 ? v.z : v.w; }
__device__ __forceinline__ void f4se(float4 &v, int q, float x)
{
    if (q == 0) v.x = x; else if (q == 1) v.y = x; else if (q == 2) v.z = x; else v.w = x;
}

__host__ __device__ inline int up_to(int x, int m) { return (x + m - 1) / m * m; }
__host__ __device__ inline int draw_gens_e(int Pmax)
{
    const int g = 4 * kThreadsE / Pmax;
    return g < 1 ? 1 : g > 8 ? 8 : g;
}

// Shared memory of one island (W = 32 Q floats per population row; trial rows XW = W + 4 apart so
// that the conversion's one-row-per-thread reads are free of bank conflicts):
//   B (two-way split of M^T 2^k_M: hi, lo) | pop[Pmax][W] | fit[Pmax (to 4)] | Xs[Pmax][XW] |
//   sR[GB][Pmax][8] | sF[2][Pmax (to 4)] (the two column parts of each trial's fitness; before
//   the products, the largest |y| of each row's two K halves) | o[W] | rm[Pmax (to 4)] (each
//   trial's epilogue scale)
struct EpochTcLayout {
    size_t b_bytes, off_pop, off_fit, off_xs, off_r, off_f, off_o, off_rm, total;
};

__host__ __device__ inline EpochTcLayout epoch_tc_layout(int Q, int Pmax)
{
    const int W = 32 * Q, XW = W + 4, Kmax = W;  // K = N <= W
    EpochTcLayout L;
    L.b_bytes = (size_t)Kmax * Kmax * 2;
    L.off_pop = (tcs::kParts * L.b_bytes + 1023) & ~(size_t)1023;
    L.off_fit = L.off_pop + (size_t)Pmax * W * 4;
    L.off_xs = L.off_fit + (size_t)up_to(Pmax, 4) * 4;
    L.off_r = L.off_xs + (size_t)Pmax * XW * 4;
    L.off_f = L.off_r + (size_t)draw_gens_e(Pmax) * Pmax * 8 * 4;
    L.off_o = L.off_f + 2 * (size_t)up_to(Pmax, 4) * 4;
    L.off_rm = L.off_o + (size_t)W * 4;
    L.total = L.off_rm + (size_t)up_to(Pmax, 4) * 4;
    return L;
}

__device__ __forceinline__ bool tc_objective(int f) { return f == SPEO_FUNC_ROTATED_RASTRIGIN || f == SPEO_FUNC_ROTATED_SPHERE; }

// The trial rows of one generation from the shared-memory population, with speo_generation's
// arithmetic: the island's (row, 4-element chunk) tasks dealt to all threads of the block (a
// thread's next task is found by stepping, not dividing). ST >= 0 compiles one DE strategy, so the
// mutant carries no dispatch and loads only its donors; ST < 0 reads the strategy at run time.
// The crossover test u01(w) < CR is the exact integer compare cr_take(w, ceil(CR 2^24)).
template <int ST, int W, int XW>
__device__ __forceinline__ void trial_rows(const float *pop, float *Xs, const int *sRg, int P, int D, int nch,
                                           int best, int st_rt, float F, uint32_t thr, float lb, float ub, uint2 key,
                                           long long row0, uint32_t gen, bool &ok_bound)
{
    const int st = ST >= 0 ? ST : st_rt;
    const int ndon = ndonors(st);
    const int tasks = P * nch, dr = kThreadsE / nch, dc = kThreadsE - dr * nch;
    int r = (int)threadIdx.x / nch, c = (int)threadIdx.x - r * nch;
    for (int t = (int)threadIdx.x; t < tasks; t += kThreadsE) {
        const int *sr = sRg + r * 8;
        const int jrand = sr[5], e0 = 4 * c;
        const float4 ti = ld4e(pop + r * W + e0);
        const float4 tb = (ST >= 0 ? strategy_uses_best(ST) && best >= 0 : best >= 0) ? ld4e(pop + best * W + e0) : ti;
        float4 tr[5];
#pragma unroll
        for (int k = 0; k < 5; ++k) tr[k] = k < ndon ? ld4e(pop + sr[k] * W + e0) : ti;
        const uint4 w = philox(make_uint4((uint32_t)c, (uint32_t)(row0 + r), gen, kTagCr), key);
        float4 x4 = make_float4(0.f, 0.f, 0.f, 0.f);
        if constexpr (ST >= 0) {
            // one strategy compiled: the mutant of every element, then a select (no branch per
            // element); the chunk's elements past D stay 0 and are not bound-checked
            const bool full = e0 + 4 <= D;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int e = e0 + q;
                float xr[5];
#pragma unroll
                for (int k = 0; k < 5; ++k) xr[k] = f4ge(tr[k], q);
                const float m = mutant<float>(st, F, f4ge(ti, q), f4ge(tb, q), xr);
                const bool take = e == jrand || cr_take(pick(w, (uint32_t)q), thr);
                float x = take ? m : f4ge(ti, q);
                if (full || e < D) {
                    x = check_bound<float>(x, lb, ub, ok_bound);
                    f4se(x4, q, x);
                }
            }
        } else {
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int e = e0 + q;
                if (e < D) {
                    float x;
                    if (e == jrand || cr_take(pick(w, (uint32_t)q), thr)) {
                        float xr[5];
#pragma unroll
                        for (int k = 0; k < 5; ++k) xr[k] = f4ge(tr[k], q);
                        x = mutant<float>(st, F, f4ge(ti, q), f4ge(tb, q), xr);
                    } else {
                        x = f4ge(ti, q);
                    }
                    x = check_bound<float>(x, lb, ub, ok_bound);
                    f4se(x4, q, x);
                }
            }
        }
        st4e(Xs + r * XW + e0, x4);
        c += dc;
        r += dr;
        if (c >= nch) {
            c -= nch;
            ++r;
        }
    }
}

// Ring migration inside a launch (k > 0): after every generation g with (pos + g + 1) % interval
// == 0 (pos: the run's generation count at the launch's first generation), each island sends its
// k best rows to the staging area, every block of the launch meets at a grid barrier, and each
// island replaces its k worst rows with its ring predecessor's (speo_ring_migrate's semantics:
// best by ascending (fitness, row), worst by descending, NaN ranks as +inf, the worst row takes
// the best emigrant). The launch is cooperative (every block resident), so the barrier ends.
constexpr int kMaxMigrantsE = 32;
struct EpochMig {
    int interval, k, pos;
    float *staging;  // 2 (parity of the migration) x islands x k x (W + 1) floats
    unsigned *bar;   // grid-barrier arrivals, zeroed before the launch
};

// Arrival number `target` of the launch's grid barrier (target = (migration + 1) x blocks);
// bounded wait. Every thread of the block calls it; returns false after a timeout.
__device__ __forceinline__ bool grid_barrier(unsigned *bar, unsigned target)
{
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(bar, 1u);
        const long long t0 = clock64();
        bool ok = true;
        while (*(volatile unsigned *)bar < target)
            if (clock64() - t0 > kWaitBudgetE) { ok = false; break; }
        __threadfence();
        s_ok = ok ? 1 : 0;
    }
    __syncthreads();
    return s_ok != 0;
}

// Arrival only, for a block that has stopped (after a timeout): the blocks still running are not
// left waiting for it, and it does not wait for them.
__device__ __forceinline__ void grid_arrive(unsigned *bar)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(bar, 1u);
    }
}

// Number of migration points among the launch's generations.
__device__ __forceinline__ int migrations_in(const EpochMig &mg, int generations)
{
    if (mg.k <= 0 || mg.interval <= 0) return 0;
    return (mg.pos + generations) / mg.interval - mg.pos / mg.interval;
}

// One in-launch migration of this block's island (rows of W floats in shared memory): each row's
// place in the best order (ascending (f, r)) and in the worst order, the k best rows to the
// staging half of this migration's parity, the grid barrier, then the k worst rows from the ring
// predecessor's emigrants (src; -1: none). Returns whether the barrier was met.
template <int W>
__device__ __noinline__ bool migrate_in_launch(float *pop, float *fit, int P, int D, const speo_segment *segs,
                                               const EpochMig &mg, int m_done, int src, int *s_best, int *s_worst)
{
    const int tid = threadIdx.x, k = mg.k, SW = W + 1;
    float *stg = mg.staging + (size_t)(m_done & 1) * gridDim.x * k * SW;
    __syncthreads();
    for (int r = tid; r < P; r += kThreadsE) {
        const float fr = rank_key(fit[r]);
        int rb = 0, rw = 0;
        for (int j = 0; j < P; ++j) {
            const float fj = rank_key(fit[j]);
            rb += (fj < fr || (fj == fr && j < r)) ? 1 : 0;
            rw += (fj > fr || (fj == fr && j > r)) ? 1 : 0;
        }
        if (rb < k) s_best[rb] = r;
        if (rw < k) s_worst[rw] = r;
    }
    __syncthreads();
    const int next = segs[blockIdx.x].ring_next;
    if (next >= 0 && P < k && tid == 0) atomicOr(&s_deverr, SPEO_DEVERR_BAD_SEGMENT);
    if (next >= 0 && P >= k) {
        for (int i = tid; i < k * D; i += kThreadsE) {
            const int t = i / D, e = i - t * D;
            stg[((size_t)blockIdx.x * k + t) * SW + e] = pop[s_best[t] * W + e];
        }
        for (int t = tid; t < k; t += kThreadsE) stg[((size_t)blockIdx.x * k + t) * SW + W] = fit[s_best[t]];
    }
    if (!grid_barrier(mg.bar, (unsigned)(m_done + 1) * gridDim.x)) return false;
    if (src >= 0) {
        const speo_segment &sp = segs[src];
        if (P < k || sp.pop_size < k || sp.ring_next < 0) {
            if (tid == 0) atomicOr(&s_deverr, SPEO_DEVERR_BAD_SEGMENT);
        } else {
            const int dm = D < sp.dim ? D : sp.dim;
            const float *from = stg + (size_t)src * k * SW;
            for (int i = tid; i < k * dm; i += kThreadsE) {
                const int t = i / dm, e = i - t * dm;
                pop[s_worst[t] * W + e] = __ldcg(from + (size_t)t * SW + e);
            }
            for (int t = tid; t < k; t += kThreadsE) fit[s_worst[t]] = __ldcg(from + (size_t)t * SW + W);
        }
    }
    __syncthreads();
    return true;
}

template <int Q>
__global__ void __launch_bounds__(kThreadsE, 1)
    k_island_epoch_tc(const speo_segment *__restrict__ segs, int Pmax, const float *pop_in, const float *fit_in,
                      float *pop_out, float *fit_out, uint32_t *gen_ctr, int generations, float *hist,
                      long long hist_ld, EpochMig mg)
{
    constexpr int W = 32 * Q, XW = W + 4;
    extern __shared__ __align__(1024) uint8_t smem_e[];
    const EpochTcLayout L = epoch_tc_layout(Q, Pmax);
    uint8_t *b_hi = smem_e;
    float *pop = reinterpret_cast<float *>(smem_e + L.off_pop);
    float *fit = reinterpret_cast<float *>(smem_e + L.off_fit);
    float *Xs = reinterpret_cast<float *>(smem_e + L.off_xs);
    int *sR = reinterpret_cast<int *>(smem_e + L.off_r);
    float *sF = reinterpret_cast<float *>(smem_e + L.off_f);
    float *so = reinterpret_cast<float *>(smem_e + L.off_o);
    float *rm = reinterpret_cast<float *>(smem_e + L.off_rm);
    __shared__ float s_bf[kWarpsE];
    __shared__ int s_bi[kWarpsE];
    __shared__ __align__(8) uint64_t bar_mma;
    __shared__ uint32_t tmem_slot;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const speo_segment &s = segs[blockIdx.x];
    const int D = s.dim, P = s.pop_size, ld = s.ld, nch = (D + 3) >> 2;
    const uint32_t gen0 = *(volatile uint32_t *)gen_ctr;
    __shared__ int s_src, s_nsrc, s_best[kMaxMigrantsE], s_worst[kMaxMigrantsE];
    const int nmig = migrations_in(mg, generations);
    int m_done = 0;  // migrations this block has taken part in (its grid-barrier arrivals)
    if (nmig > 0) {
        // the ring predecessor: the lowest-numbered segment whose ring_next is this one (several:
        // flagged, as speo_ring_migrate does), the segments scanned by all threads at once
        if (tid == 0) { s_src = 0x7fffffff; s_nsrc = 0; }
        __syncthreads();
        for (int i = tid; i < (int)gridDim.x; i += kThreadsE)
            if (segs[i].ring_next == (int)blockIdx.x) {
                atomicMin(&s_src, i);
                atomicAdd(&s_nsrc, 1);
            }
        __syncthreads();
        if (tid == 0) {
            if (s_nsrc > 1) atomicOr(&s_deverr, SPEO_DEVERR_BAD_SEGMENT);
            if (s_nsrc == 0) s_src = -1;
        }
    }
    // every thread of the block reads the same segment: the branch below is block-uniform
    const bool seg_ok = P >= 2 && P <= Pmax && Pmax <= kMaxPopE && D >= 1 && D <= W && D <= kMaxDimE &&
                        (ld & 3) == 0 && ld >= D && tc_objective(s.func_id);
    if (seg_ok) {
        const long long row0 = s.row0;
        const uint2 key = seed_key(s.seed);
        const int st = s.strategy;
        const float F = s.F, lb = s.lb, ub = s.ub;
        const uint32_t thr = cr_threshold<float>(s.CR);
        const float scale = func_scale(s.func_id);
        const int Kp = tcs::round16(D), S = Kp / 16, s_half = (S + 1) / 2, ntile = (P + tcs::kTileM - 1) / tcs::kTileM;
        const int GB = draw_gens_e(Pmax), Pf = up_to(Pmax, 4);

        if (warp == 0) {
            tc::tmem_alloc(&tmem_slot, kTmemAllocE);
            tc::tmem_relinquish();
        }
        if (tid == 32) {
            tc::mbar_init(&bar_mma, 1);
            tc::fence_mbar_init();
        }
        // ---- load the island; split M^T into the B operand (and o into so) ---------------------
        for (int i = tid; i < P * nch; i += kThreadsE) {
            const int r = i / nch, c = i - r * nch;
            st4e(pop + r * W + 4 * c, *reinterpret_cast<const float4 *>(pop_in + (row0 + r) * ld + 4 * c));
        }
        for (int r = tid; r < P; r += kThreadsE) fit[r] = fit_in[row0 + r];
        for (int k = tid; k < W; k += kThreadsE) so[k] = 0.f;
        float bm = tcs::b_absmax(s, tid, kThreadsE);
        for (int o = 16; o > 0; o >>= 1) bm = fmaxf(bm, __shfl_xor_sync(0xffffffffu, bm, o));
        if (lane == 0) s_bf[warp] = bm;
        __syncthreads();
        bm = s_bf[0];
        for (int w = 1; w < kWarpsE; ++w) bm = fmaxf(bm, s_bf[w]);
        const int k_m = tcs::b_exp(bm);
        tcs::build_b(s, Kp, b_hi, L.b_bytes, so, tid, kThreadsE, tcs::pow2i(k_m));
        tc::fence_proxy_async_smem();  // B is read by the tensor cores (async proxy)
        tc::fence_before_sync();
        __syncthreads();
        tc::fence_after_sync();
        const uint32_t tmem = tmem_slot;

        bool ok_draw = true, ok_bound = true, aborted = false;
        int g = 0;
        for (; g < generations; ++g) {
            const uint32_t gen = gen0 + (uint32_t)g;
            __syncthreads();
            // best row (strategies that use it): argmin of fit, NaN as +inf, ties lowest row
            int best = -1;
            if (strategy_uses_best(st)) {
                float bf = __int_as_float(0x7f800000);
                int bi = 0x7fffffff;
                for (int r = tid; r < P; r += kThreadsE) {
                    const float f = rank_key(fit[r]);
                    if (f < bf || (f == bf && r < bi)) { bf = f; bi = r; }
                }
                for (int o = 16; o > 0; o >>= 1) {
                    const float of = __shfl_xor_sync(0xffffffffu, bf, o);
                    const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
                    if (of < bf || (of == bf && oi < bi)) { bf = of; bi = oi; }
                }
                if (lane == 0) { s_bf[warp] = bf; s_bi[warp] = bi; }
                __syncthreads();
                bf = s_bf[0]; bi = s_bi[0];
                for (int w = 1; w < kWarpsE; ++w)
                    if (s_bf[w] < bf || (s_bf[w] == bf && s_bi[w] < bi)) { bf = s_bf[w]; bi = s_bi[w]; }
                best = bi;
            }
            // (1a) donor positions + jrand of generations g .. g + GB - 1, one thread per (gen, row)
            if (g % GB == 0) {
                const int nb = generations - g < GB ? generations - g : GB;
                for (int t = tid; t < nb * P; t += kThreadsE) {
                    const int gi = t / P, r = t - gi * P;
                    int rr[5], jr;
                    ok_draw &= draw_donors_jrand(key, (uint32_t)(row0 + r), gen + (uint32_t)gi, kTagIdx, P, D, rr, jr);
                    int *o = sR + (gi * Pmax + r) * 8;
#pragma unroll
                    for (int k = 0; k < 5; ++k) o[k] = rr[k];
                    o[5] = jr;
                }
                __syncthreads();
            }
            const int *sRg = sR + (g % GB) * Pmax * 8;
            // (1b) trial rows from the shared-memory population (the common DE/rand/1 compiled alone)
            if (st == SPEO_DE_RAND_1)
                trial_rows<SPEO_DE_RAND_1, W, XW>(pop, Xs, sRg, P, D, nch, best, st, F, thr, lb, ub, key, row0, gen,
                                                  ok_bound);
            else
                trial_rows<-1, W, XW>(pop, Xs, sRg, P, D, nch, best, st, F, thr, lb, ub, key, row0, gen, ok_bound);
            __syncthreads();
            // (2) A operand: warp w converts rows of tile (w >> 2) & 1, lane quarter w & 3, K half
            // w >> 3; the row's scale from the largest |y| of its two halves (through sF)
            {
                const int q = warp & 3, t = (warp >> 2) & 1, h = warp >> 3;
                const int m = t * tcs::kTileM + q * 32 + lane;
                const bool live = t < ntile && m < P;
                const float *row = Xs + (size_t)(live ? m : 0) * XW;
                const int s0 = h == 0 ? 0 : s_half, s1 = h == 0 ? s_half : S;
                if (live) sF[h * Pf + m] = tcs::row_absmax(row, so, 16 * s0, 16 * s1, D, true);
                __syncthreads();
                if (t < ntile) {
                    const int k_row = live ? tcs::scale_exp(fmaxf(sF[m], sF[Pf + m])) : 0;
                    if (live && h == 0) rm[m] = tcs::row_scale(scale, k_m, k_row);
                    const float rs = tcs::pow2i(k_row);
                    const uint32_t a = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(kAcolE + tcs::kParts * kApartE * t);
                    for (int k = s0; k < s1; ++k) {
                        uint32_t hi[8], lo[8];
                        tcs::convert16(row, so, 16 * k, D, live, rs, hi, lo);
                        tc::tmem_st32x8(a + (uint32_t)(8 * k), hi);
                        tc::tmem_st32x8(a + (uint32_t)(kApartE + 8 * k), lo);
                    }
                    tc::tmem_wait_st();
                }
                tc::fence_before_sync();
            }
            __syncthreads();
            // (3) products of every tile, one thread
            if (tid == 0) {
                tc::fence_after_sync();
                for (int t = 0; t < ntile; ++t)
                    tcs::issue_split_mma(tmem + (uint32_t)(kAccColsE * t),
                                         tmem + (uint32_t)(kAcolE + tcs::kParts * kApartE * t),
                                         kApartE, b_hi, L.b_bytes, Kp, Kp, 0, S);
                tc::mma_commit(&bar_mma);
            }
            // (4) two threads per row (warp w: lane quarter w & 3, tile (w >> 2) & 1, column part
            // w >> 3) read z back and reduce the objective; part p of row m lands in sF[p][m]
            const int te = (warp >> 2) & 1, he = warp >> 3;
            bool ok = true;
            if (te < ntile) ok = tc::mbar_wait_sleep(&bar_mma, (uint32_t)(g & 1), kWaitBudgetE);
            if (__syncthreads_or(!ok)) {
                aborted = true;
                break;
            }
            if (te < ntile) {
                tc::fence_after_sync();
                const int m = te * tcs::kTileM + (warp & 3) * 32 + lane, h = tcs::epi_split(D);
                const int c0 = he == 0 ? 0 : h, c1 = he == 0 ? (D < h ? D : h) : D;
                const float f = c0 < c1 ? tcs::epilogue_row(tmem + (uint32_t)(kAccColsE * te), warp, D, c0, c1,
                                                            s.func_id, m < P ? rm[m] : 0.f)
                                        : 0.f;
                if (m < P) sF[he * Pf + m] = f;
            }
            tc::fence_before_sync();
            __syncthreads();
            // (5) greedy selection in place: strict `<` (kernel_DE_CUDA.cu:312); the fitness is the
            // first column part's sum plus the second's, as speo_evaluate_tc adds them; with a
            // history buffer, generation g's fitness of the row goes to hist[g][row].
            // (5a) one thread per row decides, updates fit and leaves the decision in sF[r]
            for (int r = tid; r < P; r += kThreadsE) {
                const float tf = sF[r] + sF[Pf + r], fo = fit[r];
                const bool win = tf < fo;
                if (win) fit[r] = tf;
                if (hist) hist[(size_t)g * (size_t)hist_ld + (size_t)(row0 + r)] = win ? tf : fo;
                sF[r] = win ? 1.f : 0.f;
            }
            __syncthreads();
            // (5b) the winners' rows move, (row, chunk) tasks dealt to all threads
            {
                const int tasks = P * nch, dr = kThreadsE / nch, dc = kThreadsE - dr * nch;
                int r = tid / nch, c = tid - r * nch;
                for (int t = tid; t < tasks; t += kThreadsE) {
                    if (sF[r] != 0.f) st4e(pop + r * W + 4 * c, ld4e(Xs + r * XW + 4 * c));
                    c += dc;
                    r += dr;
                    if (c >= nch) {
                        c -= nch;
                        ++r;
                    }
                }
            }
            // (6) ring migration at the run's migration points (out of line: the generation loop
            // keeps its registers)
            if (nmig > 0 && (mg.pos + g + 1) % mg.interval == 0) {
                const bool met = migrate_in_launch<W>(pop, fit, P, D, segs, mg, m_done, s_src, s_best, s_worst);
                ++m_done;
                if (!met) {
                    aborted = true;
                    break;
                }
            }
        }
        // a block that stopped early (a timed-out wait) still arrives at the launch's remaining grid
        // barriers, without waiting
        for (; m_done < nmig; ++m_done) grid_arrive(mg.bar);
        if (!ok_draw) atomicOr(&s_deverr, SPEO_DEVERR_REDRAW_LIMIT);
        if (!ok_bound) atomicOr(&s_deverr, SPEO_DEVERR_BOUND_LIMIT);
        if (aborted && tid == 0) {
            // the products of generation g may still be running: let them finish (bounded)
            // before the tensor memory is released
            atomicOr(&s_deverr, SPEO_DEVERR_WAIT_TIMEOUT);
            tc::mbar_wait(&bar_mma, (uint32_t)(g & 1), kWaitBudgetE);
        }
        tc::fence_before_sync();
        __syncthreads();
        tc::fence_after_sync();
        if (warp == 0) tc::tmem_dealloc(tmem, kTmemAllocE);
        // ---- write the island back (after a timeout: the rows of the last whole generation) -----
        for (int i = tid; i < P * nch; i += kThreadsE) {
            const int r = i / nch, c = i - r * nch;
            *reinterpret_cast<float4 *>(pop_out + (row0 + r) * ld + 4 * c) = ld4e(pop + r * W + 4 * c);
        }
        for (int r = tid; r < P; r += kThreadsE) fit_out[row0 + r] = fit[r];
    } else {
        if (tid == 0) atomicOr(&s_deverr, SPEO_DEVERR_BAD_SEGMENT);
        for (; m_done < nmig; ++m_done) (void)grid_barrier(mg.bar, (unsigned)(m_done + 1) * gridDim.x);
    }
    // ---- advance the generation counter by `generations` once every block has read it -------
    __syncthreads();
    if (tid == 0) {
        __threadfence();
        const unsigned done = atomicAdd(gen_ctr + 1, 1u);
        if (done == gridDim.x - 1) {
            gen_ctr[1] = 0;
            gen_ctr[0] = gen0 + (uint32_t)generations;
            __threadfence();
        }
    }
}

int optin_smem()
{
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    return v;
}

size_t epoch_tc_smem(int Q, int max_pop)
{
    const EpochTcLayout L = epoch_tc_layout(Q, max_pop);
    const int limit = optin_smem();
    // more than half of the SM's shared memory: one block (one tensor-memory allocation) per SM
    return L.total > (size_t)limit / 2 + 1024 ? L.total : (size_t)limit / 2 + 1024;
}

// Per (device, Q, max_pop): the launch's shared memory and how many of its blocks fit on the device
// at once (found once: a launch then costs the host one lookup and one attribute call, and a short
// run's timed region includes the host's time to issue it). The attribute is set again on every
// launch, so a device reset (which clears it) needs nothing more.
struct EpochTcShape {
    int dev, Q, max_pop, resident;
    size_t smem;
};
std::mutex g_epoch_shape_mu;
EpochTcShape g_epoch_shape[16];
int g_epoch_shapes = 0;

template <int Q>
int epoch_tc_shape(int max_pop, EpochTcShape *out)
{
    int dev = 0;
    if (int e = check_cuda(cudaGetDevice(&dev), "cudaGetDevice")) return e;
    std::lock_guard<std::mutex> lock(g_epoch_shape_mu);
    for (int i = 0; i < g_epoch_shapes; ++i)
        if (g_epoch_shape[i].dev == dev && g_epoch_shape[i].Q == Q && g_epoch_shape[i].max_pop == max_pop) {
            *out = g_epoch_shape[i];
            return SPEO_OK;
        }
    EpochTcShape sh{dev, Q, max_pop, 0, epoch_tc_smem(Q, max_pop)};
    cudaError_t e = cudaFuncSetAttribute(k_island_epoch_tc<Q>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sh.smem);
    if (e != cudaSuccess) return check_cuda(e, "cudaFuncSetAttribute(k_island_epoch_tc)");
    int coop = 0, sms = 0, per_sm = 0;
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_island_epoch_tc<Q>, kThreadsE, sh.smem) != cudaSuccess) {
        cudaGetLastError();
        per_sm = 0;
    }
    sh.resident = coop ? per_sm * sms : 0;
    if (g_epoch_shapes < 16) g_epoch_shape[g_epoch_shapes++] = sh;
    *out = sh;
    return SPEO_OK;
}

// Whether n_segs blocks of the epoch kernel can all be resident at once (the in-launch migration's
// grid barrier needs every block running).
template <int Q>
bool epoch_tc_coresident(int n_segs, int max_pop)
{
    EpochTcShape sh;
    return epoch_tc_shape<Q>(max_pop, &sh) == SPEO_OK && sh.resident >= n_segs;
}

template <int Q>
int launch_epoch_tc(const speo_segment *segs, int n_segs, int max_pop, const float *pop_in, const float *fit_in,
                    float *pop_out, float *fit_out, uint32_t *d_gen, int generations, float *hist, long long hist_ld,
                    cudaStream_t st, EpochMig mg = EpochMig{0, 0, 0, nullptr, nullptr})
{
    EpochTcShape sh;
    if (int e = epoch_tc_shape<Q>(max_pop, &sh)) return e;
    const size_t smem = sh.smem;
    cudaError_t e = cudaFuncSetAttribute(k_island_epoch_tc<Q>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return check_cuda(e, "cudaFuncSetAttribute(k_island_epoch_tc)");
    if (mg.k > 0 && mg.interval > 0 && (mg.pos + generations) / mg.interval == mg.pos / mg.interval)
        mg.k = 0;  // no migration point among this launch's generations: an ordinary launch
    if (mg.k > 0) {
        // in-launch migration: every block resident (cooperative launch), barrier count from 0
        if (int r = check_cuda(cudaMemsetAsync(mg.bar, 0, sizeof(unsigned), st), "epoch: barrier reset")) return r;
        void *args[] = {(void *)&segs, (void *)&max_pop, (void *)&pop_in, (void *)&fit_in, (void *)&pop_out,
                        (void *)&fit_out, (void *)&d_gen, (void *)&generations, (void *)&hist, (void *)&hist_ld,
                        (void *)&mg};
        return check_cuda(cudaLaunchCooperativeKernel((const void *)k_island_epoch_tc<Q>, dim3(n_segs),
                                                      dim3(kThreadsE), args, smem, st),
                          "cooperative launch of k_island_epoch_tc");
    }
    k_island_epoch_tc<Q><<<n_segs, kThreadsE, smem, st>>>(segs, max_pop, pop_in, fit_in, pop_out, fit_out, d_gen,
                                                          generations, hist, hist_ld, mg);
    return check_launch("k_island_epoch_tc");
}

}  // namespace
}  // namespace speo

using namespace speo;

extern "C" int speo_epoch_tc_fits(int max_pop, int dim_hi)
{
    if (max_pop < 2 || max_pop > kMaxPopE || dim_hi < 1 || dim_hi > kMaxDimE) return 0;
    const int Q = dim_hi <= 32 ? 1 : 2;
    return epoch_tc_layout(Q, max_pop).total <= (size_t)optin_smem() ? 1 : 0;
}

extern "C" int speo_generation_epoch_tc(const speo_segment *segs, int n_segs, int dim_lo, int dim_hi, int max_pop,
                                        const float *pop_in, const float *fit_in, float *pop_out, float *fit_out,
                                        uint32_t *d_gen, int generations, void *stream)
{
    if (!segs || !pop_in || !fit_in || !pop_out || !fit_out || !d_gen || n_segs < 1 || generations < 1)
        return fail(SPEO_ERR_INVALID_ARG, "speo_generation_epoch_tc: bad arguments");
    if (dim_lo < 1 || dim_lo > dim_hi) return fail(SPEO_ERR_INVALID_ARG, "speo_generation_epoch_tc: dim range");
    if (!speo_epoch_tc_fits(max_pop, dim_hi))
        return fail(SPEO_ERR_UNSUPPORTED,
                    "speo_generation_epoch_tc: islands of P <= %d, D <= %d (the tensor-core epochs take P <= %d, "
                    "D <= %d)",
                    max_pop, dim_hi, kMaxPopE, kMaxDimE);
    const int Q = dim_hi <= 32 ? 1 : 2;
    if (dim_lo <= 32 && Q == 2)
        return fail(SPEO_ERR_UNSUPPORTED, "speo_generation_epoch_tc: segments must share one column class");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    return Q == 1 ? launch_epoch_tc<1>(segs, n_segs, max_pop, pop_in, fit_in, pop_out, fit_out, d_gen, generations,
                                       nullptr, 0, st)
                  : launch_epoch_tc<2>(segs, n_segs, max_pop, pop_in, fit_in, pop_out, fit_out, d_gen, generations,
                                       nullptr, 0, st);
}

// ---- the island loop over host buffers ------------------------------------------------------
// IslandEA::Execute (src/island_EA.cc:78-113) runs generations (DE_CUDA::Run) and, every `interval`
// generations, the migration; the island driver reads results back to the host. Here that loop is
// one call: tensor-core epochs of up to `interval` generations per launch, each writing every
// generation's fitness into one of two device history buffers that a second stream copies to the
// caller's host buffer while the next launch runs, and the ring migration at the migration points.
namespace {
struct IslandRunState {
    cudaStream_t copy = nullptr;
    cudaEvent_t made[2] = {nullptr, nullptr}, read[2] = {nullptr, nullptr};
    float *hist = nullptr;
    size_t cap = 0;  // floats
    float *mstg = nullptr;  // in-launch migration staging
    size_t mcap = 0;        // floats
    unsigned *mbar = nullptr;
};
// Generations per launch of the in-launch-migration path when the fitness is read back: four
// migration intervals (the history of one launch is copied while the next runs).
constexpr int kFusedIntervals = 4;
constexpr int kTailGensE = 8;  // generations of the last launch of a run that reads its fitness back

int island_mig_state(IslandRunState *r, size_t floats)
{
    if (!r->mbar)
        if (int e = check_cuda(cudaMalloc(&r->mbar, 256), "island run: barrier")) return e;
    if (r->mcap < floats) {
        if (r->mstg) cudaFree(r->mstg);
        r->mstg = nullptr;
        r->mcap = 0;
        if (int e = check_cuda(cudaMalloc(&r->mstg, sizeof(float) * floats), "island run: migration staging")) return e;
        r->mcap = floats;
    }
    return SPEO_OK;
}
thread_local IslandRunState t_island_run;

int island_run_state(size_t hist_floats, IslandRunState **out)
{
    IslandRunState &r = t_island_run;
    if (!r.copy) {
        if (int e = check_cuda(cudaStreamCreateWithFlags(&r.copy, cudaStreamNonBlocking), "island run: stream"))
            return e;
        for (int b = 0; b < 2; ++b) {
            if (int e = check_cuda(cudaEventCreateWithFlags(&r.made[b], cudaEventDisableTiming), "island run: event"))
                return e;
            if (int e = check_cuda(cudaEventCreateWithFlags(&r.read[b], cudaEventDisableTiming), "island run: event"))
                return e;
        }
    }
    if (r.cap < hist_floats) {  // the previous call synchronised: nothing uses the old buffer
        if (r.hist) cudaFree(r.hist);
        r.hist = nullptr;
        r.cap = 0;
        if (int e = check_cuda(cudaMalloc(&r.hist, sizeof(float) * hist_floats), "island run: history")) return e;
        r.cap = hist_floats;
    }
    *out = &r;
    return SPEO_OK;
}
}  // namespace

namespace {
int island_run(const speo_segment *segs, int n_segs, int dim_lo, int dim_hi, int max_pop, float *pop, float *fit,
               long long rows, uint32_t *d_gen, int first, int generations, int interval, int migrants,
               float *staging, int max_ld, float *h_fitness, bool sync, void *stream)
{
    if (!segs || !pop || !fit || !d_gen || n_segs < 1 || rows < 1 || generations < 0 || first < 0 || interval < 1)
        return fail(SPEO_ERR_INVALID_ARG, "island run: bad arguments");
    if (migrants > 0 && (!staging || max_ld < 1))
        return fail(SPEO_ERR_INVALID_ARG, "island run: migration needs a staging buffer and max_ld");
    if (dim_lo < 1 || dim_lo > dim_hi) return fail(SPEO_ERR_INVALID_ARG, "island run: dim range");
    if (!speo_epoch_tc_fits(max_pop, dim_hi))
        return fail(SPEO_ERR_UNSUPPORTED, "island run: islands of P <= %d, D <= %d are not supported",
                    max_pop, dim_hi);
    const int Q = dim_hi <= 32 ? 1 : 2;
    if (dim_lo <= 32 && Q == 2)
        return fail(SPEO_ERR_UNSUPPORTED, "island run: segments must share one column class");
    if (generations == 0) return SPEO_OK;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    IslandRunState *rs = nullptr;
    // With every island resident at once (cooperative launch), the migrations run inside the
    // launches: one launch for the whole run, or kFusedIntervals intervals per launch when the
    // fitness is read back; otherwise one launch per interval and speo_ring_migrate between.
    const bool fused = migrants > 0 && migrants <= kMaxMigrantsE &&
                       (Q == 1 ? epoch_tc_coresident<1>(n_segs, max_pop) : epoch_tc_coresident<2>(n_segs, max_pop));
    const long long span = fused ? (h_fitness ? (long long)interval * kFusedIntervals : (long long)generations)
                                 : (long long)interval;
    const size_t per = (size_t)(span < generations ? span : generations) * (size_t)rows;  // one launch's history
    if (int e = island_run_state(h_fitness ? 2 * per : 0, &rs)) return e;
    EpochMig mg{0, 0, 0, nullptr, nullptr};
    if (fused) {
        if (int e = island_mig_state(rs, (size_t)2 * n_segs * migrants * (32 * Q + 1))) return e;
        mg = EpochMig{interval, migrants, 0, rs->mstg, rs->mbar};
    }
    int e = SPEO_OK, done = 0;
    for (int i = 0; !e && done < generations; ++i) {
        const int pos = first + done;
        const int left = generations - done;
        // fused with read-back: launches of `span`, the last one at most kTailGensE generations
        // long, so that the history copy left after the last launch is short
        const int tail = interval < kTailGensE ? interval : kTailGensE;
        const int k = fused ? (!h_fitness || left <= tail ? (int)(left < span ? left : span)
                                                          : (int)(left - tail < span ? left - tail : span))
                            : (left < interval - pos % interval ? left : interval - pos % interval);
        const int b = i & 1;
        float *hb = h_fitness ? rs->hist + (size_t)b * per : nullptr;
        if (h_fitness && i >= 2) e = check_cuda(cudaStreamWaitEvent(st, rs->read[b], 0), "island run: wait");
        mg.pos = pos;
        if (!e)
            e = Q == 1 ? launch_epoch_tc<1>(segs, n_segs, max_pop, pop, fit, pop, fit, d_gen, k, hb, rows, st, mg)
                       : launch_epoch_tc<2>(segs, n_segs, max_pop, pop, fit, pop, fit, d_gen, k, hb, rows, st, mg);
        if (!e && h_fitness) {
            e = check_cuda(cudaEventRecord(rs->made[b], st), "island run: record");
            if (!e) e = check_cuda(cudaStreamWaitEvent(rs->copy, rs->made[b], 0), "island run: wait");
            if (!e)
                e = check_cuda(cudaMemcpyAsync(h_fitness + (size_t)done * (size_t)rows, hb,
                                               sizeof(float) * (size_t)k * (size_t)rows, cudaMemcpyDeviceToHost,
                                               rs->copy),
                               "island run: fitness read-back");
            if (!e) e = check_cuda(cudaEventRecord(rs->read[b], rs->copy), "island run: record");
        }
        done += k;
        if (!e && !fused && migrants > 0 && (first + done) % interval == 0)
            e = speo_ring_migrate(segs, n_segs, migrants, pop, fit, staging, max_ld, st);
    }
    if (h_fitness)
        for (int b = 0; b < 2; ++b)
            if (int e2 = check_cuda(cudaStreamWaitEvent(st, rs->read[b], 0), "island run: wait"); e2 && !e) e = e2;
    if (!sync) return e;
    const int es = check_cuda(cudaStreamSynchronize(st), "island run: sync");
    return e ? e : es;
}
}  // namespace

extern "C" int speo_island_run_tc(const speo_segment *segs, int n_segs, int dim_lo, int dim_hi, int max_pop,
                                  float *pop, float *fit, long long rows, uint32_t *d_gen, int first, int generations,
                                  int interval, int migrants, float *staging, int max_ld, float *h_fitness,
                                  void *stream)
{
    return island_run(segs, n_segs, dim_lo, dim_hi, max_pop, pop, fit, rows, d_gen, first, generations, interval,
                      migrants, staging, max_ld, h_fitness, true, stream);
}

extern "C" int speo_island_epochs_tc(const speo_segment *segs, int n_segs, int dim_lo, int dim_hi, int max_pop,
                                     float *pop, float *fit, long long rows, uint32_t *d_gen, int first,
                                     int generations, int interval, int migrants, float *staging, int max_ld,
                                     void *stream)
{
    return island_run(segs, n_segs, dim_lo, dim_hi, max_pop, pop, fit, rows, d_gen, first, generations, interval,
                      migrants, staging, max_ld, nullptr, false, stream);
}
