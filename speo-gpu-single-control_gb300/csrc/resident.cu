// resident.cu -- island-resident DE epochs: one block per island runs many generations with the
// island's population, the trials and M^T held in shared memory.
//
// The reference runs every generation as separate launches over HBM-resident buffers with a
// device sync after each (CUDA_EA_library/DE_CUDA.cc:200-216), and migrates only every
// `interval` generations (src/island_EA.cc:94-99). Between migrations an island touches nothing
// but itself, so here an epoch of up to `interval` generations is one launch: the island is read
// from HBM once, evolved in shared memory, and written back once. Each generation is the same
// computation as speo_generation (same Philox counters, same FMA order in the mutant and in the
// rotation), so the result is bit-identical to `generations` launches of it.
#include "cluster.cuh"
#include "eval_simt.cuh"
#include "host.h"

SPEO_DEFINE_DEVERR(speo_deverr_resident)

namespace speo {
namespace {

constexpr int kThreads = 512;
constexpr int kWarpsR = kThreads / 32;
constexpr int kEvalRows = kWarpsR * kRowsPerWarp;  // 128 rows per evaluation pass
constexpr int kMaxPop = 512;

__device__ __forceinline__ float4 ld4s(const float *p) { return *reinterpret_cast<const float4 *>(p); }
__device__ __forceinline__ void st4s(float *p, float4 v) { *reinterpret_cast<float4 *>(p) = v; }
__device__ __forceinline__ float f4g(const float4 &v, int q) { return q == 0 ? v.x : q == 1 ? v.y : q == 2 ? v.z : v.w; }
__device__ __forceinline__ void f4s(float4 &v, int q, float x)
{
    if (q == 0) v.x = x; else if (q == 1) v.y = x; else if (q == 2) v.z = x; else v.w = x;
}

__device__ __forceinline__ int donors_for(int st)
{
    switch (st) {
    case 0: case 2: case 6: return 2;
    case 3: case 4: case 8: return 3;
    case 1: case 7: return 4;
    default: return 5;
    }
}

__host__ __device__ __forceinline__ int round_up(int x, int m) { return (x + m - 1) / m * m; }

// Shared memory of one island with population bound Pmax and column class Q (W = 32Q):
//   pop[Pmax][W] fit[round_up(Pmax, 4)] | Xs[Pt][W] Ys[Pt][W] | Ms[D<=32Q][W] | sR[GB][Pmax][8] sF[Pt] | o[W]
// The donor draws depend only on (seed, row, generation), so the block draws them for the next GB
// generations at once (GB x P rows over all threads, instead of P rows per generation).
template <int Q> struct ResPlan {
    static constexpr int W = 32 * Q;
    static constexpr int G = Q == 1 ? 8 : 16;     // lanes per row
    static constexpr int RPP = kThreads / G;      // rows per pass of the block
};

__host__ __device__ inline int draw_gens(int Pmax)
{
    const int g = kThreads / Pmax;
    return g < 1 ? 1 : g > 8 ? 8 : g;
}

__host__ __device__ inline size_t res_smem_floats(int Q, int Pmax)
{
    const int W = 32 * Q, Pt = round_up(Pmax, kEvalRows);
    return (size_t)Pmax * W + round_up(Pmax, 4) + 2 * (size_t)Pt * W + (size_t)W * W + (size_t)draw_gens(Pmax) * Pmax * 8 +
           Pt + W;
}

template <int Q>
__global__ void __launch_bounds__(kThreads, 1)
    k_island_epoch(const speo_segment *__restrict__ segs, int Pmax, const float *pop_in, const float *fit_in,
                   float *pop_out, float *fit_out, uint32_t *gen_ctr, int generations)
{
    using Pl = ResPlan<Q>;
    constexpr int W = Pl::W, G = Pl::G;
    extern __shared__ __align__(16) float sm[];
    const int Pt = round_up(Pmax, kEvalRows);
    float *pop = sm;
    float *fit = pop + (size_t)Pmax * W;
    float *Xs = fit + round_up(Pmax, 4);  // 16-byte aligned: Xs / Ys rows are read as float4
    float *Ys = Xs + (size_t)Pt * W;
    float *Ms = Ys + (size_t)Pt * W;
    const int GB = draw_gens(Pmax);
    int *sR = reinterpret_cast<int *>(Ms + W * W);
    float *sF = reinterpret_cast<float *>(sR + GB * Pmax * 8);
    float *so = sF + Pt;
    __shared__ float s_bf[kWarpsR];
    __shared__ int s_bi[kWarpsR];

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int grp = tid / G, gl = tid % G;
    const speo_segment &s = segs[blockIdx.x];
    const int D = s.dim, P = s.pop_size, ld = s.ld, nch = (D + 3) >> 2;
    const uint32_t gen0 = *(volatile uint32_t *)gen_ctr;
    const bool seg_ok = P >= 2 && P <= Pmax && D >= 1 && D <= W && (ld & 3) == 0 && ld >= D && func_supported(s.func_id);
    if (seg_ok) {
        const long long row0 = s.row0;
        const uint2 key = seed_key(s.seed);
        const int st = s.strategy, ndon = donors_for(st);
        const float F = s.F, CR = s.CR, lb = s.lb, ub = s.ub;
        const float scale = func_scale(s.func_id);

        // ---- load the island, M^T and o ------------------------------------------------------
        for (int i = tid; i < P * nch; i += kThreads) {
            const int r = i / nch, c = i - r * nch;
            st4s(pop + r * W + 4 * c, *reinterpret_cast<const float4 *>(pop_in + (row0 + r) * ld + 4 * c));
        }
        for (int r = tid; r < P; r += kThreads) fit[r] = fit_in[row0 + r];
        load_rot_rows<float, Q>(Ms, s.rot, s.ld_rot, D, 0, D);
        for (int k = tid; k < W; k += kThreads) so[k] = k < 4 * nch ? s.shift[k] : 0.f;
        for (int i = tid; i < (Pt - P) * W; i += kThreads) Ys[P * W + i] = 0.f;

        bool ok_draw = true, ok_bound = true;
        for (int g = 0; g < generations; ++g) {
            const uint32_t gen = gen0 + (uint32_t)g;
            __syncthreads();
            // best row (strategies that use it): argmin of fit, NaN as +inf, ties lowest row
            int best = -1;
            if (strategy_uses_best(st)) {
                float bf = __int_as_float(0x7f800000);
                int bi = 0x7fffffff;
                for (int r = tid; r < P; r += kThreads) {
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
                for (int w = 1; w < kWarpsR; ++w)
                    if (s_bf[w] < bf || (s_bf[w] == bf && s_bi[w] < bi)) { bf = s_bf[w]; bi = s_bi[w]; }
                best = bi;
            }
            // (1) donor positions + jrand of generations g .. g + GB - 1, one thread per (gen, row)
            if (g % GB == 0) {
                const int nb = generations - g < GB ? generations - g : GB;
                for (int t = tid; t < nb * P; t += kThreads) {
                    const int gi = t / P, r = t - gi * P;
                    IdxStream is(key, (uint32_t)(row0 + r), gen + (uint32_t)gi, kTagIdx);
                    int rr[5];
                    ok_draw &= draw_donors(is, P, rr);
                    int *o = sR + (gi * Pmax + r) * 8;
#pragma unroll
                    for (int k = 0; k < 5; ++k) o[k] = rr[k];
                    o[5] = is.index(D);
                }
                __syncthreads();
            }
            const int *sRg = sR + (g % GB) * Pmax * 8;
            // (2) trials from the shared-memory population
            for (int r = grp; r < P; r += Pl::RPP) {
                const int jrand = sRg[r * 8 + 5];
                int dr[5];
#pragma unroll
                for (int k = 0; k < 5; ++k) dr[k] = sRg[r * 8 + k];
                const float *xi = pop + r * W;
                const float *xb = pop + (best >= 0 ? best : r) * W;
                for (int c = gl; c < nch; c += G) {
                    const int e0 = 4 * c;
                    const float4 ti = ld4s(xi + e0);
                    const float4 tb = best >= 0 ? ld4s(xb + e0) : ti;
                    float4 tr[5];
#pragma unroll
                    for (int k = 0; k < 5; ++k) tr[k] = k < ndon ? ld4s(pop + dr[k] * W + e0) : ti;
                    const uint4 w = philox(make_uint4((uint32_t)c, (uint32_t)(row0 + r), gen, kTagCr), key);
                    const float4 o4 = ld4s(so + e0);
                    float4 x4 = make_float4(0.f, 0.f, 0.f, 0.f), y4 = x4;
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        const int e = e0 + q;
                        if (e < D) {
                            const float u = u01(pick(w, (uint32_t)q));
                            float x;
                            if (e == jrand || u < CR) {
                                float xr[5];
#pragma unroll
                                for (int k = 0; k < 5; ++k) xr[k] = f4g(tr[k], q);
                                x = mutant<float>(st, F, f4g(ti, q), f4g(tb, q), xr);
                            } else {
                                x = f4g(ti, q);
                            }
                            x = check_bound<float>(x, lb, ub, ok_bound);
                            f4s(x4, q, x);
                            f4s(y4, q, __fsub_rn(x, f4g(o4, q)));
                        }
                    }
                    st4s(Xs + r * W + e0, x4);
                    st4s(Ys + r * W + e0, y4);
                }
            }
            __syncthreads();
            // (3) evaluate, 128 rows per pass
            for (int pb = 0; pb < Pt; pb += kEvalRows) {
                float acc[kRowsPerWarp][Q];
#pragma unroll
                for (int rr = 0; rr < kRowsPerWarp; ++rr)
#pragma unroll
                    for (int q = 0; q < Q; ++q) acc[rr][q] = 0.f;
                if (func_rotated(s.func_id))
                    eval_accumulate<float, Q>(acc, Ys, W, pb + warp * kRowsPerWarp, Ms, W, 0, D, lane);
                else
                    eval_identity<float, Q>(acc, Ys, W, pb + warp * kRowsPerWarp, D, lane);
                float f[kRowsPerWarp];
                eval_reduce<float, Q>(acc, D, s.func_id, scale, lane, f);
                if (lane == 0)
#pragma unroll
                    for (int rr = 0; rr < kRowsPerWarp; ++rr) sF[pb + warp * kRowsPerWarp + rr] = f[rr];
            }
            __syncthreads();
            // (4) greedy selection in place: strict `<` (kernel_DE_CUDA.cu:312)
            for (int r = grp; r < P; r += Pl::RPP) {
                const float tf = sF[r];
                if (tf < fit[r]) {
                    for (int c = gl; c < nch; c += G) st4s(pop + r * W + 4 * c, ld4s(Xs + r * W + 4 * c));
                    if (gl == 0) fit[r] = tf;
                }
            }
        }
        if (!ok_draw) atomicOr(&s_deverr, SPEO_DEVERR_REDRAW_LIMIT);
        if (!ok_bound) atomicOr(&s_deverr, SPEO_DEVERR_BOUND_LIMIT);
        __syncthreads();
        // ---- write the island back ----------------------------------------------------------
        for (int i = tid; i < P * nch; i += kThreads) {
            const int r = i / nch, c = i - r * nch;
            *reinterpret_cast<float4 *>(pop_out + (row0 + r) * ld + 4 * c) = ld4s(pop + r * W + 4 * c);
        }
        for (int r = tid; r < P; r += kThreads) fit_out[row0 + r] = fit[r];
    } else if (tid == 0) {
        atomicOr(&s_deverr, SPEO_DEVERR_BAD_SEGMENT);
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

// ---- two-block clusters: one island per cluster of 2 -------------------------------------------
// Each block of the pair keeps a full replica of the island in shared memory, double-buffered
// (pop[g % 2] is generation g), and runs the trials, evaluation and selection of one half of the
// rows. Its new rows (winner or parent) go to the next buffer of both replicas: its own, and the
// peer's through distributed shared memory. One cluster barrier per generation then makes both
// replicas whole. Donor reads are local; the per-row arithmetic is the single-block kernel's, so
// the result is bit-identical.
constexpr int kRowsPerWarp2 = 4;
constexpr int kEvalRows2 = kWarpsR * kRowsPerWarp2;  // 64 rows per evaluation pass

__host__ __device__ inline int half_rows(int Pmax) { return (Pmax + 1) / 2; }
__host__ __device__ inline int draw_gens2(int Pmax) { return draw_gens(half_rows(Pmax)); }

//   pop[2][Pmax][W] fit[2][round_up(Pmax, 4)] | Xs[Ph][W] Ys[Ph][W] | Ms[W][W] | sR[GB][h][8] sF[Ph] | o[W]
__host__ __device__ inline size_t res2_smem_floats(int Q, int Pmax)
{
    const int W = 32 * Q, h = half_rows(Pmax), Ph = round_up(h, kEvalRows2);
    return 2 * ((size_t)Pmax * W + round_up(Pmax, 4)) + 2 * (size_t)Ph * W + (size_t)W * W +
           (size_t)draw_gens2(Pmax) * h * 8 + Ph +
           W;
}

template <int Q>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(kThreads, 1)
    k_island_epoch2(const speo_segment *__restrict__ segs, int Pmax, const float *pop_in, const float *fit_in,
                    float *pop_out, float *fit_out, uint32_t *gen_ctr, int generations)
{
    using Pl = ResPlan<Q>;
    constexpr int W = Pl::W, G = Pl::G;
    extern __shared__ __align__(16) float sm[];
    const int hmax = half_rows(Pmax), Ph = round_up(hmax, kEvalRows2), GB = draw_gens2(Pmax);
    float *const pop0 = sm;                               // pop buffer b at pop0 + b * Pmax * W
    const int Pf = round_up(Pmax, 4);                     // fit buffers padded: Xs stays 16-byte aligned
    float *const fit0 = sm + 2 * (size_t)Pmax * W;        // fit buffer b at fit0 + b * Pf
    float *Xs = fit0 + 2 * Pf;
    float *Ys = Xs + (size_t)Ph * W;
    float *Ms = Ys + (size_t)Ph * W;
    int *sR = reinterpret_cast<int *>(Ms + W * W);
    float *sF = reinterpret_cast<float *>(sR + GB * hmax * 8);
    float *so = sF + Ph;
    __shared__ float s_bf[kWarpsR];
    __shared__ int s_bi[kWarpsR];

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int grp = tid / G, gl = tid % G;
    const uint32_t me = cluster_rank(), peer = me ^ 1u;
    const speo_segment &s = segs[blockIdx.x >> 1];
    const int D = s.dim, P = s.pop_size, ld = s.ld, nch = (D + 3) >> 2;
    const uint32_t gen0 = *(volatile uint32_t *)gen_ctr;
    // both blocks of a cluster read the same segment, so they take the same branch and pass the
    // same number of cluster barriers
    const bool seg_ok = P >= 2 && P <= Pmax && D >= 1 && D <= W && (ld & 3) == 0 && ld >= D && func_supported(s.func_id);
    if (seg_ok) {
        const long long row0 = s.row0;
        const uint2 key = seed_key(s.seed);
        const int st = s.strategy, ndon = donors_for(st);
        const float F = s.F, CR = s.CR, lb = s.lb, ub = s.ub;
        const float scale = func_scale(s.func_id);
        const int h = half_rows(P);
        const int rb = (int)me * h, nr = (P - rb < h ? P - rb : h);  // this block's rows [rb, rb + nr)

        for (int i = tid; i < P * nch; i += kThreads) {
            const int r = i / nch, c = i - r * nch;
            st4s(pop0 + r * W + 4 * c, *reinterpret_cast<const float4 *>(pop_in + (row0 + r) * ld + 4 * c));
        }
        for (int r = tid; r < P; r += kThreads) fit0[r] = fit_in[row0 + r];
        load_rot_rows<float, Q>(Ms, s.rot, s.ld_rot, D, 0, D);
        for (int k = tid; k < W; k += kThreads) so[k] = k < 4 * nch ? s.shift[k] : 0.f;
        for (int i = tid; i < Ph * W; i += kThreads) Ys[i] = 0.f;
        const uint32_t peer_pop0 = map_peer(pop0, peer), peer_fit0 = map_peer(fit0, peer);
        cluster_sync();

        bool ok_draw = true, ok_bound = true;
        for (int g = 0; g < generations; ++g) {
            const uint32_t gen = gen0 + (uint32_t)g;
            const int cur = g & 1, nxt = cur ^ 1;
            const float *pop = pop0 + (size_t)cur * Pmax * W;
            const float *fit = fit0 + cur * Pf;
            int best = -1;
            if (strategy_uses_best(st)) {
                float bf = __int_as_float(0x7f800000);
                int bi = 0x7fffffff;
                for (int r = tid; r < P; r += kThreads) {
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
                for (int w = 1; w < kWarpsR; ++w)
                    if (s_bf[w] < bf || (s_bf[w] == bf && s_bi[w] < bi)) { bf = s_bf[w]; bi = s_bi[w]; }
                best = bi;
            }
            // (1) donor positions + jrand of this block's rows for generations g .. g + GB - 1
            if (g % GB == 0) {
                const int nb = generations - g < GB ? generations - g : GB;
                for (int t = tid; t < nb * nr; t += kThreads) {
                    const int gi = t / nr, lr = t - gi * nr;
                    IdxStream is(key, (uint32_t)(row0 + rb + lr), gen + (uint32_t)gi, kTagIdx);
                    int rr[5];
                    ok_draw &= draw_donors(is, P, rr);
                    int *o = sR + (gi * hmax + lr) * 8;
#pragma unroll
                    for (int k = 0; k < 5; ++k) o[k] = rr[k];
                    o[5] = is.index(D);
                }
                __syncthreads();
            }
            const int *sRg = sR + (g % GB) * hmax * 8;
            float *npop = pop0 + (size_t)nxt * Pmax * W;
            float *nfit = fit0 + nxt * Pf;
            const uint32_t ppop = peer_pop0 + (uint32_t)(nxt * Pmax * W * sizeof(float));
            const uint32_t pfit = peer_fit0 + (uint32_t)(nxt * Pf * sizeof(float));
            // (2)-(4) per warp, for its kRowsPerWarp2 rows of each 64-row pass: trials, evaluation,
            // greedy selection (strict `<`, kernel_DE_CUDA.cu:312) into the next buffer of both
            // replicas. A row's trial, fitness and selection stay in its warp: no block barrier.
            for (int pb = 0; pb < nr; pb += kEvalRows2) {
                const int lr0 = pb + warp * kRowsPerWarp2;
                if (lr0 >= nr) break;  // warp-uniform
                const int nrw = nr - lr0 < kRowsPerWarp2 ? nr - lr0 : kRowsPerWarp2;
                for (int t = lane; t < nrw * nch; t += 32) {
                    const int lr = lr0 + t / nch, c = t % nch, r = rb + lr;
                    const int jrand = sRg[lr * 8 + 5];
                    int dr[5];
#pragma unroll
                    for (int k = 0; k < 5; ++k) dr[k] = sRg[lr * 8 + k];
                    const float *xi = pop + r * W;
                    const float *xb = pop + (best >= 0 ? best : r) * W;
                    const int e0 = 4 * c;
                    const float4 ti = ld4s(xi + e0);
                    const float4 tb = best >= 0 ? ld4s(xb + e0) : ti;
                    float4 tr[5];
#pragma unroll
                    for (int k = 0; k < 5; ++k) tr[k] = k < ndon ? ld4s(pop + dr[k] * W + e0) : ti;
                    const uint4 w = philox(make_uint4((uint32_t)c, (uint32_t)(row0 + r), gen, kTagCr), key);
                    const float4 o4 = ld4s(so + e0);
                    float4 x4 = make_float4(0.f, 0.f, 0.f, 0.f), y4 = x4;
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        const int e = e0 + q;
                        if (e < D) {
                            const float u = u01(pick(w, (uint32_t)q));
                            float x;
                            if (e == jrand || u < CR) {
                                float xr[5];
#pragma unroll
                                for (int k = 0; k < 5; ++k) xr[k] = f4g(tr[k], q);
                                x = mutant<float>(st, F, f4g(ti, q), f4g(tb, q), xr);
                            } else {
                                x = f4g(ti, q);
                            }
                            x = check_bound<float>(x, lb, ub, ok_bound);
                            f4s(x4, q, x);
                            f4s(y4, q, __fsub_rn(x, f4g(o4, q)));
                        }
                    }
                    st4s(Xs + lr * W + e0, x4);
                    st4s(Ys + lr * W + e0, y4);
                }
                __syncwarp();
                float acc[kRowsPerWarp2][Q];
#pragma unroll
                for (int rr = 0; rr < kRowsPerWarp2; ++rr)
#pragma unroll
                    for (int q = 0; q < Q; ++q) acc[rr][q] = 0.f;
                if (func_rotated(s.func_id))
                    eval_accumulate<float, Q>(acc, Ys, W, lr0, Ms, W, 0, D, lane);
                else
                    eval_identity<float, Q>(acc, Ys, W, lr0, D, lane);
                float f[kRowsPerWarp2];
                eval_reduce<float, Q>(acc, D, s.func_id, scale, lane, f);
                if (lane == 0)
#pragma unroll
                    for (int rr = 0; rr < kRowsPerWarp2; ++rr) sF[lr0 + rr] = f[rr];
                __syncwarp();
                for (int t = lane; t < nrw * nch; t += 32) {
                    const int lr = lr0 + t / nch, c = t % nch, r = rb + lr;
                    const float tf = sF[lr];
                    const bool win = tf < fit[r];
                    const float4 v = ld4s((win ? Xs + lr * W : pop + r * W) + 4 * c);
                    st4s(npop + r * W + 4 * c, v);
                    st_peer4(ppop + (uint32_t)((r * W + 4 * c) * sizeof(float)), v);
                    if (c == 0) {
                        const float nf = win ? tf : fit[r];
                        nfit[r] = nf;
                        st_peer1(pfit + (uint32_t)(r * sizeof(float)), nf);
                    }
                }
            }
            cluster_sync();
        }
        if (!ok_draw) atomicOr(&s_deverr, SPEO_DEVERR_REDRAW_LIMIT);
        if (!ok_bound) atomicOr(&s_deverr, SPEO_DEVERR_BOUND_LIMIT);
        // ---- write this block's rows back --------------------------------------------------------
        const float *pop = pop0 + (size_t)(generations & 1) * Pmax * W;
        const float *fit = fit0 + (generations & 1) * Pf;
        for (int i = tid; i < nr * nch; i += kThreads) {
            const int lr = i / nch, c = i - lr * nch, r = rb + lr;
            *reinterpret_cast<float4 *>(pop_out + (row0 + r) * ld + 4 * c) = ld4s(pop + r * W + 4 * c);
        }
        for (int lr = tid; lr < nr; lr += kThreads) fit_out[row0 + rb + lr] = fit[rb + lr];
    } else if (tid == 0) {
        atomicOr(&s_deverr, SPEO_DEVERR_BAD_SEGMENT);
    }
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

int max_optin()
{
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    return v;
}

}  // namespace
}  // namespace speo

using namespace speo;

extern "C" int speo_epoch_fits(int max_pop, int dim_hi)
{
    if (max_pop < 2 || max_pop > kMaxPop || dim_hi < 1 || dim_hi > 64) return 0;
    const int Q = dim_hi <= 32 ? 1 : 2;
    return res_smem_floats(Q, max_pop) * sizeof(float) <= (size_t)max_optin() ? 1 : 0;
}

extern "C" int speo_generation_epoch_ex(const speo_segment *segs, int n_segs, int dim_lo, int dim_hi, int max_pop,
                                        const float *pop_in, const float *fit_in, float *pop_out, float *fit_out,
                                        uint32_t *d_gen, int generations, int cluster, void *stream)
{
    if (cluster < 0 || cluster > 2) return fail(SPEO_ERR_INVALID_ARG, "speo_generation_epoch_ex: cluster %d", cluster);
    if (!segs || !pop_in || !fit_in || !pop_out || !fit_out || !d_gen || n_segs < 1 || generations < 1)
        return fail(SPEO_ERR_INVALID_ARG, "speo_generation_epoch: bad arguments");
    if (dim_lo < 1 || dim_lo > dim_hi) return fail(SPEO_ERR_INVALID_ARG, "speo_generation_epoch: dim range");
    if (!speo_epoch_fits(max_pop, dim_hi))
        return fail(SPEO_ERR_UNSUPPORTED,
                    "speo_generation_epoch: islands of P <= %d, D <= %d do not fit one block's shared memory",
                    max_pop, dim_hi);
    const int Q = dim_hi <= 32 ? 1 : 2;
    if (dim_lo <= 32 && Q == 2)
        return fail(SPEO_ERR_UNSUPPORTED, "speo_generation_epoch: segments must share one column class");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t e;
    // two-block clusters when there are SMs for two blocks per island
    const size_t smem2 = res2_smem_floats(Q, max_pop) * sizeof(float);
    const bool pair = cluster != 1 && (cluster == 2 || 2LL * n_segs <= sm_count()) && smem2 <= (size_t)max_optin();
    if (cluster == 2 && !pair)
        return fail(SPEO_ERR_UNSUPPORTED, "speo_generation_epoch_ex: two-block islands need %zu B of shared memory", smem2);
    if (pair) {
        if (Q == 1) {
            e = cudaFuncSetAttribute(k_island_epoch2<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem2);
            if (e != cudaSuccess) return check_cuda(e, "cudaFuncSetAttribute(k_island_epoch2)");
            k_island_epoch2<1><<<2 * n_segs, kThreads, smem2, st>>>(segs, max_pop, pop_in, fit_in, pop_out, fit_out,
                                                                     d_gen, generations);
        } else {
            e = cudaFuncSetAttribute(k_island_epoch2<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem2);
            if (e != cudaSuccess) return check_cuda(e, "cudaFuncSetAttribute(k_island_epoch2)");
            k_island_epoch2<2><<<2 * n_segs, kThreads, smem2, st>>>(segs, max_pop, pop_in, fit_in, pop_out, fit_out,
                                                                     d_gen, generations);
        }
        return check_launch("k_island_epoch2");
    }
    const size_t smem = res_smem_floats(Q, max_pop) * sizeof(float);
    if (Q == 1) {
        e = cudaFuncSetAttribute(k_island_epoch<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return check_cuda(e, "cudaFuncSetAttribute(k_island_epoch)");
        k_island_epoch<1><<<n_segs, kThreads, smem, st>>>(segs, max_pop, pop_in, fit_in, pop_out, fit_out, d_gen,
                                                          generations);
    } else {
        e = cudaFuncSetAttribute(k_island_epoch<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return check_cuda(e, "cudaFuncSetAttribute(k_island_epoch)");
        k_island_epoch<2><<<n_segs, kThreads, smem, st>>>(segs, max_pop, pop_in, fit_in, pop_out, fit_out, d_gen,
                                                          generations);
    }
    return check_launch("k_island_epoch");
}

extern "C" int speo_generation_epoch(const speo_segment *segs, int n_segs, int dim_lo, int dim_hi, int max_pop,
                                     const float *pop_in, const float *fit_in, float *pop_out, float *fit_out,
                                     uint32_t *d_gen, int generations, void *stream)
{
    return speo_generation_epoch_ex(segs, n_segs, dim_lo, dim_hi, max_pop, pop_in, fit_in, pop_out, fit_out, d_gen,
                                    generations, 0, stream);
}
