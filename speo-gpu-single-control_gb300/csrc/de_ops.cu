// de_ops.cu -- the reference-shaped DE operator entry points (group 1 of speo_gb300.h):
// population initialisation, best-in-sub-island search, DE mutation + binomial crossover +
// reflection, and greedy selection, for `real` = float and `real` = double.
//
// Reference kernels restated: CUDA_EA_library/kernel_EA_CUDA.cu:85-134 (init),
// CUDA_EA_library/kernel_DE_CUDA.cu:120-338 (best, generate, select).
// Layout: rows of `np2` = max(32, next_pow2(dim)) elements (EA_CUDA.cc:197-206); one warp
// per target row, lanes over elements, draws from Philox instead of per-lane XORWOW states.
#include <cmath>

#include "dropin.cuh"

SPEO_DEFINE_DEVERR(speo_deverr_de_ops)

namespace speo {
namespace {

constexpr int kWarps = 8;  // targets per 256-thread block

int np2_of(int dim)
{
    int y = 1;
    while (y < dim) y <<= 1;
    return y < 32 ? 32 : y;
}

// global_SetupRandomState + global_InitiPopulation (kernel_EA_CUDA.cu:85-118): one thread per
// (row, group of 4 elements); x = lb + u*(ub - lb).
template <typename T>
__global__ void k_init(T *elems, int n, int ld, int dim, T lb, T ub, uint2 key, RngState *rng)
{
    const int groups = (dim + 3) >> 2;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (rng && t == 0) {
        rng->key0 = key.x;
        rng->key1 = key.y;
        rng->gen = 0;
        rng->done = 0;
    }
    if (t >= (long long)n * groups) return;
    const int row = (int)(t / groups), g = (int)(t % groups);
    const uint4 w = philox(make_uint4((uint32_t)g, (uint32_t)row, 0u, kTagInit), key);
    const T range = ub - lb;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int e = 4 * g + q;
        if (e < dim) elems[(size_t)row * ld + e] = fma_rn((T)u01(pick(w, q)), range, lb);
    }
}

// global_DE_FindBestIndividualInIsland (kernel_DE_CUDA.cu:120-158), one warp per sub-island,
// positions s*S .. s*S+S-1 (the reference reads the first sub-island's positions for all s).
template <typename T>
__global__ void k_best(const T *fit, const int *perm, int S, int nsub, int *best_id)
{
    const int s = blockIdx.x * kWarps + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (s >= nsub) return;
    T bf = T(INFINITY);
    int bp = 0x7fffffff;
    for (int i = lane; i < S; i += 32) {
        const T f = rank_t(fit[perm[s * S + i]]);
        if (f < bf || (f == bf && i < bp)) { bf = f; bp = i; }
    }
    for (int o = 16; o > 0; o >>= 1) {
        const T of = __shfl_xor_sync(0xffffffffu, bf, o);
        const int op = __shfl_xor_sync(0xffffffffu, bp, o);
        if (of < bf || (of == bf && op < bp)) { bf = of; bp = op; }
    }
    if (lane == 0) best_id[s] = perm[s * S + bp];
}

// The same search for large sub-islands: one 512-thread block per sub-island. The (fitness,
// position) minimum is order-independent, so the result equals the warp version's.
template <typename T>
__global__ void __launch_bounds__(512) k_best_block(const T *fit, const int *perm, int S, int *best_id)
{
    __shared__ T wf[16];
    __shared__ int wp[16];
    const int s = blockIdx.x, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    T bf = T(INFINITY);
    int bp = 0x7fffffff;
    for (int i = threadIdx.x; i < S; i += blockDim.x) {
        const T f = rank_t(fit[perm[(size_t)s * S + i]]);
        if (f < bf || (f == bf && i < bp)) { bf = f; bp = i; }
    }
    for (int o = 16; o > 0; o >>= 1) {
        const T of = __shfl_xor_sync(0xffffffffu, bf, o);
        const int op = __shfl_xor_sync(0xffffffffu, bp, o);
        if (of < bf || (of == bf && op < bp)) { bf = of; bp = op; }
    }
    if (lane == 0) { wf[warp] = bf; wp[warp] = bp; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w)
            if (wf[w] < bf || (wf[w] == bf && wp[w] < bp)) { bf = wf[w]; bp = wp[w]; }
        best_id[s] = perm[(size_t)s * S + bp];
    }
}

// global_DE_GenerateNewPopulation (kernel_DE_CUDA.cu:172-289).
// One warp owns ppw (1 .. 32) consecutive positions: lane l < ppw draws the donors and jrand of
// position l (Philox on those lanes at once). The warp's ppw x nch (row, 16-byte chunk) tasks are
// then dealt to the lanes in order, task t = it * 32 + lane, so no lane idles whatever D is; each
// task reads its row's draws from the drawing lane with shuffles. Two tasks in flight per lane.
// Small populations take small ppw so that enough warps cover the GPU.
template <typename T>
__global__ void __launch_bounds__(256) k_generate(T *cand, const T *pop, int ld, int dim, int island_size, int S,
                                                  const int *perm, const typename DeInfoT<T>::type *info,
                                                  const int *best_id, T lb, T ub, RngState *rng, int ppw)
{
    using V = typename Vec<T>::type;
    constexpr int VN = Vec<T>::n;
    const uint32_t gen = *(volatile uint32_t *)&rng->gen;
    const uint2 key = make_uint2(rng->key0, rng->key1);
    const int lane = threadIdx.x & 31;
    const int wbase = (blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * ppw;
    // ---- draws of position wbase + lane ------------------------------------------------------
    int d0 = 0, d1 = 0, d2 = 0, d3 = 0, d4 = 0, jr = 0, sel = 0, isl = 0;
    {
        const int pos = wbase + lane;
        if (lane < ppw && pos < island_size) {
            isl = pos / S;
            IdxStream s(key, (uint32_t)pos, gen, kTagIdx);
            int r[5];
            if (!draw_donors(s, S, r)) atomicOr(&s_deverr, SPEO_DEVERR_REDRAW_LIMIT);
            d0 = perm[r[0] + isl * S]; d1 = perm[r[1] + isl * S]; d2 = perm[r[2] + isl * S];
            d3 = perm[r[3] + isl * S]; d4 = perm[r[4] + isl * S];
            jr = s.index(dim);
            sel = perm[pos];
        }
    }
    const int nch = (dim + VN - 1) / VN;
    const int q32 = 32 / nch, r32 = 32 % nch;  // task t -> t + 32 advances (row, chunk) by these
    int src = lane / nch, c = lane - src * nch;
    const int iters = (ppw * nch + 31) / 32;   // uniform trip count
    bool ok_bound = true;
#pragma unroll 2
    for (int it = 0; it < iters; ++it) {
        const int s_lane = src < 32 ? src : 31;
        const int pos = wbase + src;
        const int rsel = __shfl_sync(0xffffffffu, sel, s_lane), risl = __shfl_sync(0xffffffffu, isl, s_lane);
        const int rjr = __shfl_sync(0xffffffffu, jr, s_lane);
        const int rd[5] = {__shfl_sync(0xffffffffu, d0, s_lane), __shfl_sync(0xffffffffu, d1, s_lane),
                           __shfl_sync(0xffffffffu, d2, s_lane), __shfl_sync(0xffffffffu, d3, s_lane),
                           __shfl_sync(0xffffffffu, d4, s_lane)};
        const int e0 = VN * c;
        const bool live = src < ppw && pos < island_size;
        src += q32;
        c += r32;
        if (c >= nch) { c -= nch; ++src; }
        if (!live) continue;
        const T F = info[risl].F;
        const uint32_t thr = cr_threshold<T>(info[risl].CR);
        const int st = info[risl].strategy_ID;
        const int nd = ndonors(st);
        const int b = strategy_uses_best(st) ? best_id[risl] : rsel;
        const T *xi = pop + (size_t)rsel * ld;
        const T *xb = pop + (size_t)b * ld;
        T *out = cand + (size_t)rsel * ld;
        const V ti = *reinterpret_cast<const V *>(xi + e0);
        const V tb = strategy_uses_best(st) ? *reinterpret_cast<const V *>(xb + e0) : ti;
        V tr[5];
#pragma unroll
        for (int k = 0; k < 5; ++k)
            tr[k] = k < nd ? *reinterpret_cast<const V *>(pop + (size_t)rd[k] * ld + e0) : ti;
        const uint4 w = philox(make_uint4((uint32_t)(e0 >> 2), (uint32_t)pos, gen, kTagCr), key);
        V o = ti;
        if (st == SPEO_DE_RAND_1) {  // rand/1, the default strategy (DE_CUDA.cc:63): no switch
#pragma unroll
            for (int q = 0; q < VN; ++q) {
                const int e = e0 + q;
                T v = vget<T>(ti, q);
                if (e == rjr || cr_take(pick(w, (uint32_t)(e & 3)), thr))
                    v = fma_rn(F, sub_rn(vget<T>(tr[1], q), vget<T>(tr[2], q)), vget<T>(tr[0], q));
                vset<T>(o, q, check_bound<T>(v, lb, ub, ok_bound));
            }
        } else {
#pragma unroll
            for (int q = 0; q < VN; ++q) {
                const int e = e0 + q;
                T v;
                if (e == rjr || cr_take(pick(w, (uint32_t)(e & 3)), thr)) {
                    T xr[5];
#pragma unroll
                    for (int k = 0; k < 5; ++k) xr[k] = vget<T>(tr[k], q);
                    v = mutant<T>(st, F, vget<T>(ti, q), vget<T>(tb, q), xr);
                } else {
                    v = vget<T>(ti, q);
                }
                vset<T>(o, q, check_bound<T>(v, lb, ub, ok_bound));
            }
        }
        if (e0 + VN <= dim) {
            *reinterpret_cast<V *>(out + e0) = o;
        } else {  // ragged last chunk: elements past D are never written (as in the reference)
#pragma unroll
            for (int q = 0; q < VN; ++q)
                if (e0 + q < dim) out[e0 + q] = vget<T>(o, q);
        }
    }
    if (!ok_bound) atomicOr(&s_deverr, SPEO_DEVERR_BOUND_LIMIT);
    finish_launch(rng, gen);
}

// global_DE_SelectSurvival (kernel_DE_CUDA.cu:305-327): strict `<`. One warp per group of 32
// rows: a coalesced compare of the two fitness arrays (the next group's pair is loaded before the
// current group's rows move), a ballot, then the winners' (row, chunk) copies dealt round-robin to
// all 32 lanes, kTasks per lane at a time with every load issued before the first store (bytes in
// flight, not instruction count, bound a sparse row copy; a chunk per lane per row would leave 7
// of 32 lanes idle at D = 100). Rows whose trial loses move no data.
template <typename T>
__global__ void __launch_bounds__(256) k_select(T *pop, T *pop_fit, const T *cand, const T *cand_fit, int n, int ld,
                                                int dim)
{
    using V = typename Vec<T>::type;
    constexpr int VN = Vec<T>::n, kTasks = 8;
    __shared__ int s_rows[8][32];  // the winners of each warp's current group, in lane order
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int nch = (dim + VN - 1) / VN, full_ch = dim / VN;
    const long long groups = ((long long)n + 31) / 32;
    const long long nwarps = (long long)gridDim.x * (blockDim.x >> 5);
    long long g = (long long)blockIdx.x * (blockDim.x >> 5) + wib;
    T fc = T(0), fp = T(0);
    if (g < groups && g * 32 + lane < n) {
        fc = cand_fit[g * 32 + lane];
        fp = pop_fit[g * 32 + lane];
    }
    for (; g < groups; g += nwarps) {
        const long long row = g * 32 + lane;
        const bool win = row < n && fc < fp;
        if (win) pop_fit[row] = fc;
        const long long gn = g + nwarps, rn = gn * 32 + lane;
        if (gn < groups && rn < n) {
            fc = cand_fit[rn];
            fp = pop_fit[rn];
        }
        const unsigned m = __ballot_sync(0xffffffffu, win);
        if (win) s_rows[wib][__popc(m & ((1u << lane) - 1u))] = (int)row;
        __syncwarp();
        const int tasks = __popc(m) * nch;
        for (int t0 = 0; t0 < tasks; t0 += 32 * kTasks) {
            V v[kTasks];
#pragma unroll
            for (int k = 0; k < kTasks; ++k) {
                const int t = t0 + 32 * k + lane;
                if (t < tasks) {
                    const int q = t / nch, c = t - q * nch;
                    if (c < full_ch) v[k] = *reinterpret_cast<const V *>(cand + (size_t)s_rows[wib][q] * ld + VN * c);
                }
            }
#pragma unroll
            for (int k = 0; k < kTasks; ++k) {
                const int t = t0 + 32 * k + lane;
                if (t < tasks) {
                    const int q = t / nch, c = t - q * nch;
                    const size_t base = (size_t)s_rows[wib][q] * ld;
                    if (c < full_ch) {
                        *reinterpret_cast<V *>(pop + base + VN * c) = v[k];
                    } else {  // ragged last chunk: elements past D are never written
                        for (int e = VN * c; e < dim; ++e) pop[base + e] = cand[base + e];
                    }
                }
            }
        }
        __syncwarp();
    }
}

template <typename T>
int validate(const T *elems, const speo_island_info &ii, int dim, const char *who)
{
    if (!elems) return fail(SPEO_ERR_INVALID_ARG, "%s: null population", who);
    if (ii.island_size <= 0 || ii.subisland_num <= 0)
        return fail(SPEO_ERR_INVALID_ARG, "%s: island_size %d, subisland_num %d", who, ii.island_size, ii.subisland_num);
    if (ii.island_size % ii.subisland_num)
        return fail(SPEO_ERR_INVALID_ARG, "%s: island_size %d not divisible by subisland_num %d", who,
                    ii.island_size, ii.subisland_num);
    if (dim < 1 || dim > SPEO_MAX_DIM) return fail(SPEO_ERR_INVALID_ARG, "%s: dim %d out of range", who, dim);
    return SPEO_OK;
}

template <typename T, typename Pop, typename Prob>
int initilize(Pop pop, speo_rng_state *d_rng, speo_island_info ii, Prob pi)
{
    if (int st = validate<T>(pop.elements, ii, pi.dim, "API_Initilize")) return st;
    const int ld = np2_of(pi.dim);
    const long long threads = (long long)ii.island_size * ((pi.dim + 3) / 4);
    const int blocks = (int)((threads + 255) / 256);
    const uint64_t seed = (uint64_t)(uint32_t)pi.seed;
    k_init<T><<<blocks, 256, 0, api_stream()>>>(pop.elements, ii.island_size, ld, pi.dim, (T)pi.min_bound,
                                                 (T)pi.max_bound, make_uint2((uint32_t)seed, (uint32_t)(seed >> 32)),
                                                 reinterpret_cast<RngState *>(d_rng));
    return check_launch("API_Initilize");
}

// with_best = false leaves d_best as it is (for callers that know no sub-island's strategy reads it
// and that the ids are refreshed before anyone reads them).
template <typename T, typename Pop, typename Info, typename Prob>
int generate(Pop cand, Pop pop, int *d_best, speo_island_info ii, Info *d_info, speo_rng_state *d_rng, Prob pi,
             bool with_best = true)
{
    if (int st = validate<T>(pop.elements, ii, pi.dim, "API_DE_GenerateNewPopulation")) return st;
    if (!cand.elements || !pop.fitness_value || !ii.permutated_index || !d_info || !d_rng || !d_best)
        return fail(SPEO_ERR_INVALID_ARG, "API_DE_GenerateNewPopulation: null pointer argument");
    const int S = ii.island_size / ii.subisland_num;
    if (S < 2) return fail(SPEO_ERR_INVALID_ARG, "API_DE_GenerateNewPopulation: sub-island size %d < 2", S);
    const int ld = np2_of(pi.dim);
    cudaStream_t st = api_stream();
    if (with_best) {
        if (S >= 1024)
            k_best_block<T><<<ii.subisland_num, 512, 0, st>>>(pop.fitness_value, ii.permutated_index, S, d_best);
        else
            k_best<T><<<(ii.subisland_num + kWarps - 1) / kWarps, 32 * kWarps, 0, st>>>(
                pop.fitness_value, ii.permutated_index, S, ii.subisland_num, d_best);
        if (int e = check_launch("global_DE_FindBestIndividualInIsland")) return e;
    }
    // 16-byte chunks cover D (np2 rows keep every chunk in bounds). Positions per warp: the
    // largest of 32, 16, 8, 4, 2, 1 that still gives about 16 warps per SM.
    int ppw = 32;
    while (ppw > 1 && (long long)ii.island_size < (long long)ppw * 16 * sm_count()) ppw >>= 1;
    const int grid = (ii.island_size + 8 * ppw - 1) / (8 * ppw);  // 8 warps per block
    const auto *inf = reinterpret_cast<const typename DeInfoT<T>::type *>(d_info);
    RngState *rs = reinterpret_cast<RngState *>(d_rng);
    k_generate<T><<<grid, 256, 0, st>>>(cand.elements, pop.elements, ld, pi.dim, ii.island_size, S,
                                        ii.permutated_index, inf, d_best, (T)pi.min_bound, (T)pi.max_bound, rs, ppw);
    return check_launch("global_DE_GenerateNewPopulation");
}

template <typename T, typename Pop, typename Prob>
int select(Pop pop, Pop cand, speo_island_info ii, Prob pi)
{
    if (int st = validate<T>(pop.elements, ii, pi.dim, "API_DE_SelectSurvival")) return st;
    if (!cand.elements || !pop.fitness_value || !cand.fitness_value)
        return fail(SPEO_ERR_INVALID_ARG, "API_DE_SelectSurvival: null pointer argument");
    const int ld = np2_of(pi.dim);
    const long long want = ((long long)ii.island_size + 32 * 8 - 1) / (32 * 8);  // 8 warps of 32 rows
    const int grid = (int)(want < 8LL * sm_count() ? want : 8LL * sm_count());
    k_select<T><<<grid, 256, 0, api_stream()>>>(
        pop.elements, pop.fitness_value, cand.elements, cand.fitness_value, ii.island_size, ld, pi.dim);
    return check_launch("global_DE_SelectSurvival");
}

}  // namespace

int dropin_generate_f32(speo_population_f32 c, speo_population_f32 p, int *b, speo_island_info ii,
                        speo_de_info_f32 *info, speo_rng_state *r, speo_problem_info_f32 pi, bool with_best)
{
    return generate<float>(c, p, b, ii, info, r, pi, with_best);
}
int dropin_generate_f64(speo_population_f64 c, speo_population_f64 p, int *b, speo_island_info ii,
                        speo_de_info_f64 *info, speo_rng_state *r, speo_problem_info_f64 pi, bool with_best)
{
    return generate<double>(c, p, b, ii, info, r, pi, with_best);
}

}  // namespace speo

using namespace speo;

extern "C" int API_Initilize(speo_population_f64 p, speo_rng_state *r, speo_island_info ii, speo_problem_info_f64 pi)
{
    return initilize<double>(p, r, ii, pi);
}
extern "C" int API_Initilize_f32(speo_population_f32 p, speo_rng_state *r, speo_island_info ii,
                                 speo_problem_info_f32 pi)
{
    return initilize<float>(p, r, ii, pi);
}
extern "C" int API_DE_GenerateNewPopulation(speo_population_f64 c, speo_population_f64 p, int *b, speo_island_info ii,
                                            speo_de_info_f64 *info, speo_rng_state *r, speo_problem_info_f64 pi)
{
    return generate<double>(c, p, b, ii, info, r, pi);
}
extern "C" int API_DE_GenerateNewPopulation_f32(speo_population_f32 c, speo_population_f32 p, int *b,
                                                speo_island_info ii, speo_de_info_f32 *info, speo_rng_state *r,
                                                speo_problem_info_f32 pi)
{
    return generate<float>(c, p, b, ii, info, r, pi);
}
extern "C" int API_DE_SelectSurvival(speo_population_f64 p, speo_population_f64 c, speo_island_info ii,
                                     speo_problem_info_f64 pi)
{
    return select<double>(p, c, ii, pi);
}
extern "C" int API_DE_SelectSurvival_f32(speo_population_f32 p, speo_population_f32 c, speo_island_info ii,
                                         speo_problem_info_f32 pi)
{
    return select<float>(p, c, ii, pi);
}
