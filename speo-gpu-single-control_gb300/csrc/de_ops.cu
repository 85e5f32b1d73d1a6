// de_ops.cu -- the reference-shaped DE operator entry points (group 1 of speo_gb300.h):
// population initialisation, best-in-sub-island search, DE mutation + binomial crossover +
// reflection, and greedy selection, for `real` = float and `real` = double.
//
// Reference kernels restated: CUDA_EA_library/kernel_EA_CUDA.cu:85-134 (init),
// CUDA_EA_library/kernel_DE_CUDA.cu:120-338 (best, generate, select).
// Layout: rows of `np2` = max(32, next_pow2(dim)) elements (EA_CUDA.cc:197-206); one warp
// per target row, lanes over elements, draws from Philox instead of per-lane XORWOW states.
#include <cmath>

#include "common.cuh"
#include "host.h"

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

template <typename T> struct DeInfoT;
template <> struct DeInfoT<float> { using type = speo_de_info_f32; };
template <> struct DeInfoT<double> { using type = speo_de_info_f64; };

// Advances the generation counter once every block of this launch has read it.
__device__ __forceinline__ void finish_launch(RngState *rng, uint32_t gen)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned t = atomicAdd(&rng->done, 1u);
        if (t == gridDim.x - 1) {
            rng->done = 0;
            rng->gen = gen + 1;
            __threadfence();
        }
    }
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
__device__ __forceinline__ T rank_t(T f) { return isnan(f) ? T(INFINITY) : f; }

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

// global_DE_GenerateNewPopulation (kernel_DE_CUDA.cu:172-289): one warp per position.
template <typename T>
__global__ void __launch_bounds__(256) k_generate(T *cand, const T *pop, int ld, int dim, int island_size, int S,
                                                  const int *perm, const typename DeInfoT<T>::type *info,
                                                  const int *best_id, T lb, T ub, RngState *rng)
{
    const uint32_t gen = *(volatile uint32_t *)&rng->gen;
    const uint2 key = make_uint2(rng->key0, rng->key1);
    const int pos = blockIdx.x * kWarps + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (pos < island_size) {
        const int sel = perm[pos];
        const int isl = pos / S;
        IdxStream s(key, (uint32_t)pos, gen, kTagIdx);
        int r[5];
        const bool ok_draw = draw_donors(s, S, r);
        bool ok_bound = true;
#pragma unroll
        for (int i = 0; i < 5; ++i) r[i] = perm[r[i] + isl * S];
        const int jrand = s.index(dim);
        const T F = info[isl].F, CR = info[isl].CR;
        const int st = info[isl].strategy_ID;
        const int b = strategy_uses_best(st) ? best_id[isl] : sel;
        const T *xi = pop + (size_t)sel * ld;
        const T *xb = pop + (size_t)b * ld;
        for (int e = lane; e < dim; e += 32) {
            const uint4 w = philox(make_uint4((uint32_t)(e >> 2), (uint32_t)pos, gen, kTagCr), key);
            const float u = u01(pick(w, (uint32_t)(e & 3)));
            T v;
            if (e == jrand || (T)u < CR) {
                T xr[5];
#pragma unroll
                for (int i = 0; i < 5; ++i) xr[i] = pop[(size_t)r[i] * ld + e];
                v = mutant<T>(st, F, xi[e], xb[e], xr);
            } else {
                v = xi[e];
            }
            v = check_bound<T>(v, lb, ub, ok_bound);
            cand[(size_t)sel * ld + e] = v;
        }
        if (!ok_draw && lane == 0) atomicOr(&s_deverr, SPEO_DEVERR_REDRAW_LIMIT);
        if (!ok_bound) atomicOr(&s_deverr, SPEO_DEVERR_BOUND_LIMIT);
    }
    finish_launch(rng, gen);
}

// global_DE_SelectSurvival (kernel_DE_CUDA.cu:305-327): strict `<`, one warp per row.
template <typename T>
__global__ void k_select(T *pop, T *pop_fit, const T *cand, const T *cand_fit, int n, int ld, int dim)
{
    const int i = blockIdx.x * kWarps + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (i >= n) return;
    const T fc = cand_fit[i];
    if (fc < pop_fit[i]) {
        for (int e = lane; e < dim; e += 32) pop[(size_t)i * ld + e] = cand[(size_t)i * ld + e];
        if (lane == 0) pop_fit[i] = fc;
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

template <typename T, typename Pop, typename Info, typename Prob>
int generate(Pop cand, Pop pop, int *d_best, speo_island_info ii, Info *d_info, speo_rng_state *d_rng, Prob pi)
{
    if (int st = validate<T>(pop.elements, ii, pi.dim, "API_DE_GenerateNewPopulation")) return st;
    if (!cand.elements || !pop.fitness_value || !ii.permutated_index || !d_info || !d_rng || !d_best)
        return fail(SPEO_ERR_INVALID_ARG, "API_DE_GenerateNewPopulation: null pointer argument");
    const int S = ii.island_size / ii.subisland_num;
    if (S < 2) return fail(SPEO_ERR_INVALID_ARG, "API_DE_GenerateNewPopulation: sub-island size %d < 2", S);
    const int ld = np2_of(pi.dim);
    cudaStream_t st = api_stream();
    k_best<T><<<(ii.subisland_num + kWarps - 1) / kWarps, 32 * kWarps, 0, st>>>(
        pop.fitness_value, ii.permutated_index, S, ii.subisland_num, d_best);
    if (int e = check_launch("global_DE_FindBestIndividualInIsland")) return e;
    k_generate<T><<<(ii.island_size + kWarps - 1) / kWarps, 32 * kWarps, 0, st>>>(
        cand.elements, pop.elements, ld, pi.dim, ii.island_size, S, ii.permutated_index,
        reinterpret_cast<const typename DeInfoT<T>::type *>(d_info), d_best, (T)pi.min_bound, (T)pi.max_bound,
        reinterpret_cast<RngState *>(d_rng));
    return check_launch("global_DE_GenerateNewPopulation");
}

template <typename T, typename Pop, typename Prob>
int select(Pop pop, Pop cand, speo_island_info ii, Prob pi)
{
    if (int st = validate<T>(pop.elements, ii, pi.dim, "API_DE_SelectSurvival")) return st;
    if (!cand.elements || !pop.fitness_value || !cand.fitness_value)
        return fail(SPEO_ERR_INVALID_ARG, "API_DE_SelectSurvival: null pointer argument");
    const int ld = np2_of(pi.dim);
    k_select<T><<<(ii.island_size + kWarps - 1) / kWarps, 32 * kWarps, 0, api_stream()>>>(
        pop.elements, pop.fitness_value, cand.elements, cand.fitness_value, ii.island_size, ld, pi.dim);
    return check_launch("global_DE_SelectSurvival");
}

}  // namespace
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
