// generation.cu -- one fused DE generation over a segment table, and the on-device ring
// migration between segments.
//
// The reference runs a generation as five launches with three device syncs
// (CUDA_EA_library/DE_CUDA.cc:200-216 -> kernel_DE_CUDA.cu:291-338 and
// kernel_CEC2014_CUDA.cu:1672-1797), writes every trial to a candidate buffer, re-reads it to
// rotate it, writes the rotated copy, re-reads it to reduce, and re-reads both to select.
// Here one kernel reads the target and its donors once (float4, coalesced), keeps the trial in
// registers and its (x - o) copy in shared memory, evaluates it on CUDA cores, and writes only
// the winner: 4 reads + 1 write of a row per individual-generation. Population buffers are
// double-buffered (pop_in -> pop_out), so donors are always the previous generation's rows as
// in the reference's candidate/population split.
//
// Migration replaces src/migrate.cc:46-136 (host MPI exchange of random individuals) with the
// ring of best-k -> neighbour's worst-k on the device.
#include <mutex>

#include "eval_simt.cuh"
#include "host.h"

SPEO_DEFINE_DEVERR(speo_deverr_generation)

namespace speo {
namespace {


__device__ __forceinline__ float4 ld4(const float *p) { return *reinterpret_cast<const float4 *>(p); }
__device__ __forceinline__ void st4(float *p, float4 v) { *reinterpret_cast<float4 *>(p) = v; }
__device__ __forceinline__ float f4get(const float4 &v, int q) { return q == 0 ? v.x : q == 1 ? v.y : q == 2 ? v.z : v.w; }
__device__ __forceinline__ void f4set(float4 &v, int q, float x)
{
    if (q == 0) v.x = x; else if (q == 1) v.y = x; else if (q == 2) v.z = x; else v.w = x;
}

// Donor rows each strategy reads (kernel_DE_CUDA.cu:243-276).
__device__ __forceinline__ int donors_needed(int st)
{
    switch (st) {
    case 0: case 2: case 6: return 2;
    case 3: case 4: case 8: return 3;
    case 1: case 7: return 4;
    default: return 5;
    }
}

// Argmin of fit over a segment (NaN as +inf, ties lowest row) by the whole block.
__device__ long long block_seg_best(const float *fit, long long row0, int P, float *sf, long long *sr)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float bf = __int_as_float(0x7f800000);
    long long br = 0x7fffffffffffffffLL;
    for (int i = threadIdx.x; i < P; i += blockDim.x) {
        const float f = rank_key(fit[row0 + i]);
        if (better(f, row0 + i, bf, br)) { bf = f; br = row0 + i; }
    }
    for (int o = 16; o > 0; o >>= 1) {
        const float of = __shfl_xor_sync(0xffffffffu, bf, o);
        const long long orr = __shfl_xor_sync(0xffffffffu, br, o);
        if (better(of, orr, bf, br)) { bf = of; br = orr; }
    }
    __syncthreads();
    if (lane == 0) { sf[warp] = bf; sr[warp] = br; }
    __syncthreads();
    if (threadIdx.x == 0)
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w)
            if (better(sf[w], sr[w], sf[0], sr[0])) { sf[0] = sf[w]; sr[0] = sr[w]; }
    __syncthreads();
    return sr[0];
}

struct GenArgs {
    const speo_segment *segs;
    const speo_work_item *items;
    int n_items;
    const float *pop_in, *fit_in;
    float *pop_out, *fit_out;
    uint32_t *gen_ctr;
    float *trial_out, *trial_fit_out;
};

__host__ __device__ __forceinline__ int q_class(int D) { return D <= 32 ? 1 : D <= 64 ? 2 : D <= 128 ? 4 : 8; }

// Shared-memory plan of one block for column class Q (W = 32Q columns):
//   Ys[64][W]  (x - o) of the trials      Xs[64][W]  the trials
//   Ms[KC][W]  rows of M^T                sR[64][8]  donor positions + jrand
//   sPF[64]    parent fitness             sF[64]     trial fitness
template <int Q> struct GenPlan {
    static constexpr int W = 32 * Q;
    static constexpr int KC = Q <= 2 ? 32 * Q : 32;                 // M^T rows staged at once
    static constexpr int G = Q == 1 ? 8 : Q == 2 ? 16 : 32;          // lanes per row (float4 chunks)
    static constexpr int CPL = Q == 8 ? 2 : 1;                       // chunks per lane
    static constexpr int RPP = 256 / G;                              // rows per pass of the block
    static constexpr int NPASS = kEvalTile / RPP;
    static constexpr size_t floats = (size_t)2 * kEvalTile * W + (size_t)KC * W + kEvalTile * 8 + 2 * kEvalTile;
    static constexpr size_t bytes = floats * sizeof(float);
};

// One tile: (1) donor indices per row, (2) trials, (3) evaluation, (4) greedy selection.
template <int Q>
__device__ __forceinline__ void gen_tile(const GenArgs &a, const speo_work_item &it, const speo_segment &s,
                                         uint32_t gen, float *smem, float *s_bf, long long *s_br)
{
    using Pl = GenPlan<Q>;
    constexpr int W = Pl::W, G = Pl::G;
    float *Ys = smem;
    float *Xs = Ys + kEvalTile * W;
    float *Ms = Xs + kEvalTile * W;
    int *sR = reinterpret_cast<int *>(Ms + Pl::KC * W);
    float *sPF = reinterpret_cast<float *>(sR + kEvalTile * 8);
    float *sF = sPF + kEvalTile;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int grp = tid / G, gl = tid % G;
    const float *__restrict__ pop_in = a.pop_in;

    const int D = s.dim, P = s.pop_size, ld = s.ld, count = it.count;
    const long long row0 = s.row0 + it.first;
    const uint2 key = seed_key(s.seed);
    const int st = s.strategy;
    const float F = s.F, CR = s.CR, lb = s.lb, ub = s.ub;
    const int nch = (D + 3) >> 2;
    const int ndon = donors_needed(st);

    __syncthreads();  // the previous tile is done with the shared buffers
    const long long best_row = strategy_uses_best(st) ? block_seg_best(a.fit_in, s.row0, P, s_bf, s_br) : -1;

    // ---- (1) donor positions and jrand, one thread per row; the rest stage M^T --------------
    if (tid < count) {
        IdxStream is(key, (uint32_t)(row0 + tid), gen, kTagIdx);
        int r[5];
        if (!draw_donors(is, P, r)) atomicOr(&s_deverr, SPEO_DEVERR_REDRAW_LIMIT);
#pragma unroll
        for (int k = 0; k < 5; ++k) sR[tid * 8 + k] = r[k];
        sR[tid * 8 + 5] = is.index(D);
        sPF[tid] = a.fit_in[row0 + tid];
    }
    load_rot_rows<float, Q>(Ms, s.rot, s.ld_rot, D, 0, min(D, Pl::KC));
    __syncthreads();

    // ---- (2) trials: G lanes per row, float4 chunks -----------------------------------------
    bool ok_bound = true;
#pragma unroll 2
    for (int p = 0; p < Pl::NPASS; ++p) {
        const int lr = p * Pl::RPP + grp;
        float *yrow = Ys + lr * W;
        float *xrow = Xs + lr * W;
        if (lr < count) {
            const long long row = row0 + lr;
            int r[5];
#pragma unroll
            for (int k = 0; k < 5; ++k) r[k] = sR[lr * 8 + k];
            const int jrand = sR[lr * 8 + 5];
            const float *xi = pop_in + row * ld;
            const float *xb = pop_in + (best_row >= 0 ? best_row : row) * ld;
#pragma unroll
            for (int v = 0; v < Pl::CPL; ++v) {
                const int c = gl + G * v;
                if (c >= nch) continue;
                const int e0 = 4 * c;
                const float4 ti = ld4(xi + e0);
                const float4 tb = best_row >= 0 ? ld4(xb + e0) : ti;
                float4 tr[5];
#pragma unroll
                for (int k = 0; k < 5; ++k) tr[k] = k < ndon ? ld4(pop_in + (s.row0 + r[k]) * ld + e0) : ti;
                const uint4 w = philox(make_uint4((uint32_t)c, (uint32_t)row, gen, kTagCr), key);
                const float4 o4 = ld4(s.shift + e0);
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
                            for (int k = 0; k < 5; ++k) xr[k] = f4get(tr[k], q);
                            x = mutant<float>(st, F, f4get(ti, q), f4get(tb, q), xr);
                        } else {
                            x = f4get(ti, q);
                        }
                        x = check_bound<float>(x, lb, ub, ok_bound);
                        f4set(x4, q, x);
                        f4set(y4, q, __fsub_rn(x, f4get(o4, q)));
                    }
                }
                st4(xrow + e0, x4);
                st4(yrow + e0, y4);
            }
        } else if (lr < kEvalTile) {
#pragma unroll
            for (int v = 0; v < Pl::CPL; ++v) {
                const int c = gl + G * v;
                if (c < nch) st4(yrow + 4 * c, make_float4(0.f, 0.f, 0.f, 0.f));
            }
        }
    }
    if (!ok_bound) atomicOr(&s_deverr, SPEO_DEVERR_BOUND_LIMIT);

    // ---- (3) evaluate: z = M (x - o) on CUDA cores, 8 rows per warp -------------------------
    float acc[kRowsPerWarp][Q];
#pragma unroll
    for (int rr = 0; rr < kRowsPerWarp; ++rr)
#pragma unroll
        for (int q = 0; q < Q; ++q) acc[rr][q] = 0.f;
    if (func_rotated(s.func_id)) {
        for (int kc = 0; kc < D; kc += Pl::KC) {
            const int ke = min(kc + Pl::KC, D);
            __syncthreads();
            if (kc > 0) {
                load_rot_rows<float, Q>(Ms, s.rot, s.ld_rot, D, kc, ke);
                __syncthreads();
            }
            eval_accumulate<float, Q>(acc, Ys, W, warp * kRowsPerWarp, Ms, W, kc, ke, lane);
        }
    } else {  // ids 8 and 10: no rotation
        __syncthreads();
        eval_identity<float, Q>(acc, Ys, W, warp * kRowsPerWarp, D, lane);
    }
    float f[kRowsPerWarp];
    eval_reduce<float, Q>(acc, D, s.func_id, func_scale(s.func_id), lane, f);
    if (lane == 0) {
#pragma unroll
        for (int rr = 0; rr < kRowsPerWarp; ++rr) {
            const int lr = warp * kRowsPerWarp + rr;
            if (lr < count) {
                sF[lr] = f[rr];
                if (a.trial_fit_out) a.trial_fit_out[row0 + lr] = f[rr];
            }
        }
    }
    __syncthreads();

    // ---- (4) select: strict `<` (kernel_DE_CUDA.cu:312); write the winner -------------------
#pragma unroll 2
    for (int p = 0; p < Pl::NPASS; ++p) {
        const int lr = p * Pl::RPP + grp;
        if (lr >= count) continue;
        const long long row = row0 + lr;
        const float pf = sPF[lr], tf = sF[lr];
        const bool win = tf < pf;
#pragma unroll
        for (int v = 0; v < Pl::CPL; ++v) {
            const int c = gl + G * v;
            if (c >= nch) continue;
            const float4 t4 = ld4(Xs + lr * W + 4 * c);
            st4(a.pop_out + row * ld + 4 * c, win ? t4 : ld4(pop_in + row * ld + 4 * c));
            if (a.trial_out) st4(a.trial_out + row * ld + 4 * c, t4);
        }
        if (gl == 0) a.fit_out[row] = win ? tf : pf;
    }
}

__device__ __forceinline__ bool tile_ok(const speo_work_item &it, const speo_segment &s)
{
    return it.count >= 1 && it.count <= kEvalTile && s.pop_size >= 2 && s.dim >= 1 && s.dim <= SPEO_MAX_DIM &&
           (s.ld & 3) == 0 && s.ld >= s.dim && it.first >= 0 && it.first + it.count <= s.pop_size &&
           func_supported(s.func_id);
}

// Advances the generation counter once every block of the launch has read it.
__device__ __forceinline__ void advance_gen(uint32_t *gen_ctr, uint32_t gen)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned done = atomicAdd(gen_ctr + 1, 1u);
        if (done == gridDim.x - 1) {
            gen_ctr[1] = 0;
            gen_ctr[0] = gen + 1;
            __threadfence();
        }
    }
}

// All tiles share one column class.
template <int Q>
__global__ void __launch_bounds__(256, 2) k_generation(GenArgs a)
{
    extern __shared__ __align__(16) float smem_f[];
    __shared__ float s_bf[8];
    __shared__ long long s_br[8];
    const uint32_t gen = *(volatile uint32_t *)a.gen_ctr;
    for (int t = blockIdx.x; t < a.n_items; t += gridDim.x) {
        const speo_work_item it = a.items[t];
        const speo_segment &s = a.segs[it.segment];
        if (!tile_ok(it, s) || q_class(s.dim) != Q) {
            if (threadIdx.x == 0) atomicOr(&s_deverr, SPEO_DEVERR_BAD_SEGMENT);
            continue;
        }
        gen_tile<Q>(a, it, s, gen, smem_f, s_bf, s_br);
    }
    advance_gen(a.gen_ctr, gen);
}

// Batched uneven segments: one launch per generation, the column class picked per tile.
// `max_q` is the largest column class the launch's shared memory was sized for.
__global__ void __launch_bounds__(256, 2) k_generation_mixed(GenArgs a, int max_q)
{
    extern __shared__ __align__(16) float smem_f[];
    __shared__ float s_bf[8];
    __shared__ long long s_br[8];
    const uint32_t gen = *(volatile uint32_t *)a.gen_ctr;
    for (int t = blockIdx.x; t < a.n_items; t += gridDim.x) {
        const speo_work_item it = a.items[t];
        const speo_segment &s = a.segs[it.segment];
        if (!tile_ok(it, s) || q_class(s.dim) > max_q) {
            if (threadIdx.x == 0) atomicOr(&s_deverr, SPEO_DEVERR_BAD_SEGMENT);
            continue;
        }
        switch (q_class(s.dim)) {
        case 1: gen_tile<1>(a, it, s, gen, smem_f, s_bf, s_br); break;
        case 2: gen_tile<2>(a, it, s, gen, smem_f, s_bf, s_br); break;
        case 4: gen_tile<4>(a, it, s, gen, smem_f, s_bf, s_br); break;
        default: gen_tile<8>(a, it, s, gen, smem_f, s_bf, s_br); break;
        }
    }
    advance_gen(a.gen_ctr, gen);
}

// ---- ring migration ----------------------------------------------------------------------
constexpr int kMaxMigrants = 32;

// k extreme rows of a segment by the whole block: best (ascending (f,row)) or worst
// (descending (f,row)). NaN ranks as +inf.
__device__ void block_extremes(const float *fit, long long row0, int P, int k, bool worst, long long *out,
                               float *sf, long long *sr)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int t = 0; t < k; ++t) {
        float bf = worst ? -__int_as_float(0x7f800000) : __int_as_float(0x7f800000);
        long long br = worst ? -1 : 0x7fffffffffffffffLL;
        for (int i = threadIdx.x; i < P; i += blockDim.x) {
            const long long row = row0 + i;
            bool taken = false;
            for (int u = 0; u < t; ++u) taken |= (out[u] == row);
            if (taken) continue;
            const float f = rank_key(fit[row]);
            const bool take = worst ? (f > bf || (f == bf && row > br)) : better(f, row, bf, br);
            if (take) { bf = f; br = row; }
        }
        for (int o = 16; o > 0; o >>= 1) {
            const float of = __shfl_xor_sync(0xffffffffu, bf, o);
            const long long orr = __shfl_xor_sync(0xffffffffu, br, o);
            const bool take = worst ? (of > bf || (of == bf && orr > br)) : better(of, orr, bf, br);
            if (take) { bf = of; br = orr; }
        }
        if (lane == 0) { sf[warp] = bf; sr[warp] = br; }
        __syncthreads();
        if (threadIdx.x == 0) {
            for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
                const bool take = worst ? (sf[w] > sf[0] || (sf[w] == sf[0] && sr[w] > sr[0]))
                                        : better(sf[w], sr[w], sf[0], sr[0]);
                if (take) { sf[0] = sf[w]; sr[0] = sr[w]; }
            }
            out[t] = sr[0];
        }
        __syncthreads();
    }
}

// Phase 1: every segment with a ring successor copies its k best rows (+ fitness) to staging.
__global__ void __launch_bounds__(256) k_emigrate(const speo_segment *segs, int k, const float *pop, const float *fit,
                                                  float *staging, int max_ld)
{
    __shared__ long long sel[kMaxMigrants];
    __shared__ float sf[8];
    __shared__ long long sr[8];
    const speo_segment &s = segs[blockIdx.x];
    if (s.ring_next < 0) return;
    if (s.pop_size < k || s.dim < 1 || s.dim > max_ld) {
        if (threadIdx.x == 0) atomicOr(&s_deverr, SPEO_DEVERR_BAD_SEGMENT);
        return;
    }
    block_extremes(fit, s.row0, s.pop_size, k, false, sel, sf, sr);
    for (int t = 0; t < k; ++t) {
        float *dst = staging + ((size_t)blockIdx.x * k + t) * (max_ld + 1);
        for (int e = threadIdx.x; e < s.dim; e += blockDim.x) dst[e] = pop[sel[t] * s.ld + e];
        if (threadIdx.x == 0) dst[max_ld] = fit[sel[t]];
    }
}

// Phase 2: every segment that is some segment's successor replaces its k worst rows, worst
// first, with that predecessor's emigrants, best first.
__global__ void __launch_bounds__(256) k_immigrate(const speo_segment *segs, int n_segs, int k, float *pop, float *fit,
                                                   const float *staging, int max_ld)
{
    __shared__ long long sel[kMaxMigrants];
    __shared__ float sf[8];
    __shared__ long long sr[8];
    __shared__ int src, nsrc;
    const int d = blockIdx.x;
    const speo_segment &s = segs[d];
    // the predecessor (the lowest-numbered segment whose ring_next is d), all threads scanning
    if (threadIdx.x == 0) { src = 0x7fffffff; nsrc = 0; }
    __syncthreads();
    for (int i = threadIdx.x; i < n_segs; i += blockDim.x)
        if (segs[i].ring_next == d) {
            atomicMin(&src, i);
            atomicAdd(&nsrc, 1);
        }
    __syncthreads();
    if (threadIdx.x == 0) {
        if (nsrc > 1) atomicOr(&s_deverr, SPEO_DEVERR_BAD_SEGMENT);
        if (nsrc == 0) src = -1;
    }
    __syncthreads();
    if (src < 0) return;
    if (s.pop_size < k || s.dim < 1 || segs[src].pop_size < k || segs[src].dim > max_ld) {
        if (threadIdx.x == 0) atomicOr(&s_deverr, SPEO_DEVERR_BAD_SEGMENT);
        return;
    }
    block_extremes(fit, s.row0, s.pop_size, k, true, sel, sf, sr);
    const int dim = min(s.dim, segs[src].dim);
    for (int t = 0; t < k; ++t) {
        const float *from = staging + ((size_t)src * k + t) * (max_ld + 1);
        for (int e = threadIdx.x; e < dim; e += blockDim.x) pop[sel[t] * s.ld + e] = from[e];
        if (threadIdx.x == 0) fit[sel[t]] = from[max_ld];
    }
}

// Initial rows of every segment: x = lb + u*(ub-lb), u from philox({e/4, row, 0, INIT}, seed).
__global__ void k_init_segments(const speo_segment *segs, const speo_work_item *items, int n_items, float *pop)
{
    for (int t = blockIdx.x; t < n_items; t += gridDim.x) {
        const speo_work_item it = items[t];
        const speo_segment &s = segs[it.segment];
        if (it.count < 1 || it.first < 0 || it.first + it.count > s.pop_size || s.dim < 1 || s.dim > s.ld) {
            if (threadIdx.x == 0) atomicOr(&s_deverr, SPEO_DEVERR_BAD_SEGMENT);
            continue;
        }
        const int groups = (s.dim + 3) >> 2;
        const uint2 key = seed_key(s.seed);
        const float range = s.ub - s.lb;
        for (int i = threadIdx.x; i < it.count * groups; i += blockDim.x) {
            const int lr = i / groups, g = i - lr * groups;
            const long long row = s.row0 + it.first + lr;
            const uint4 w = philox(make_uint4((uint32_t)g, (uint32_t)row, 0u, kTagInit), key);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int e = 4 * g + q;
                if (e < s.dim) pop[row * s.ld + e] = __fmaf_rn(u01(pick(w, (uint32_t)q)), range, s.lb);
            }
        }
    }
}

template <typename K, typename... Extra>
int launch_gen(K kernel, size_t smem, const GenArgs &a, cudaStream_t st, Extra... extra)
{
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return check_cuda(e, "cudaFuncSetAttribute(k_generation)");
    const int grid = a.n_items < 2 * sm_count() ? a.n_items : 2 * sm_count();
    kernel<<<grid, 256, smem, st>>>(a, extra...);
    return check_launch("k_generation");
}

size_t gen_smem(int Q)
{
    return Q == 1 ? GenPlan<1>::bytes : Q == 2 ? GenPlan<2>::bytes : Q == 4 ? GenPlan<4>::bytes : GenPlan<8>::bytes;
}

}  // namespace
}  // namespace speo

using namespace speo;

extern "C" int speo_generation(const speo_segment *segs, const speo_work_item *items, int n_items, int dim_lo,
                               int dim_hi, const float *pop_in, const float *fit_in, float *pop_out, float *fit_out,
                               uint32_t *d_gen, int use_tc, float *trial_out, float *trial_fit_out, void *stream)
{
    if (!segs || !items || !pop_in || !fit_in || !pop_out || !fit_out || !d_gen || n_items < 1)
        return fail(SPEO_ERR_INVALID_ARG, "speo_generation: bad arguments");
    if (pop_in == pop_out || fit_in == fit_out)
        return fail(SPEO_ERR_INVALID_ARG, "speo_generation: input and output buffers must differ");
    if (dim_lo < 1 || dim_hi > SPEO_MAX_DIM || dim_lo > dim_hi)
        return fail(SPEO_ERR_INVALID_ARG, "speo_generation: dim range [%d, %d]", dim_lo, dim_hi);
    if (use_tc)  // the tensor-core generation needs the flat buffer's extent: speo_generation_tc
        return fail(SPEO_ERR_UNSUPPORTED, "speo_generation: use_tc = 1 is speo_generation_tc (rows, ld, trial buffers)");
    GenArgs a{segs, items, n_items, pop_in, fit_in, pop_out, fit_out, d_gen, trial_out, trial_fit_out};
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int qlo = q_class(dim_lo), qhi = q_class(dim_hi);
    if (qlo != qhi) return launch_gen(k_generation_mixed, gen_smem(qhi), a, st, qhi);
    switch (qhi) {
    case 1: return launch_gen(k_generation<1>, gen_smem(1), a, st);
    case 2: return launch_gen(k_generation<2>, gen_smem(2), a, st);
    case 4: return launch_gen(k_generation<4>, gen_smem(4), a, st);
    default: return launch_gen(k_generation<8>, gen_smem(8), a, st);
    }
}

extern "C" int speo_ring_migrate(const speo_segment *segs, int n_segs, int k, float *pop, float *fit, float *staging,
                                 int max_ld, void *stream)
{
    if (!segs || !pop || !fit || !staging || n_segs < 1 || max_ld < 1)
        return fail(SPEO_ERR_INVALID_ARG, "speo_ring_migrate: bad arguments");
    if (k < 1 || k > kMaxMigrants)
        return fail(SPEO_ERR_INVALID_ARG, "speo_ring_migrate: k = %d outside [1, %d]", k, kMaxMigrants);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    k_emigrate<<<n_segs, 256, 0, st>>>(segs, k, pop, fit, staging, max_ld);
    if (int e = check_launch("k_emigrate")) return e;
    k_immigrate<<<n_segs, 256, 0, st>>>(segs, n_segs, k, pop, fit, staging, max_ld);
    return check_launch("k_immigrate");
}

extern "C" int speo_init_population(const speo_segment *segs, int n_segs, const speo_work_item *items, int n_items,
                                    float *pop, void *stream)
{
    if (!segs || !items || !pop || n_segs < 1 || n_items < 1)
        return fail(SPEO_ERR_INVALID_ARG, "speo_init_population: bad arguments");
    const int grid = n_items < 4 * sm_count() ? n_items : 4 * sm_count();
    k_init_segments<<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(segs, items, n_items, pop);
    return check_launch("k_init_segments");
}

// ---- ring migration without caller-provided scratch -----------------------------------------
// Staging for callers that cannot allocate device memory: a fixed array in the library's own
// device image. Every GPU that loads the library holds it until the process exits.
namespace {
static __device__ __align__(256) float g_migration_staging[SPEO_NOALLOC_STAGING_FLOATS];

// The array's device address belongs to the CUDA context that loaded the module: a device reset
// makes a new primary context, and a caller may bind a context of its own. So the address is
// kept per (device, context) and looked up again on every call made outside stream capture;
// a call during capture (when the lookup may not run) takes the address that the last call
// outside capture found in the same context.
struct StagingAddr {
    int dev;
    void *ctx;
    float *addr;
};
constexpr int kStagingSlots = 64;
std::mutex g_staging_mu;
StagingAddr g_staging[kStagingSlots];
int g_staging_used = 0;

// The current context (CUcontext) through the driver's cuCtxGetCurrent, found by the runtime's
// entry-point query (the library does not link the driver API); null where it is unavailable.
void *current_context()
{
    using CtxGetCurrent = int (*)(void **);
    static CtxGetCurrent fn = [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess) {
            cudaGetLastError();
            return static_cast<CtxGetCurrent>(nullptr);
        }
        return reinterpret_cast<CtxGetCurrent>(p);
    }();
    void *ctx = nullptr;
    if (!fn || fn(&ctx) != 0) return nullptr;
    return ctx;
}

StagingAddr *staging_slot(int dev, void *ctx)
{
    for (int i = 0; i < g_staging_used; ++i)
        if (g_staging[i].dev == dev && g_staging[i].ctx == ctx) return &g_staging[i];
    return nullptr;
}

// Device address of g_migration_staging for the current device and context.
int staging_address(cudaStream_t st, float **out)
{
    int dev = 0;
    if (int e = check_cuda(cudaGetDevice(&dev), "speo_ring_migrate_noalloc: cudaGetDevice")) return e;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cap) != cudaSuccess) {
        cudaGetLastError();  // e.g. the legacy stream queried while another stream captures: no lookup now
        cap = cudaStreamCaptureStatusActive;
    }
    std::lock_guard<std::mutex> lock(g_staging_mu);
    if (cap == cudaStreamCaptureStatusNone) {
        void *addr = nullptr;
        if (int e = check_cuda(cudaGetSymbolAddress(&addr, g_migration_staging),
                               "speo_ring_migrate_noalloc: cudaGetSymbolAddress"))
            return e;
        void *ctx = current_context();  // the lookup above made the device's context current
        StagingAddr *slot = staging_slot(dev, ctx);
        if (!slot) {
            slot = &g_staging[g_staging_used < kStagingSlots ? g_staging_used++ : kStagingSlots - 1];
            slot->dev = dev;
            slot->ctx = ctx;
        }
        slot->addr = static_cast<float *>(addr);
        *out = slot->addr;
        return SPEO_OK;
    }
    const StagingAddr *slot = staging_slot(dev, current_context());
    if (!slot)
        return fail(SPEO_ERR_INVALID_ARG,
                    "speo_ring_migrate_noalloc: called during stream capture before any call outside capture on "
                    "device %d in this context; make one call outside capture first",
                    dev);
    *out = slot->addr;
    return SPEO_OK;
}
}  // namespace

extern "C" int speo_ring_migrate_noalloc(const speo_segment *segs, int n_segs, int k, float *pop, float *fit,
                                         int max_ld, void *stream)
{
    if (!segs || !pop || !fit || n_segs < 1 || max_ld < 1)
        return fail(SPEO_ERR_INVALID_ARG, "speo_ring_migrate_noalloc: bad arguments");
    if (k < 1 || k > kMaxMigrants)
        return fail(SPEO_ERR_INVALID_ARG, "speo_ring_migrate_noalloc: k = %d outside [1, %d]", k, kMaxMigrants);
    const unsigned long long need = (unsigned long long)n_segs * (unsigned long long)k * ((unsigned long long)max_ld + 1ULL);
    if (need > SPEO_NOALLOC_STAGING_FLOATS)
        return fail(SPEO_ERR_INVALID_ARG,
                    "speo_ring_migrate_noalloc: %d segments x %d migrants x (max_ld %d + 1) = %llu staging floats "
                    "exceed the fixed %d; use speo_ring_migrate with a caller buffer",
                    n_segs, k, max_ld, need, SPEO_NOALLOC_STAGING_FLOATS);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    float *staging = nullptr;
    if (int e = staging_address(st, &staging)) return e;
    k_emigrate<<<n_segs, 256, 0, st>>>(segs, k, pop, fit, staging, max_ld);
    if (int e = check_launch("k_emigrate")) return e;
    k_immigrate<<<n_segs, 256, 0, st>>>(segs, n_segs, k, pop, fit, staging, max_ld);
    return check_launch("k_immigrate");
}
