// objective.cu -- exact objective evaluation on CUDA cores:
//   * API_evaluateFitness / API_evaluateFitness_f32: the reference-shaped entry point
//     (CUDA_EA_library/CEC2014_CUDA.h:35-37, kernel_CEC2014_CUDA.cu:1672-1797) for ids 1-16
//     and 31 (rotated sphere), reference data layout; ids 17-30 in objective_multi.cu;
//   * speo_evaluate: the same evaluation over the segment/work-item tables (FP32), ids 1-31;
//   * speo_best_reeval_f64: per segment argmin + FP64 re-evaluation of the best row.
#include <cmath>

#include "eval_tile.cuh"
#include "host.h"

SPEO_DEFINE_DEVERR(speo_deverr_objective)

namespace speo {
namespace {

// Piece `sub` (64 rows) of work item t; work items may be any size.
__device__ __forceinline__ bool seg_tile(int t, int sub, const speo_segment *segs, const speo_work_item *items,
                                         const float *pop, float *fit, TileDesc &d)
{
    const speo_work_item it = items[t];
    const speo_segment &s = segs[it.segment];
    if (it.count < 1 || it.first < 0 || it.first + it.count > s.pop_size || s.dim < 1 || s.dim > SPEO_MAX_DIM ||
        s.ld < s.dim)
        return false;
    const long long row = s.row0 + it.first + (long long)sub * kEvalTile;
    d.x = pop + row * s.ld;
    d.ldx = s.ld;
    d.count = min(kEvalTile, it.count - sub * kEvalTile);
    d.D = s.dim;
    d.func = s.func_id;
    d.ld_rot = s.ld_rot;
    d.shift = s.shift;
    d.rot = s.rot;
    d.fit = fit + row;
    d.shift_cs = d.shuf_cs = s.ld_rot;
    d.rot_cs = (long long)s.dim * s.ld_rot;
    d.shuf = s.shuffle;
    return true;
}

// G: the generic variant (ids other than 8, 9, 31); G = false: per-coordinate sums only.
template <typename T, int Q, bool G>
__device__ void eval_one_tile(const TileDesc &d, T *Ys, T *Ms)
{
    constexpr int W = 32 * Q;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const T *X = static_cast<const T *>(d.x);
    const T *o = static_cast<const T *>(d.shift);
    const T *rot = static_cast<const T *>(d.rot);
    __syncthreads();  // previous tile done with Ys / Ms
    for (int i = threadIdx.x; i < kEvalTile * W; i += blockDim.x) {
        const int r = i / W, k = i - r * W;
        Ys[i] = (r < d.count && k < d.D) ? X[(size_t)r * d.ldx + k] - o[k] : T(0);
    }
    T acc[kRowsPerWarp][Q];
#pragma unroll
    for (int rr = 0; rr < kRowsPerWarp; ++rr)
#pragma unroll
        for (int q = 0; q < Q; ++q) acc[rr][q] = T(0);
    if (func_rotated(d.func)) {
        for (int kc = 0; kc < d.D; kc += kChunk) {
            const int ke = min(kc + kChunk, d.D);
            __syncthreads();
            load_rot_rows<T, Q>(Ms, rot, d.ld_rot, d.D, kc, ke);
            __syncthreads();
            eval_accumulate<T, Q>(acc, Ys, W, warp * kRowsPerWarp, Ms, W, kc, ke, lane);
        }
    } else {  // ids 8 and 10: no rotation
        __syncthreads();
        eval_identity<T, Q>(acc, Ys, W, warp * kRowsPerWarp, d.D, lane);
    }
    T f[kRowsPerWarp];
    const T scale = sizeof(T) == 4 ? (T)func_scale(d.func) : (T)func_scale_f64(d.func);
    eval_reduce<T, Q, kRowsPerWarp, G>(acc, d.D, d.func, scale, lane, f);
    if (lane == 0) {
        T *fit = static_cast<T *>(d.fit);
#pragma unroll
        for (int rr = 0; rr < kRowsPerWarp; ++rr) {
            const int r = warp * kRowsPerWarp + rr;
            if (r < d.count) fit[r] = f[rr];
        }
    }
}

template <typename T, int Q, bool G>
__global__ void __launch_bounds__(256) k_eval_ref(const T *X, int ldx, int P, int D, int func, const T *shift,
                                                  const T *rot, T *fit)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *Ys = reinterpret_cast<T *>(smem_raw);
    T *Ms = Ys + kEvalTile * 32 * Q;
    const int tiles = (P + kEvalTile - 1) / kEvalTile;
    for (int t = blockIdx.x; t < tiles; t += gridDim.x)
        eval_one_tile<T, Q, G>(ref_tile<T>(t, X, ldx, P, D, func, shift, rot, fit), Ys, Ms);
}

// Four blocks per SM where that fits 64 registers without spilling (per-coordinate sums, Q = 1, 4).
template <int Q, bool G>
__global__ void __launch_bounds__(256, (!G && (Q == 1 || Q == 4)) ? 4 : 1) k_eval_seg(const speo_segment *segs, const speo_work_item *items, int n_items,
                                                  const float *pop, float *fit)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float *Ys = reinterpret_cast<float *>(smem_raw);
    float *Ms = Ys + kEvalTile * 32 * Q;
    for (int t = blockIdx.x; t < n_items; t += gridDim.x) {
        const int pieces = (items[t].count + kEvalTile - 1) / kEvalTile;
        for (int sub = 0; sub < pieces; ++sub) {
            TileDesc d;
            if (!seg_tile(t, sub, segs, items, pop, fit, d)) {
                if (threadIdx.x == 0) atomicOr(&s_deverr, SPEO_DEVERR_BAD_SEGMENT);
                break;
            }
            if ((d.D + 31) / 32 > Q) break;  // handled by the launch for its own Q
            if (Q > 1 && (d.D + 31) / 32 <= Q / 2) break;
            if (func_sum_form(d.func) == G) break;  // handled by the other variant's launch
            if (G && func_multi(d.func)) {
                if (!multi_dim_ok(d.func, d.D) || (d.ld_rot & 3) || d.ld_rot < d.D) {
                    if (threadIdx.x == 0) atomicOr(&s_deverr, SPEO_DEVERR_BAD_SEGMENT);
                    break;
                }
                float *Xs, *fbuf, *sbuf;
                int *Ss;
                multi_smem<float, Q>(smem_raw, Ys, Ms, Xs, fbuf, sbuf, Ss);
                eval_multi_tile<float, Q>(d, Ys, Ms, Xs, Ss, fbuf, sbuf, &s_deverr, 0, func_components(d.func), true);
                continue;
            }
            if (!func_supported(d.func)) {
                if (threadIdx.x == 0) atomicOr(&s_deverr, SPEO_DEVERR_BAD_SEGMENT);
                break;
            }
            eval_one_tile<float, Q, G>(d, Ys, Ms);
        }
    }
}

// Per segment: argmin of fit (NaN as +inf, ties lowest row), then FP64 f(x) - f* of that row.
__global__ void __launch_bounds__(256) k_best_reeval(const speo_segment *segs, const float *pop, const float *fit,
                                                     int64_t *best_row, double *best_err)
{
    __shared__ double ys[SPEO_MAX_DIM], zs[SPEO_MAX_DIM];
    __shared__ float bfs[8];
    __shared__ long long brs[8];
    const speo_segment &s = segs[blockIdx.x];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (s.pop_size < 1 || s.dim < 1 || s.dim > SPEO_MAX_DIM || !func_any(s.func_id)) {
        if (threadIdx.x == 0) {
            atomicOr(&s_deverr, SPEO_DEVERR_BAD_SEGMENT);
            best_err[blockIdx.x] = __longlong_as_double(0x7ff8000000000000LL);
            best_row[blockIdx.x] = -1;
        }
        return;
    }
    float bf = __int_as_float(0x7f800000);
    long long br = 0x7fffffffffffffffLL;
    for (int i = threadIdx.x; i < s.pop_size; i += blockDim.x) {
        const float f = rank_key(fit[s.row0 + i]);
        if (better(f, s.row0 + i, bf, br)) { bf = f; br = s.row0 + i; }
    }
    for (int o = 16; o > 0; o >>= 1) {
        const float of = __shfl_xor_sync(0xffffffffu, bf, o);
        const long long orr = __shfl_xor_sync(0xffffffffu, br, o);
        if (better(of, orr, bf, br)) { bf = of; br = orr; }
    }
    if (lane == 0) { bfs[warp] = bf; brs[warp] = br; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < blockDim.x / 32; ++w)
            if (better(bfs[w], brs[w], bfs[0], brs[0])) { bfs[0] = bfs[w]; brs[0] = brs[w]; }
    }
    __syncthreads();
    const long long row = brs[0];
    const int D = s.dim, fid = s.func_id;
    // ids 17-30: each component in turn (shift / matrix / shuffle c), then the mixing
    const bool multi = func_multi(fid);
    if (multi && (!multi_dim_ok(fid, D) || (s.ld_rot & 3) || s.ld_rot < D)) {
        if (threadIdx.x == 0) {
            atomicOr(&s_deverr, SPEO_DEVERR_BAD_SEGMENT);
            best_err[blockIdx.x] = __longlong_as_double(0x7ff8000000000000LL);
            best_row[blockIdx.x] = row;
        }
        return;
    }
    __shared__ int ss[SPEO_MAX_DIM];
    __shared__ double cfit[kMaxComp], csq[kMaxComp];
    const int nc = func_components(fid);
    for (int c = 0; c < nc; ++c) {
        const int h = multi_hybrid(fid, c);
        const CompPiece pc = func_composition(fid) ? comp_piece(fid, c) : CompPiece{fid, func_rotated(fid), 0.0, 0.0};
        const float *o = s.shift + (size_t)c * s.ld_rot;
        const float *rot = s.rot + (size_t)c * D * s.ld_rot;
        __syncthreads();
        for (int k = threadIdx.x; k < D; k += blockDim.x) {
            ys[k] = (double)pop[row * s.ld + k] - (double)o[k];
            if (h >= 0) {
                int v = s.shuffle ? s.shuffle[(size_t)c * s.ld_rot + k] - 1 : -1;
                if (v < 0 || v >= D) {
                    atomicOr(&s_deverr, SPEO_DEVERR_BAD_SEGMENT);
                    v = 0;
                }
                ss[k] = v;
            }
        }
        __syncthreads();
        const double scale = h >= 0 ? 1.0 : func_scale_f64(pc.fid);
        const double fs = h >= 0 ? 0.0 : func_fixed_shift<double>(pc.fid);
        for (int j = threadIdx.x; j < D; j += blockDim.x) {
            double z = ys[j];
            if (h >= 0 || pc.rotated) {
                z = 0.0;
                for (int k = 0; k < D; ++k) z = __fma_rn(ys[k], (double)rot[(size_t)k * s.ld_rot + j], z);
            }
            zs[j] = z * scale + fs;
        }
        __syncthreads();
        if (warp == 0) {
            double f;
            if (h >= 0) {
                f = hybrid_row_warp<double>(zs, ss, h, D, lane);
            } else {
                RowAcc<double> a;
                for (int j = lane; j < D; j += 32) row_push(a, pc.fid, j, zs[j], zs[j + 1 < D ? j + 1 : 0], D);
                a.s1 = warp_sum(a.s1);
                a.s2 = warp_sum(a.s2);
                a.p = warp_prod(a.p);
                f = row_finish(a, pc.fid, D);
                if (pc.den != 0.0) f = pc.num * f / pc.den;
            }
            double sq = 0.0;
            for (int k = lane; k < D; k += 32) sq += ys[k] * ys[k];
            sq = warp_sum(sq);
            if (lane == 0) { cfit[c] = f; csq[c] = sq; }
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        best_err[blockIdx.x] = func_composition(fid) ? comp_combine<double>(fid, D, cfit, csq) : cfit[0];
        best_row[blockIdx.x] = row;
    }
}

template <typename T, int Q>
int launch_ref(const T *X, int ldx, int P, int D, int func, const T *shift, const T *rot, T *fit, cudaStream_t st)
{
    const size_t smem = sizeof(T) * (size_t)(kEvalTile + kChunk) * 32 * Q;
    const bool generic = !func_sum_form(func);
    cudaError_t e = cudaFuncSetAttribute(generic ? k_eval_ref<T, Q, true> : k_eval_ref<T, Q, false>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return check_cuda(e, "cudaFuncSetAttribute(k_eval_ref)");
    const int tiles = (P + kEvalTile - 1) / kEvalTile;
    const int grid = tiles < 4 * sm_count() ? tiles : 4 * sm_count();
    if (generic)
        k_eval_ref<T, Q, true><<<grid, 256, smem, st>>>(X, ldx, P, D, func, shift, rot, fit);
    else
        k_eval_ref<T, Q, false><<<grid, 256, smem, st>>>(X, ldx, P, D, func, shift, rot, fit);
    return check_launch("k_eval_ref");
}

template <typename T>
int eval_ref(T *fit, T *X, T *shift, T *rot, const int *shuf, int P, int D, int func)
{
    if (!func_any(func))
        return fail(SPEO_ERR_UNSUPPORTED, "API_evaluateFitness: function_ID %d is not implemented (1-31)", func);
    if (!fit || !X || !shift || !rot) return fail(SPEO_ERR_INVALID_ARG, "API_evaluateFitness: null pointer");
    if (P <= 0 || D < 1 || D > SPEO_MAX_DIM)
        return fail(SPEO_ERR_INVALID_ARG, "API_evaluateFitness: pop_size %d, dim %d", P, D);
    if (func_uses_shuffle(func) && !shuf)
        return fail(SPEO_ERR_INVALID_ARG, "API_evaluateFitness: function_ID %d needs the shuffle data", func);
    if (func_multi(func) && !multi_dim_ok(func, D))
        return fail(SPEO_ERR_INVALID_ARG, "API_evaluateFitness: function_ID %d is not defined for dim %d", func, D);
    int ldx = 1;
    while (ldx < D) ldx <<= 1;
    if (ldx < 32) ldx = 32;
    cudaStream_t st = api_stream();
    if (func_multi(func)) return eval_ref_multi<T>(fit, X, shift, rot, shuf, P, D, func, st);
    switch ((D + 31) / 32) {
    case 1: return launch_ref<T, 1>(X, ldx, P, D, func, shift, rot, fit, st);
    case 2: return launch_ref<T, 2>(X, ldx, P, D, func, shift, rot, fit, st);
    case 3: case 4: return launch_ref<T, 4>(X, ldx, P, D, func, shift, rot, fit, st);
    default: return launch_ref<T, 8>(X, ldx, P, D, func, shift, rot, fit, st);
    }
}

template <int Q>
int launch_seg(const speo_segment *segs, const speo_work_item *items, int n_items, const float *pop, float *fit,
               cudaStream_t st)
{
    const size_t smem = sizeof(float) * (size_t)(kEvalTile + kChunk) * 32 * Q;
    constexpr size_t smem_g = multi_smem_bytes<float, Q>();  // the generic variant also runs ids 17-30
    static_assert(smem_g <= 227 * 1024, "tile buffers exceed the shared memory of one block");
    // two variants: the per-coordinate sums (8, 9, 31) and the other ids; each skips the other's tiles
    cudaError_t e = cudaFuncSetAttribute(k_eval_seg<Q, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_eval_seg<Q, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_g);
    if (e != cudaSuccess) return check_cuda(e, "cudaFuncSetAttribute(k_eval_seg)");
    const int grid = n_items < 4 * sm_count() ? n_items : 4 * sm_count();
    k_eval_seg<Q, false><<<grid, 256, smem, st>>>(segs, items, n_items, pop, fit);
    if (int r = check_launch("k_eval_seg")) return r;
    k_eval_seg<Q, true><<<grid, 256, smem_g, st>>>(segs, items, n_items, pop, fit);
    return check_launch("k_eval_seg");
}

}  // namespace
}  // namespace speo

using namespace speo;

extern "C" void API_evaluateFitness(double *f, double *, double *, double *X, double *shift, double *M, int *shuffle,
                                    double *, double *, double *, int P, int D, double, int fid)
{
    eval_ref<double>(f, X, shift, M, shuffle, P, D, fid);
}

extern "C" void API_evaluateFitness_f32(float *f, float *, float *, float *X, float *shift, float *M, int *shuffle,
                                        float *, float *, float *, int P, int D, float, int fid)
{
    eval_ref<float>(f, X, shift, M, shuffle, P, D, fid);
}

extern "C" int speo_evaluate(const speo_segment *segs, const speo_work_item *items, int n_items, int dim_lo,
                             int dim_hi, const float *pop, float *fit, void *stream)
{
    if (!segs || !items || !pop || !fit || n_items < 0)
        return fail(SPEO_ERR_INVALID_ARG, "speo_evaluate: bad arguments");
    if (n_items == 0) return SPEO_OK;
    if (dim_lo < 1 || dim_hi > SPEO_MAX_DIM || dim_lo > dim_hi)
        return fail(SPEO_ERR_INVALID_ARG, "speo_evaluate: dim range [%d, %d]", dim_lo, dim_hi);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // One launch per column-group width present in [dim_lo, dim_hi]; each skips other widths.
    for (int Q : {1, 2, 4, 8}) {
        const int qmin = Q == 1 ? 1 : Q == 2 ? 33 : Q == 4 ? 65 : 129, qmax = 32 * Q;
        if (dim_hi < qmin || dim_lo > qmax) continue;
        int r = SPEO_OK;
        switch (Q) {
        case 1: r = launch_seg<1>(segs, items, n_items, pop, fit, st); break;
        case 2: r = launch_seg<2>(segs, items, n_items, pop, fit, st); break;
        case 4: r = launch_seg<4>(segs, items, n_items, pop, fit, st); break;
        case 8: r = launch_seg<8>(segs, items, n_items, pop, fit, st); break;
        }
        if (r) return r;
    }
    return SPEO_OK;
}

extern "C" int speo_best_reeval_f64(const speo_segment *segs, int n_segs, const float *pop, const float *fit,
                                    int64_t *best_row, double *best_err, void *stream)
{
    if (!segs || !pop || !fit || !best_row || !best_err || n_segs < 0)
        return fail(SPEO_ERR_INVALID_ARG, "speo_best_reeval_f64: bad arguments");
    if (n_segs == 0) return SPEO_OK;
    k_best_reeval<<<n_segs, 256, 0, static_cast<cudaStream_t>(stream)>>>(segs, pop, fit, best_row, best_err);
    return check_launch("k_best_reeval");
}
