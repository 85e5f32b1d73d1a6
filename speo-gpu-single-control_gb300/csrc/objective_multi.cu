// objective_multi.cu -- API_evaluateFitness for the CEC2014 hybrid (17-22) and composition
// (23-30) functions (CUDA_EA_library/kernel_CEC2014_CUDA.cu:1204-1670, HybirdFunc1-6 and
// CompFunc1-8; CPU definitions CEC2014.cc:954-1520) on the reference's device data layout: one
// launch per call, every component's shift + rotation + body fused per 64-row tile, the
// composition weights and mixing in the same kernel.
#include "eval_tile.cuh"
#include "host.h"

SPEO_DEFINE_DEVERR(speo_deverr_objective_multi)

namespace speo {
namespace {

// Tiles of 8 * RPW rows: RPW = 2 while 64-row tiles would leave SMs idle (the reference's
// islands of a few thousand rows), RPW = 8 above that.
template <typename T, int Q, int RPW>
__global__ void __launch_bounds__(256) k_eval_ref_multi(const T *X, int ldx, int P, int D, int func, const T *shift,
                                                        const T *rot, const int *shuf, T *fit)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *Ys, *Ms, *Xs, *fbuf, *sbuf;
    int *Ss;
    multi_smem<T, Q, RPW>(smem_raw, Ys, Ms, Xs, fbuf, sbuf, Ss);
    constexpr int kTile = 8 * RPW;
    const int tiles = (P + kTile - 1) / kTile;
    for (int t = blockIdx.x; t < tiles; t += gridDim.x)
        eval_multi_tile<T, Q, RPW>(ref_tile_multi<T, kTile>(t, X, ldx, P, D, func, shift, rot, shuf, fit), Ys, Ms, Xs,
                                   Ss, fbuf, sbuf, &s_deverr, 0, func_components(func), true);
}

template <typename T, int Q, int RPW>
int launch_ref_multi_rpw(const T *X, int ldx, int P, int D, int func, const T *shift, const T *rot, const int *shuf,
                         T *fit, cudaStream_t st)
{
    constexpr size_t smem = multi_smem_bytes<T, Q, RPW>();
    static_assert(smem <= 227 * 1024, "tile buffers exceed the shared memory of one block");
    cudaError_t e =
        cudaFuncSetAttribute(k_eval_ref_multi<T, Q, RPW>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return check_cuda(e, "cudaFuncSetAttribute(k_eval_ref_multi)");
    const int tiles = (P + 8 * RPW - 1) / (8 * RPW);
    const int fit_sm = (int)((220u * 1024u) / smem), per_sm = fit_sm < 1 ? 1 : fit_sm > 4 ? 4 : fit_sm;
    const int grid = tiles < per_sm * sm_count() ? tiles : per_sm * sm_count();
    k_eval_ref_multi<T, Q, RPW><<<grid, 256, smem, st>>>(X, ldx, P, D, func, shift, rot, shuf, fit);
    return check_launch("k_eval_ref_multi");
}

template <typename T, int Q>
int launch_ref_multi(const T *X, int ldx, int P, int D, int func, const T *shift, const T *rot, const int *shuf, T *fit,
                     cudaStream_t st)
{
    // FP64 with D > 128 keeps 16-row tiles: a 64-row tile's buffers would not fit in shared memory
    if constexpr (sizeof(T) == 8 && Q == 8) {
        return launch_ref_multi_rpw<T, Q, 2>(X, ldx, P, D, func, shift, rot, shuf, fit, st);
    } else {
        if ((P + kEvalTile - 1) / kEvalTile < 2 * sm_count())
            return launch_ref_multi_rpw<T, Q, 2>(X, ldx, P, D, func, shift, rot, shuf, fit, st);
        return launch_ref_multi_rpw<T, Q, kRowsPerWarp>(X, ldx, P, D, func, shift, rot, shuf, fit, st);
    }
}

}  // namespace

template <typename T>
int eval_ref_multi(T *fit, const T *X, const T *shift, const T *rot, const int *shuf, int P, int D, int func,
                   cudaStream_t st)
{
    int ldx = 1;
    while (ldx < D) ldx <<= 1;
    if (ldx < 32) ldx = 32;
    switch ((D + 31) / 32) {
    case 1: return launch_ref_multi<T, 1>(X, ldx, P, D, func, shift, rot, shuf, fit, st);
    case 2: return launch_ref_multi<T, 2>(X, ldx, P, D, func, shift, rot, shuf, fit, st);
    case 3: case 4: return launch_ref_multi<T, 4>(X, ldx, P, D, func, shift, rot, shuf, fit, st);
    default: return launch_ref_multi<T, 8>(X, ldx, P, D, func, shift, rot, shuf, fit, st);
    }
}
template int eval_ref_multi<float>(float *, const float *, const float *, const float *, const int *, int, int, int,
                                   cudaStream_t);
template int eval_ref_multi<double>(double *, const double *, const double *, const double *, const int *, int, int,
                                    int, cudaStream_t);

}  // namespace speo
