// eval_simt.cuh -- CUDA-core evaluation of a tile of rows: z = s * M (x - o), f = sum term(z).
//
// Replaces global_ShiftAndRotation + global_f8 (CUDA_EA_library/kernel_CEC2014_CUDA.cu:147-181,
// 557-587) with one pass: the (x - o) tile sits in shared memory, M^T is read row by row from
// shared memory (conflict-free: lane j reads column j), every warp keeps the z accumulators of
// its 8 rows in registers and reduces the objective with shuffles. Nothing is written back
// except the fitness.
#pragma once

#include "common.cuh"

namespace speo {

constexpr int kRowsPerWarp = 8;
constexpr int kEvalWarps = 8;
constexpr int kEvalTile = kRowsPerWarp * kEvalWarps;  // 64 rows per 256-thread block

// acc[rr][q] += sum_k Y[row0+rr][k] * Ms[(k-kbeg)*ms_ld + lane + 32q], k in [kbeg, kend), for the
// RPW rows of the warp. Ys rows are ys_ld apart (multiple of 4 for float); columns >= D of Ms must
// be zero or unused. The order of the FMAs of one row does not depend on RPW.
template <typename T, int Q, int RPW>
__device__ __forceinline__ void eval_accumulate(T (&acc)[RPW][Q], const T *__restrict__ Ys, int ys_ld, int row0,
                                                const T *__restrict__ Ms, int ms_ld, int kbeg, int kend, int lane)
{
    int k = kbeg;
    if constexpr (sizeof(T) == 4) {
        for (; k + 4 <= kend; k += 4) {
            T m[4][Q];
#pragma unroll
            for (int kk = 0; kk < 4; ++kk)
#pragma unroll
                for (int q = 0; q < Q; ++q) m[kk][q] = Ms[(k + kk - kbeg) * ms_ld + lane + 32 * q];
#pragma unroll
            for (int rr = 0; rr < RPW; ++rr) {
                const float4 y = *reinterpret_cast<const float4 *>(Ys + (row0 + rr) * ys_ld + k);
#pragma unroll
                for (int q = 0; q < Q; ++q) {
                    acc[rr][q] = __fmaf_rn(y.x, m[0][q], acc[rr][q]);
                    acc[rr][q] = __fmaf_rn(y.y, m[1][q], acc[rr][q]);
                    acc[rr][q] = __fmaf_rn(y.z, m[2][q], acc[rr][q]);
                    acc[rr][q] = __fmaf_rn(y.w, m[3][q], acc[rr][q]);
                }
            }
        }
    }
    for (; k < kend; ++k) {
        T m[Q];
#pragma unroll
        for (int q = 0; q < Q; ++q) m[q] = Ms[(k - kbeg) * ms_ld + lane + 32 * q];
#pragma unroll
        for (int rr = 0; rr < RPW; ++rr) {
            const T y = Ys[(row0 + rr) * ys_ld + k];
#pragma unroll
            for (int q = 0; q < Q; ++q) acc[rr][q] = fma_rn(y, m[q], acc[rr][q]);
        }
    }
}

// The unrotated functions (8, 10): acc[rr][q] = Y[row0+rr][lane + 32q] (0 past D).
template <typename T, int Q, int RPW>
__device__ __forceinline__ void eval_identity(T (&acc)[RPW][Q], const T *__restrict__ Ys, int ys_ld, int row0, int D,
                                              int lane)
{
#pragma unroll
    for (int rr = 0; rr < RPW; ++rr)
#pragma unroll
        for (int q = 0; q < Q; ++q) acc[rr][q] = lane + 32 * q < D ? Ys[(row0 + rr) * ys_ld + lane + 32 * q] : T(0);
}

// One row's objective, z_j in lane j % 32 of element j / 32 (all lanes call it together). Out of
// line, so that the kernels' per-coordinate-sum path carries none of its registers or stack.
template <typename T, int Q> struct ZRow {
    T v[Q];
};
template <typename T, int Q>
__device__ __noinline__ T row_objective_warp(ZRow<T, Q> z, int D, int func_id, int lane)
{
    const T z0 = __shfl_sync(0xffffffffu, z.v[0], 0);
    RowAcc<T> a;
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const T dn = __shfl_down_sync(0xffffffffu, z.v[q], 1);
        const T up = q + 1 < Q ? __shfl_sync(0xffffffffu, z.v[q + 1 < Q ? q + 1 : q], 0) : z0;
        const int j = lane + 32 * q;
        const T zn = j == D - 1 ? z0 : (lane < 31 ? dn : up);
        if (j < D) row_push(a, func_id, j, z.v[q], zn, D);
    }
    a.s1 = warp_sum(a.s1);
    a.s2 = warp_sum(a.s2);
    a.p = warp_prod(a.p);
    return row_finish(a, func_id, D);
}

// f[rr] = objective of the row whose column j = lane + 32q holds scale * acc[rr][q] (+ the fixed
// shift); result valid on every lane. Sums of per-coordinate terms (8, 9, 31) add each lane's
// columns in order and then reduce across the warp; the other functions run the row accumulator
// per lane, with the next coordinate fetched from the neighbouring lane.
// kGeneric = false compiles the per-coordinate-sum path alone (the caller guarantees such an id), so
// the hot kernels carry none of the row accumulator's code.
template <typename T, int Q, int RPW, bool kGeneric = true>
__device__ __forceinline__ void eval_reduce(const T (&acc)[RPW][Q], int D, int func_id, T scale, int lane, T (&f)[RPW])
{
    if (!kGeneric || func_sum_form(func_id)) {
#pragma unroll
        for (int rr = 0; rr < RPW; ++rr) {
            T s = T(0);
#pragma unroll
            for (int q = 0; q < Q; ++q)
                if (lane + 32 * q < D) s += obj_term(func_id, acc[rr][q] * scale);
            f[rr] = warp_sum(s);
        }
        return;
    }
    if constexpr (kGeneric) {
        const T fs = func_fixed_shift<T>(func_id);
#pragma unroll
        for (int rr = 0; rr < RPW; ++rr) {
            ZRow<T, Q> z;
#pragma unroll
            for (int q = 0; q < Q; ++q) z.v[q] = acc[rr][q] * scale + fs;
            f[rr] = row_objective_warp<T, Q>(z, D, func_id, lane);
        }
    }
}

// Cooperative copy of M^T rows [kbeg, kend) into Ms (row stride ms_ld = 32*Q), zero-padding
// columns D .. 32Q-1. rot rows are ld_rot apart.
template <typename T, int Q>
__device__ __forceinline__ void load_rot_rows(T *__restrict__ Ms, const T *__restrict__ rot, int ld_rot, int D,
                                              int kbeg, int kend)
{
    constexpr int W = 32 * Q;
    const int n = (kend - kbeg) * W;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int kk = i / W, j = i - kk * W;
        Ms[i] = j < D ? rot[(size_t)(kbeg + kk) * ld_rot + j] : T(0);
    }
}

}  // namespace speo
