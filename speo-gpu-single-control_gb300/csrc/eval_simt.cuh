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

// f[rr] = sum over columns j < D of term(scale * acc[rr][j]); result valid on every lane.
template <typename T, int Q, int RPW>
__device__ __forceinline__ void eval_reduce(const T (&acc)[RPW][Q], int D, int func_id, T scale, int lane, T (&f)[RPW])
{
#pragma unroll
    for (int rr = 0; rr < RPW; ++rr) {
        T s = T(0);
#pragma unroll
        for (int q = 0; q < Q; ++q)
            if (lane + 32 * q < D) s += obj_term(func_id, acc[rr][q] * scale);
        f[rr] = warp_sum(s);
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
