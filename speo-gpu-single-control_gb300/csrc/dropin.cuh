// dropin.cuh -- helpers shared by the kernels of the reference-shaped drop-in path: the DEInfo
// type per precision, the generation-counter advance, 16-byte vectors of `real`, the donor count
// per strategy and the exact integer form of the crossover test.
#pragma once

#include "common.cuh"
#include "host.h"

namespace speo {

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

template <typename T>
__device__ __forceinline__ T rank_t(T f) { return isnan(f) ? T(INFINITY) : f; }

template <typename T> struct Vec;
template <> struct Vec<float> { using type = float4; static constexpr int n = 4; };
template <> struct Vec<double> { using type = double2; static constexpr int n = 2; };

template <typename T>
__device__ __forceinline__ T vget(const typename Vec<T>::type &v, int q)
{
    if constexpr (Vec<T>::n == 4) return q == 0 ? v.x : q == 1 ? v.y : q == 2 ? v.z : v.w;
    else return q == 0 ? v.x : v.y;
}
template <typename T>
__device__ __forceinline__ void vset(typename Vec<T>::type &v, int q, T x)
{
    if constexpr (Vec<T>::n == 4) { if (q == 0) v.x = x; else if (q == 1) v.y = x; else if (q == 2) v.z = x; else v.w = x; }
    else { if (q == 0) v.x = x; else v.y = x; }
}

__device__ __forceinline__ int ndonors(int st)
{
    switch (st) {
    case 0: case 2: case 6: return 2;
    case 3: case 4: case 8: return 3;
    case 1: case 7: return 4;
    default: return 5;
    }
}

// Crossover test `(T)u01(w) < CR` as an integer compare: u01(w) = k * 2^-24 with
// k = (w >> 8) + 1, so u < CR  <=>  k < CR * 2^24  <=>  k < ceil(CR * 2^24) for integer k (the
// scaling by 2^24 is exact). NaN CR takes no element, as the float compare does.
template <typename T>
__device__ __forceinline__ uint32_t cr_threshold(T CR)
{
    const T x = ceil(CR * (T)16777216.0);
    if (!(x > (T)0)) return 0u;               // also NaN
    return x >= (T)33554432.0 ? 33554432u : (uint32_t)x;
}
__device__ __forceinline__ bool cr_take(uint32_t w, uint32_t thr) { return (w >> 8) + 1u < thr; }

}  // namespace speo
