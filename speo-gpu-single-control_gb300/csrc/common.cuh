// common.cuh -- device helpers shared by the sm_103a kernels of libspeo_gb300.
//
// Counter-based Philox-4x32-10 draws, the DE mutation/reflection element rules
// (reference: CUDA_EA_library/kernel_DE_CUDA.cu:160-276), objective terms and the
// bounded-loop error flags.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/speo_gb300.h"

namespace speo {

constexpr int kRedrawIters = 4096;  // bound of the distinct-index rejection loop
constexpr int kBoundIters = 64;     // bound of the reflection loop

constexpr uint32_t kTagIdx = 1u;
constexpr uint32_t kTagCr = 2u;
constexpr uint32_t kTagInit = 3u;
constexpr uint32_t kTagSample = 4u;  // surrogate training batches

// ---------------------------------------------------------------------------------------
// Philox-4x32-10 (Salmon et al., SC'11). Ten rounds, Weyl key schedule.
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ uint4 philox(uint4 c, uint2 k)
{
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r) { k.x += 0x9E3779B9u; k.y += 0xBB67AE85u; }
        const uint32_t hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
        const uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
        c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
    }
    return c;
}

// Out-of-line copy for the rarely refilled index-draw stream: keeps one Philox body in the
// instruction stream instead of one per draw site (IdxStreamT<true> refills inline instead).
__device__ __noinline__ static uint4 philox_block(uint4 c, uint2 k) { return philox(c, k); }

__device__ __forceinline__ uint2 seed_key(uint64_t seed)
{
    return make_uint2((uint32_t)seed, (uint32_t)(seed >> 32));
}

// u32 -> (0, 1]: ((w >> 8) + 1) * 2^-24, exact in binary32.
__device__ __forceinline__ float u01(uint32_t w)
{
    return __fmul_rn(__uint2float_rn((w >> 8) + 1u), 5.9604644775390625e-8f);
}

__device__ __forceinline__ uint32_t pick(uint4 v, uint32_t i)
{
    return i == 0 ? v.x : i == 1 ? v.y : i == 2 ? v.z : v.w;
}

// Sequential index-draw stream of one target: draw k is word k%4 of
// philox({k/4, row, gen, tag}, key). Inline: the refill in line rather than through the
// out-of-line philox_block (faster in the island-resident tensor-core kernel, whose register
// state an out-of-line call saves through local memory; slower in the others).
template <bool Inline>
struct IdxStreamT {
    uint2 key;
    uint32_t row, gen, tag;
    uint32_t k;
    uint4 blk;
    __device__ __forceinline__ IdxStreamT(uint2 key_, uint32_t row_, uint32_t gen_, uint32_t tag_)
        : key(key_), row(row_), gen(gen_), tag(tag_), k(0), blk(make_uint4(0, 0, 0, 0)) {}
    __device__ __forceinline__ float next()
    {
        if ((k & 3u) == 0)
            blk = Inline ? philox(make_uint4(k >> 2, row, gen, tag), key)
                         : philox_block(make_uint4(k >> 2, row, gen, tag), key);
        const float u = u01(pick(blk, k & 3u));
        ++k;
        return u;
    }
    // (int)(u * n) in binary32, as kernel_DE_CUDA.cu:193 (GPU_SINGLE_PRECISION build).
    __device__ __forceinline__ int index(int n) { return (int)__fmul_rn(next(), (float)n); }
};
using IdxStream = IdxStreamT<false>;

// The five donor positions of kernel_DE_CUDA.cu:187-212, in [0, S), including the reference's
// sequential (not pairwise-complete) distinctness check. Returns false if the bounded
// rejection loop gave up.
template <typename Stream>
__device__ __forceinline__ bool draw_donors(Stream &s, int S, int r[5])
{
    bool ok = true;
#pragma unroll 1
    for (int i = 0; i < 5; ++i) {
        r[i] = s.index(S);
        if (r[i] == S) r[i]--;
#pragma unroll 1
        for (int j = 0; j < i; ++j) {
            int guard = 0;
            while (r[i] == r[j]) {
                r[i] = s.index(S);
                if (++guard >= kRedrawIters) { ok = false; break; }
            }
        }
        if (r[i] == S) r[i]--;
    }
    return ok;
}

// draw_donors followed by index(D) (jrand) on one IdxStream, with the common case made short: the
// first eight draws come from two Philox blocks computed side by side; when the five donors of
// words 0-4 are distinct, the sequential algorithm redraws nothing, so they and word 5 (jrand)
// are its result; otherwise it runs from the start of the stream.
__device__ __forceinline__ bool draw_donors_jrand(uint2 key, uint32_t row, uint32_t gen, uint32_t tag, int S, int D,
                                                  int r[5], int &jrand)
{
    const uint4 b0 = philox(make_uint4(0u, row, gen, tag), key);
    const uint4 b1 = philox(make_uint4(1u, row, gen, tag), key);
    const uint32_t w[5] = {b0.x, b0.y, b0.z, b0.w, b1.x};
    bool distinct = true;
#pragma unroll
    for (int i = 0; i < 5; ++i) {
        const int v = (int)__fmul_rn(u01(w[i]), (float)S);
        r[i] = v == S ? S - 1 : v;
#pragma unroll
        for (int j = 0; j < i; ++j) distinct &= r[i] != r[j];
    }
    if (distinct) {
        jrand = (int)__fmul_rn(u01(b1.y), (float)D);
        return true;
    }
    IdxStreamT<true> is(key, row, gen, tag);
    const bool ok = draw_donors(is, S, r);
    jrand = is.index(D);
    return ok;
}

// device_CheckBound (kernel_DE_CUDA.cu:160-170), bounded.
template <typename T>
__device__ __forceinline__ T check_bound(T v, T lb, T ub, bool &ok)
{
    // the loop's first pass as selects (a value in bounds passes through unchanged), the rest
    // only for a value still outside after one reflection each way
    v = (v < lb) ? lb + (lb - v) : v;
    v = (v > ub) ? ub - (v - ub) : v;
    int it = 1;
    while ((v < lb) || (v > ub)) {
        if (v < lb) v = lb + (lb - v);
        if (v > ub) v = ub - (v - ub);
        if (++it >= kBoundIters) { ok = false; v = lb; break; }
    }
    return v;
}

__device__ __forceinline__ float fma_rn(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fma_rn(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }

// Mutant element for strategy st (kernel_DE_CUDA.cu:243-276): terms added left to right,
// each F*(a-b) fused into the running sum.
template <typename T>
__device__ __forceinline__ T mutant(int st, T F, T xi, T xb, const T xr[5])
{
    T v;
    switch (st) {
    case 0: v = fma_rn(F, sub_rn(xr[0], xr[1]), xi); break;
    case 1: v = fma_rn(F, sub_rn(xr[2], xr[3]), fma_rn(F, sub_rn(xr[0], xr[1]), xi)); break;
    case 2: v = fma_rn(F, sub_rn(xr[0], xr[1]), fma_rn(F, sub_rn(xb, xi), xi)); break;
    case 3:
        v = fma_rn(F, sub_rn(xr[1], xr[2]), fma_rn(F, sub_rn(xr[0], xr[1]), fma_rn(F, sub_rn(xb, xi), xi)));
        break;
    case 4: v = fma_rn(F, sub_rn(xr[1], xr[2]), xr[0]); break;
    case 5: v = fma_rn(F, sub_rn(xr[3], xr[4]), fma_rn(F, sub_rn(xr[1], xr[2]), xr[0])); break;
    case 6: v = fma_rn(F, sub_rn(xr[0], xr[1]), xb); break;
    case 7: v = fma_rn(F, sub_rn(xr[2], xr[3]), fma_rn(F, sub_rn(xr[0], xr[1]), xb)); break;
    case 8: v = fma_rn(F, sub_rn(xr[1], xr[2]), fma_rn(F, sub_rn(xr[0], xi), xi)); break;
    default: v = xi; break;
    }
    return v;
}

__host__ __device__ __forceinline__ bool strategy_uses_best(int st)
{
    return st == 2 || st == 3 || st == 6 || st == 7;
}

// ---- CEC2014 functions 1-16 and the rotated sphere (31) -------------------------------------
// The reference's EvaluateFitness dispatch (CUDA_EA_library/CEC2014.cc:14-144): each id shifts,
// scales by a rate, rotates (all but 8 and 10) and, for 4 and 15, adds a fixed shift of 1 before
// the function body. z = rate * M (x - o) here (the same value as the reference's M (rate (x - o))
// up to rounding).
__host__ __device__ __forceinline__ bool func_supported(int f) { return (f >= 1 && f <= 16) || f == 31; }
__host__ __device__ __forceinline__ bool func_rotated(int f) { return f != 8 && f != 10; }
// Sums of one term per coordinate (8, 9, 31): the kernels' fast path; the others take the row
// accumulator below.
__host__ __device__ __forceinline__ bool func_sum_form(int f) { return f == 8 || f == 9 || f == 31; }
__host__ __device__ __forceinline__ double func_scale_f64(int f)
{
    switch (f) {
    case 4: return 2.048 / 100.0;
    case 6: return 0.5 / 100.0;
    case 7: return 6.0;
    case 8: case 9: return 5.12 / 100.0;
    case 10: case 11: return 10.0;
    case 12: case 13: case 14: case 15: return 5.0 / 100.0;
    default: return 1.0;
    }
}
__host__ __device__ __forceinline__ float func_scale(int f) { return (float)func_scale_f64(f); }
template <typename T>
__host__ __device__ __forceinline__ T func_fixed_shift(int f) { return (f == 4 || f == 15) ? T(1) : T(0); }

// sin(pi r) for |r| <= 1/2 from its Taylor series, odd terms through r^11 (truncation
// (pi/2)^13 / 13! < 6e-8 relative at |r| = 1/2, exact limit r -> 0), Horner in r^2.
__device__ __forceinline__ float sin_pi_reduced(float r)
{
    const float r2 = r * r;
    float p = -7.3704309762e-03f;            // -pi^11 / 11!
    p = __fmaf_rn(p, r2, 8.2145884633e-02f);  //  pi^9 / 9!
    p = __fmaf_rn(p, r2, -5.9926450253e-01f); // -pi^7 / 7!
    p = __fmaf_rn(p, r2, 2.5501639843e+00f);  //  pi^5 / 5!
    p = __fmaf_rn(p, r2, -5.1677126884e+00f); // -pi^3 / 3!
    p = __fmaf_rn(p, r2, 3.1415927410e+00f);  //  pi
    return r * p;                             // max relative error 1.3e-7 on [-1/2, 1/2]
}

// Per-coordinate objective term. Rastrigin's z^2 - 10 cos(2 pi z) + 10 (CEC2014.cc:680) is
// computed as z^2 + 20 sin^2(pi z), the same function without the cancellation at z ~ 0; the
// sine is reduced exactly (z - rint(z), exact in binary32 for |z| < 2^23; sin^2 has period 1).
__device__ __forceinline__ float obj_term(int func_id, float z)
{
    if (func_id == SPEO_FUNC_ROTATED_RASTRIGIN || func_id == 8) {
        const float s = sin_pi_reduced(__fsub_rn(z, rintf(z)));
        return __fmaf_rn(z, z, 20.0f * s * s);
    }
    return z * z;
}
__device__ __forceinline__ double obj_term(int func_id, double z)
{
    if (func_id == SPEO_FUNC_ROTATED_RASTRIGIN || func_id == 8) {
        const double s = sinpi(z);
        return z * z + 20.0 * s * s;
    }
    return z * z;
}

// Row objective as a streaming accumulator: push(j, z_j, z_next) for each coordinate (z_next =
// z_{j+1}, or z_0 for the last coordinate), partial states combine by sum / product, finish(D)
// applies the function's outer formula. Function bodies follow CEC2014.cc: ellips :481-497, bent
// cigar :499-516, discus :518-531, Rosenbrock :552-567, Ackley :590-613, Weierstrass :615-644,
// Griewank :646-666, Rastrigin :668-683, Schwefel :705-737, Katsuura :739-763, Griewank-Rosenbrock
// :842-868, expanded Scaffer F6 :870-905, HappyCat :907-929, HGBat :931-953, sphere :462-478.
// Weierstrass and Katsuura reduce their high harmonics (arguments amplified by up to 3^20 and
// 2^32) exactly: in integer arithmetic (FP32) or in FP64.
// Weierstrass' inner sum for a binary32 z: sum_{k=0}^{20} 0.5^k cos(2 pi 3^k (z + 1/2)) =
// -sum_k 0.5^k cos(2 pi frac(3^k |z|)) (3^k is odd and cos is even). frac(3^k |z|) is exact:
// |z| = m 2^e with m < 2^24, and 3^k m < 2^56 is an exact 64-bit product whose bits below the
// binary point are the fraction; only the cosine of the reduced argument is rounded.
__device__ __forceinline__ float weierstrass_sum_f32(float z)
{
    const float az = fabsf(z);
    if (!(az < __int_as_float(0x7f800000))) return z - z;  // inf / NaN -> NaN
    if (az == 0.f) return -(2.f - 9.5367431640625e-07f);
    int e;
    const float mf = frexpf(az, &e);                              // az = mf 2^e, mf in [0.5, 1)
    unsigned long long p = (unsigned long long)(mf * 16777216.f); // exact, < 2^24
    e -= 24;                                                      // az = p 2^e
    if (e >= 0) return -(2.f - 9.5367431640625e-07f);             // an integer: every cosine is 1
    const unsigned long long mask = -e >= 64 ? ~0ull : (1ull << -e) - 1ull;
    float s = 0.f, ak = 1.f;
#pragma unroll 1
    for (int k = 0; k <= 20; ++k) {
        const float fr = ldexpf(__ull2float_rn(p & mask), e);    // frac(3^k |z|)
        s = __fmaf_rn(ak, cospif(2.f * fr), s);
        ak *= 0.5f;
        p *= 3ull;
    }
    return -s;
}

template <typename T> struct RowAcc {
    T s1 = T(0), s2 = T(0), p = T(1);
};

__device__ __forceinline__ float cos2pi(float z) { return cospif(2.f * z); }
__device__ __forceinline__ double cos2pi(double z) { return cospi(2.0 * z); }

template <typename T>
__device__ __forceinline__ void row_push(RowAcc<T> &a, int f, int j, T z, T zn, int D)
{
    switch (f) {
    case 1: {
        // 10^(6j/(D-1)); exp10 rather than pow(10, .): the same value to an ulp at a fraction of the cost
        const T w = sizeof(T) == 4 ? (T)exp10f(6.f * (float)j / (float)(D - 1)) : (T)exp10(6.0 * j / (D - 1));
        a.s1 += w * z * z;
        break;
    }
    case 2: a.s1 += (j == 0 ? T(1) : T(1e6)) * z * z; break;
    case 3: a.s1 += (j == 0 ? T(1e6) : T(1)) * z * z; break;
    case 4:
        if (j < D - 1) {
            const T t1 = z * z - zn, t2 = z - T(1);
            a.s1 += T(100) * t1 * t1 + t2 * t2;
        }
        break;
    case 5: a.s1 += z * z; a.s2 += cos2pi(z); break;
    case 6:
        if constexpr (sizeof(T) == 4) {
            a.s1 += weierstrass_sum_f32(z);
        } else {
            double s = 0.0, ak = 1.0, bk = 1.0;
            for (int k = 0; k <= 20; ++k) {
                s += ak * cospi(2.0 * bk * ((double)z + 0.5));
                ak *= 0.5;
                bk *= 3.0;
            }
            a.s1 += (T)s;
        }
        break;
    case 7: a.s1 += z * z; a.p *= cos(z / sqrt(T(j + 1))); break;
    case 10: case 11: {
        const T zi = z + T(4.209687462275036e+002);
        if (zi > T(500)) {
            const T m = T(500) - fmod(zi, T(500));
            a.s1 -= m * sin(sqrt(m));
            const T t = (zi - T(500)) / T(100);
            a.s1 += t * t / T(D);
        } else if (zi < T(-500)) {
            const T m = fmod(fabs(zi), T(500));
            a.s1 -= (T(-500) + m) * sin(sqrt(T(500) - m));
            const T t = (zi + T(500)) / T(100);
            a.s1 += t * t / T(D);
        } else {
            a.s1 -= zi * sin(sqrt(fabs(zi)));
        }
        break;
    }
    case 12:
        if constexpr (sizeof(T) == 4) {
            // 2^k z, its distance to the nearest integer and the division by 2^k are exact in binary32
            float t = 0.f;
            for (int k = 1; k <= 32; ++k) {
                const float b = ldexpf(z, k);
                t += ldexpf(fabsf(b - rintf(b)), -k);
            }
            a.p *= powf(1.f + (float)(j + 1) * t, 10.f / powf((float)D, 1.2f));
        } else {
            double t = 0.0, p2 = 1.0;
            for (int k = 1; k <= 32; ++k) {
                p2 *= 2.0;
                const double b = p2 * (double)z;
                t += fabs(b - floor(b + 0.5)) / p2;
            }
            a.p *= (T)pow(1.0 + (j + 1) * t, 10.0 / pow((double)D, 1.2));
        }
        break;
    case 13: case 14: {
        const T zz = z - T(1);
        a.s1 += zz * zz;
        a.s2 += zz;
        break;
    }
    case 15: {
        const T t1 = z * z - zn, t2 = z - T(1);
        const T t = T(100) * t1 * t1 + t2 * t2;
        a.s1 += (t * t) / T(4000) - cos(t) + T(1);
        break;
    }
    case 16: {
        const T s2 = D == 1 ? z * z : z * z + zn * zn;
        const T t1 = sin(sqrt(s2)), t2 = T(1) + T(0.001) * s2;
        a.s1 += T(0.5) + (t1 * t1 - T(0.5)) / (t2 * t2);
        break;
    }
    default: a.s1 += obj_term(f, z); break;  // 8, 9, 31: sum of per-coordinate terms
    }
}

template <typename T>
__device__ __forceinline__ T row_finish(const RowAcc<T> &a, int f, int D)
{
    switch (f) {
    case 5:
        return T(2.7182818284590452354) - T(20) * exp(T(-0.2) * sqrt(a.s1 / T(D))) + T(20) - exp(a.s2 / T(D));
    case 6: return a.s1 + T(D) * (T(2) - T(9.5367431640625e-07));  // - D sum_k 0.5^k cos(pi 3^k)
    case 7: return T(1) + a.s1 / T(4000) - a.p;
    case 10: case 11: return a.s1 + T(4.189828872724338e+002) * T(D);
    case 12: {
        const T c = T(10) / T(D) / T(D);
        return a.p * c - c;
    }
    case 13: return pow(fabs(a.s1 - T(D)), T(0.25)) + (T(0.5) * a.s1 + a.s2) / T(D) + T(0.5);
    case 14: return sqrt(fabs(a.s1 * a.s1 - a.s2 * a.s2)) + (T(0.5) * a.s1 + a.s2) / T(D) + T(0.5);
    default: return a.s1;
    }
}

__device__ __forceinline__ float warp_sum(float v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

template <typename T>
__device__ __forceinline__ T warp_prod(T v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v *= __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// NaN ranks as +inf in every best/worst search.
__device__ __forceinline__ float rank_key(float f) { return isnan(f) ? __int_as_float(0x7f800000) : f; }

// (f, row) "better" order: smaller f, then smaller row.
__device__ __forceinline__ bool better(float fa, long long ra, float fb, long long rb)
{
    return fa < fb || (fa == fb && ra < rb);
}

}  // namespace speo

// Per-translation-unit device error word; the host accessor returns its device address (on the
// current device), which speo_device_error_bits reads and clears with one gather kernel.
#define SPEO_DEFINE_DEVERR(name)                                                         \
    static __device__ unsigned int s_deverr;                                             \
    extern "C" void *name(void)                                                          \
    {                                                                                    \
        void *p = nullptr;                                                               \
        if (cudaGetSymbolAddress(&p, s_deverr) != cudaSuccess) {                          \
            cudaGetLastError();                                                          \
            return nullptr;                                                              \
        }                                                                                \
        return p;                                                                        \
    }
