// tc_split.cuh -- the pieces of the split-FP16 tensor-core rotation that every kernel using it
// shares, so that the same rows give bit-identical fitness whichever kernel evaluates them.
//
// Each operand is scaled by a power of two and split two ways into FP16: v 2^k = v_hi + v_lo +
// O(2^-22 |v 2^k|), v_hi the FP16 rounding of v 2^k and v_lo that of the (exact) remainder. A row
// y = x - o of the A operand takes its own exponent k (the largest |y_j| of the row lands in
// [2^14, 2^15), so no part overflows FP16 and the low parts of the row's large elements stay
// normal); M (B operand, one exponent per instance) likewise. Per 16-wide K step three products,
// smallest first: y_lo M_hi, y_hi M_lo, y_hi M_hi; the term left out (y_lo M_lo) is ~2^-22 of the
// leading one. The FP32 accumulator holds z 2^(k_row + k_M); the epilogue multiplies by
// scale 2^-(k_row + k_M) (exact powers of two: the same rounding as z * scale). The rotation
// carries the FP32 accumulation's rounding like a CUDA-core rotation (fitness within 1e-5 of
// FP64), with half the tensor work and two thirds of the operand storage of a three-way BF16
// split, whose exponent range needs no scaling but whose 8-bit significands need six products.
//
// Replaces global_ShiftAndRotation + global_f8 (CUDA_EA_library/kernel_CEC2014_CUDA.cu:147-181,
// 557-587).
#pragma once

#include <cuda_fp16.h>

#include "common.cuh"
#include "tcgen05.cuh"

namespace speo {
namespace tcs {

constexpr int kTileM = 128;   // MMA rows (one TMEM lane per row)
constexpr int kParts = 2;     // FP16 parts per operand

__host__ __device__ __forceinline__ int round16(int x) { return (x + 15) & ~15; }

// 2^k as a binary32, exact for -149 <= k <= 127.
__device__ __forceinline__ float pow2i(int k)
{
    return k >= -126 ? __uint_as_float((uint32_t)(k + 127) << 23) : __uint_as_float(1u << (k + 149));
}

// The exponent k that brings the largest magnitude m (>= 0) of a row or matrix into [2^14, 2^15):
// 14 - floor(log2 m) for a normal m, at most 127 (m subnormal); 0 when m is 0 or not finite (a
// row holding an infinity evaluates to a non-finite fitness either way).
__device__ __forceinline__ int scale_exp(float m)
{
    const uint32_t b = __float_as_uint(m);
    const int e = (int)(b >> 23);
    if (b == 0u || e >= 255) return 0;
    const int k = 14 - (e == 0 ? -127 : e - 127);
    return k > 127 ? 127 : k;
}

// The epilogue's multiplier of a row: the objective's input scale fs times 2^-(k_M + k_row), in
// this order (exact unless it underflows).
__device__ __forceinline__ float row_scale(float fs, int k_m, int k_row) { return fs * pow2i(-k_m) * pow2i(-k_row); }

// FP16 two-way split of the pair (a, b), packed two per 32-bit word (a in the low half):
// a = hi.x + lo.x + O(2^-22 |a|) for |a| < 2^15; a - hi.x is exact in binary32.
__device__ __forceinline__ void split2h(float a, float b, uint32_t &hi, uint32_t &lo)
{
    const __half2 h = __floats2half2_rn(a, b);
    const float2 hf = __half22float2(h);
    const __half2 l = __floats2half2_rn(a - hf.x, b - hf.y);
    hi = *reinterpret_cast<const uint32_t *>(&h);
    lo = *reinterpret_cast<const uint32_t *>(&l);
}

// The exponent k_M of M's scale: 14 while the largest |M[n][k]| lies in [2^-6, 2) (2^14 M then stays
// below 2^15 and its low parts stay normal, so B can be built in the same pass that finds the
// largest value), else the general rule scale_exp.
__device__ __forceinline__ int b_exp(float m) { return (m >= 0.015625f && m < 2.f) ? 14 : scale_exp(m); }

// Largest |M[n][k]| = |rot[k*ld_rot + n]| over the entries thread t of `nthr` visits (the caller
// reduces the threads' values and takes k_M = b_exp of the maximum).
__device__ __forceinline__ float b_absmax(const speo_segment &s, int t, int nthr)
{
    const int D = s.dim;
    float m = 0.f;
    for (int i = t; i < D * D; i += nthr) {
        const int k = i / D, n = i - k * D;
        m = fmaxf(m, fabsf(s.rot[(size_t)k * s.ld_rot + n]));
    }
    return m;
}

// Builds B = split2(M 2^k_M) (mscale = 2^k_M) for an instance with `nthr` threads (index t):
// B[n][k] = M[n][k] = rot[k*ld_rot + n] (zero past D), and the shift o. The parts are b_bytes apart.
// Returns the largest |M[n][k]| this thread read (for b_exp after the threads' reduction).
__device__ __forceinline__ float build_b(const speo_segment &s, int Kp, uint8_t *b_hi, size_t b_bytes, float *so, int t,
                                         int nthr, float mscale)
{
    const int D = s.dim;
    const int pairs = Kp * (Kp / 8);
    float mx = 0.f;
    for (int i = t; i < pairs; i += nthr) {
        const int n = i % Kp, kc = i / Kp;
        float v[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) {
            const int k = 8 * kc + e;
            const float mv = (n < D && k < D) ? s.rot[(size_t)k * s.ld_rot + n] : 0.f;
            mx = fmaxf(mx, fabsf(mv));
            v[e] = mv * mscale;
        }
        uint32_t h[4], l[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) split2h(v[2 * e], v[2 * e + 1], h[e], l[e]);
        const uint32_t off = tc::kmajor_offset(n, 8 * kc, Kp);
        *reinterpret_cast<uint4 *>(b_hi + off) = make_uint4(h[0], h[1], h[2], h[3]);
        *reinterpret_cast<uint4 *>(b_hi + b_bytes + off) = make_uint4(l[0], l[1], l[2], l[3]);
    }
    for (int k = t; k < Kp; k += nthr) so[k] = k < D ? s.shift[k] : 0.f;
    return mx;
}

// y = x - o over the 16 columns k0 .. k0+15 of a staged row (zero past D or for a dead row); whole
// 4-column groups two columns per packed subtraction (the same rounding as one at a time).
__device__ __forceinline__ void load_y16(const float *row, const float *so, int k0, int D, bool live, float (&v)[16])
{
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const float4 x = reinterpret_cast<const float4 *>(row + k0)[q];
        const float4 o = reinterpret_cast<const float4 *>(so + k0)[q];
        const int k = k0 + 4 * q;
        if (live && k + 4 <= D) {
            tc::upk2(tc::sub2(tc::pk2(x.x, x.y), tc::pk2(o.x, o.y)), v[4 * q + 0], v[4 * q + 1]);
            tc::upk2(tc::sub2(tc::pk2(x.z, x.w), tc::pk2(o.z, o.w)), v[4 * q + 2], v[4 * q + 3]);
        } else {
            v[4 * q + 0] = (live && k + 0 < D) ? __fsub_rn(x.x, o.x) : 0.f;
            v[4 * q + 1] = (live && k + 1 < D) ? __fsub_rn(x.y, o.y) : 0.f;
            v[4 * q + 2] = (live && k + 2 < D) ? __fsub_rn(x.z, o.z) : 0.f;
            v[4 * q + 3] = (live && k + 3 < D) ? __fsub_rn(x.w, o.w) : 0.f;
        }
    }
}

__device__ __forceinline__ float absmax16(const float (&v)[16])
{
    float m = 0.f;
#pragma unroll
    for (int e = 0; e < 16; ++e) m = fmaxf(m, fabsf(v[e]));
    return m;
}

// One K step of the A operand from its 16 values of y: scaled by the row's power of two `rs` and
// split two ways into FP16 hi / lo, packed two per 32-bit word (even k in the low half), as
// tcgen05.mma reads A from tensor memory. The scaling and the remainder run two columns per packed
// operation (exact either way: a power-of-two product, a remainder exact in binary32).
__device__ __forceinline__ void split16(const float (&v)[16], float rs, uint32_t (&hi)[8], uint32_t (&lo)[8])
{
    const uint64_t s2 = tc::pk2(rs, rs);
#pragma unroll
    for (int p = 0; p < 8; ++p) {
        const uint64_t a = tc::mul2(tc::pk2(v[2 * p], v[2 * p + 1]), s2);
        float a0, a1;
        tc::upk2(a, a0, a1);
        const __half2 h = __floats2half2_rn(a0, a1);
        const float2 hf = __half22float2(h);
        float r0, r1;
        tc::upk2(tc::sub2(a, tc::pk2(hf.x, hf.y)), r0, r1);
        const __half2 l = __floats2half2_rn(r0, r1);
        hi[p] = *reinterpret_cast<const uint32_t *>(&h);
        lo[p] = *reinterpret_cast<const uint32_t *>(&l);
    }
}

// Largest |x_k - o_k| over the steps of columns [k0, k1) (multiples of 16; k < D) of a staged
// row; 0 for a dead row. The subtraction is the conversion's, so the maximum is of the values split.
__device__ __forceinline__ float row_absmax(const float *row, const float *so, int k0, int k1, int D, bool live)
{
    float m = 0.f;
    if (!live) return m;
    for (int k = k0; k < k1 && k < D; k += 16) {
        float v[16];
        load_y16(row, so, k, D, true, v);
        m = fmaxf(m, absmax16(v));
    }
    return m;
}

// load_y16 + split16.
__device__ __forceinline__ void convert16(const float *row, const float *so, int k0, int D, bool live, float rs,
                                          uint32_t (&hi)[8], uint32_t (&lo)[8])
{
    float v[16];
    load_y16(row, so, k0, D, live, v);
    split16(v, rs, hi, lo);
}

// One thread: the three split products over K steps [s0, s1) into the TMEM accumulator (step 0
// overwrites it), smallest first; A hi / lo in tensor memory at a_hi + {0, 1} apart (8 columns per
// step, step s at 8 s), B hi / lo in shared memory b_bytes apart.
__device__ __forceinline__ void issue_split_mma(uint32_t acc, uint32_t a_hi, uint32_t apart, const uint8_t *b_hi,
                                                size_t b_bytes, int Kp, int Np, int s0, int s1)
{
    const uint32_t idesc = tc::idesc_f16_f32(kTileM, Np);
    const uint32_t sbo = (uint32_t)Kp * 16;  // 8-row groups
    const uint32_t lbo = 128;                // adjacent core matrices along K
    // a K step moves B by two core matrices (256 B: 16 in the descriptor's address field, which
    // holds smem address >> 4 and cannot carry for addresses below 256 KB) and A by 8 columns
    const uint32_t b0 = tc::smem_u32(b_hi) + (uint32_t)s0 * 256u;
    uint64_t dh = tc::smem_desc(b0, lbo, sbo);
    uint64_t dl = tc::smem_desc(b0 + (uint32_t)b_bytes, lbo, sbo);
    uint32_t ah = a_hi + (uint32_t)s0 * 8u, al = ah + apart;
    for (int s = s0; s < s1; ++s) {
        tc::mma_bf16_ta(acc, al, dh, idesc, s > 0);
        tc::mma_bf16_ta(acc, ah, dl, idesc, 1);
        tc::mma_bf16_ta(acc, ah, dh, idesc, 1);
        dh += 16;
        dl += 16;
        ah += 8;
        al += 8;
    }
}

// Two objective terms at once (f32x2): z - rint(z) (rint by adding and subtracting 1.5 * 2^23,
// exact for |z| < 2^22), sin(pi r) = r P(r^2) with P of degree 4, and z*z + (20 s) s. P is a
// near-minimax fit of sin(pi r) / r over |r| <= 1/2 (iteratively reweighted least squares on
// Chebyshev nodes, relative weights): evaluated in FP32 its relative error is 1.8e-7, the same as
// the degree-11 Taylor sine of the CUDA-core objective (one fused multiply-add fewer per pair).
__device__ __forceinline__ uint64_t obj_term2(int func, uint64_t z)
{
    using namespace tc;
    if (func != SPEO_FUNC_ROTATED_RASTRIGIN) return mul2(z, z);
    const uint64_t C = pk2(12582912.0f, 12582912.0f);
    const uint64_t r = sub2(z, sub2(add2(z, C), C));
    const uint64_t r2 = mul2(r, r);
    uint64_t p = pk2(7.756077498e-02f, 7.756077498e-02f);
    p = fma2(p, r2, pk2(-5.982423425e-01f, -5.982423425e-01f));
    p = fma2(p, r2, pk2(2.550069809e+00f, 2.550069809e+00f));
    p = fma2(p, r2, pk2(-5.167709827e+00f, -5.167709827e+00f));
    p = fma2(p, r2, pk2(3.141592741e+00f, 3.141592741e+00f));
    const uint64_t sn = mul2(r, p);
    return fma2(z, z, mul2(mul2(pk2(20.0f, 20.0f), sn), sn));
}

// The per-coordinate-sum epilogue splits a row's columns between two threads: [0, h) and [h, D)
// with h = D / 2 rounded to a multiple of 16 (at least 16), so both parts hold about half the
// columns (D = 100: 48 and 52); the second part's sum is added to the first's. Every kernel using
// this epilogue splits the same way, so a row's fitness does not depend on the kernel.
__host__ __device__ __forceinline__ int epi_split(int D)
{
    const int h = 16 * ((D + 16) / 32);
    return h < 16 ? 16 : h;
}

// sum_j term(scale * z_j) of one N-column chunk starting at column c (j < D), added to the packed
// pair accumulator two columns per operation, in column order.
template <int N>
__device__ __forceinline__ void row_terms(uint64_t &acc, const uint32_t (&r)[N], int c, int D, int func, uint64_t sc)
{
    using namespace tc;
    if (c + N <= D) {
#pragma unroll
        for (int j = 0; j < N; j += 2)
            acc = add2(acc, obj_term2(func, mul2(pk2(__uint_as_float(r[j]), __uint_as_float(r[j + 1])), sc)));
    } else {
#pragma unroll
        for (int j = 0; j < N; j += 2) {
            if (c + j < D) {
                const float z1 = (c + j + 1 < D) ? __uint_as_float(r[j + 1]) : 0.f;
                acc = add2(acc, obj_term2(func, mul2(pk2(__uint_as_float(r[j]), z1), sc)));
            }
        }
    }
}

__device__ __forceinline__ float pair_sum(uint64_t acc)
{
    float a, b;
    tc::upk2(acc, a, b);
    return a + b;
}

// Warps of one TMEM lane quarter (warp % 4), one lane (= tile row) per thread:
// sum_j term(scale * z_j) over the columns j in [c0, c1), j < D, two columns per packed op, 16
// columns per TMEM load (c0 a multiple of 16), a last chunk of at most 4 columns by a 4-column
// load. `scale` is the row's: the objective's input scale times 2^-(k_row + k_M). (Loads of 8 or
// 32 columns, and loading the next chunk while one is summed, measured slower.)
__device__ __forceinline__ float epilogue_row(uint32_t tmem, int warp, int D, int c0, int c1, int func, float scale)
{
    const uint32_t lane_base = tmem + ((uint32_t)((warp & 3) * 32) << 16);
    const uint64_t sc = tc::pk2(scale, scale);
    uint64_t acc = tc::pk2(0.f, 0.f);
    for (int c = c0; c < c1; c += 16) {
        if (c + 4 >= D) {
            uint32_t r[4];
            tc::tmem_ld4(lane_base + (uint32_t)c, r);
            row_terms<4>(acc, r, c, D, func, sc);
            break;
        }
        uint32_t r[16];
        tc::tmem_ld16(lane_base + (uint32_t)c, r);
        row_terms<16>(acc, r, c, D, func, sc);
    }
    return pair_sum(acc);
}

}  // namespace tcs
}  // namespace speo
