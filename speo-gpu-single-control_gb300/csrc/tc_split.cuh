// tc_split.cuh -- the pieces of the split-BF16 tensor-core rotation that every kernel using it
// shares, so that the same rows give bit-identical fitness whichever kernel evaluates them:
// the three-way BF16 split of M (B operand, shared memory) and of y = x - o (A operand, tensor
// memory): v = v_hi + v_mid + v_lo, each part the BF16 rounding of what the previous parts leave,
// residue ~2^-27 |v|; the six products per 16-wide K step whose size is at least 2^-18 of the
// leading one (y_lo M_hi, y_mid M_mid, y_hi M_lo, y_mid M_hi, y_hi M_mid, y_hi M_hi, smallest
// first; the terms left out are ~2^-27 of it), so the rotation carries the FP32 accumulation's
// rounding like a CUDA-core rotation; and the fused objective epilogue of the per-coordinate sums
// (rotated Rastrigin 9 and sphere 31). Three products of two-way splits of both operands leave
// three 2^-18 terms (measured: fitness up to 1.2e-5 relative from FP64), and five products with a
// two-way split of y one of them (1.1e-5); both are above the 1e-5 bar of FP32 fitness.
//
// Replaces global_ShiftAndRotation + global_f8 (CUDA_EA_library/kernel_CEC2014_CUDA.cu:147-181,
// 557-587).
#pragma once

#include "common.cuh"
#include "tcgen05.cuh"

namespace speo {
namespace tcs {

constexpr int kTileM = 128;   // MMA rows (one TMEM lane per row)
constexpr int kApartMax = 64; // TMEM columns of one A part (K <= 128: 64 BF16 pairs)

__host__ __device__ __forceinline__ int round16(int x) { return (x + 15) & ~15; }

// Builds B = split3(M) for an instance with `nthr` threads (index t): B[n][k] = M[n][k] =
// rot[k*ld_rot + n] (zero past D), and the shift o. The three parts are b_bytes apart.
__device__ __forceinline__ void build_b(const speo_segment &s, int Kp, uint8_t *b_hi, size_t b_bytes, float *so, int t,
                                        int nthr)
{
    const int D = s.dim;
    const int pairs = Kp * (Kp / 8);
    for (int i = t; i < pairs; i += nthr) {
        const int n = i % Kp, kc = i / Kp;
        float v[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) {
            const int k = 8 * kc + e;
            v[e] = (n < D && k < D) ? s.rot[(size_t)k * s.ld_rot + n] : 0.f;
        }
        uint4 h, m, l;
        tc::split8x3(v, h, m, l);
        const uint32_t off = tc::kmajor_offset(n, 8 * kc, Kp);
        *reinterpret_cast<uint4 *>(b_hi + off) = h;
        *reinterpret_cast<uint4 *>(b_hi + b_bytes + off) = m;
        *reinterpret_cast<uint4 *>(b_hi + 2 * b_bytes + off) = l;
    }
    for (int k = t; k < Kp; k += nthr) so[k] = k < D ? s.shift[k] : 0.f;
}

// One row's K step of the A operand: y = x - o over the 16 columns k0 .. k0+15 of a staged row
// (zero past D or for a dead row), split three ways into BF16 hi / mid / lo and packed two per
// 32-bit word (even k in the low half), as tcgen05.mma reads A from tensor memory.
__device__ __forceinline__ void convert16(const float *row, const float *so, int k0, int D, bool live,
                                          uint32_t (&hi)[8], uint32_t (&mid)[8], uint32_t (&lo)[8])
{
    float v[16];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const float4 x = reinterpret_cast<const float4 *>(row + k0)[q];
        const float4 o = reinterpret_cast<const float4 *>(so + k0)[q];
        const int k = k0 + 4 * q;
        if (live && k + 4 <= D) {
            v[4 * q + 0] = __fsub_rn(x.x, o.x); v[4 * q + 1] = __fsub_rn(x.y, o.y);
            v[4 * q + 2] = __fsub_rn(x.z, o.z); v[4 * q + 3] = __fsub_rn(x.w, o.w);
        } else {
            v[4 * q + 0] = (live && k + 0 < D) ? __fsub_rn(x.x, o.x) : 0.f;
            v[4 * q + 1] = (live && k + 1 < D) ? __fsub_rn(x.y, o.y) : 0.f;
            v[4 * q + 2] = (live && k + 2 < D) ? __fsub_rn(x.z, o.z) : 0.f;
            v[4 * q + 3] = (live && k + 3 < D) ? __fsub_rn(x.w, o.w) : 0.f;
        }
    }
#pragma unroll
    for (int p = 0; p < 8; ++p) {
        const __nv_bfloat162 hh = __floats2bfloat162_rn(v[2 * p], v[2 * p + 1]);
        const float2 hf = __bfloat1622float2(hh);
        const float r0 = v[2 * p] - hf.x, r1 = v[2 * p + 1] - hf.y;  // exact
        const __nv_bfloat162 mm = __floats2bfloat162_rn(r0, r1);
        const float2 mf = __bfloat1622float2(mm);
        const __nv_bfloat162 ll = __floats2bfloat162_rn(r0 - mf.x, r1 - mf.y);  // r - mid exact
        hi[p] = *reinterpret_cast<const uint32_t *>(&hh);
        mid[p] = *reinterpret_cast<const uint32_t *>(&mm);
        lo[p] = *reinterpret_cast<const uint32_t *>(&ll);
    }
}

// One thread: the six split products over K steps [s0, s1) into the TMEM accumulator (step 0
// overwrites it), smallest first; A hi / mid / lo in tensor memory at a_hi + {0, 1, 2} apart (8
// columns per step, step s at 8 s), B hi / mid / lo in shared memory b_bytes apart.
__device__ __forceinline__ void issue_split_mma(uint32_t acc, uint32_t a_hi, uint32_t apart, const uint8_t *b_hi,
                                                size_t b_bytes, int Kp, int Np, int s0, int s1)
{
    const uint32_t idesc = tc::idesc_bf16_f32(kTileM, Np);
    const uint32_t sbo = (uint32_t)Kp * 16;  // 8-row groups
    const uint32_t lbo = 128;                // adjacent core matrices along K
    // a K step moves B by two core matrices (256 B: 16 in the descriptor's address field, which
    // holds smem address >> 4 and cannot carry for addresses below 256 KB) and A by 8 columns
    const uint32_t b0 = tc::smem_u32(b_hi) + (uint32_t)s0 * 256u;
    uint64_t dh = tc::smem_desc(b0, lbo, sbo);
    uint64_t dm = tc::smem_desc(b0 + (uint32_t)b_bytes, lbo, sbo);
    uint64_t dl = tc::smem_desc(b0 + 2u * (uint32_t)b_bytes, lbo, sbo);
    uint32_t ah = a_hi + (uint32_t)s0 * 8u, am = ah + apart, al = ah + 2u * apart;
    for (int s = s0; s < s1; ++s) {
        tc::mma_bf16_ta(acc, al, dh, idesc, s > 0);
        tc::mma_bf16_ta(acc, am, dm, idesc, 1);
        tc::mma_bf16_ta(acc, ah, dl, idesc, 1);
        tc::mma_bf16_ta(acc, am, dh, idesc, 1);
        tc::mma_bf16_ta(acc, ah, dm, idesc, 1);
        tc::mma_bf16_ta(acc, ah, dh, idesc, 1);
        dh += 16;
        dm += 16;
        dl += 16;
        ah += 8;
        am += 8;
        al += 8;
    }
}

// Two objective terms at once (f32x2); per element the same operations as obj_term: z - rint(z)
// (rint by adding and subtracting 1.5 * 2^23, exact for |z| < 2^22), the Taylor sine, and
// z*z + (20 s) s.
__device__ __forceinline__ uint64_t obj_term2(int func, uint64_t z)
{
    using namespace tc;
    if (func != SPEO_FUNC_ROTATED_RASTRIGIN) return mul2(z, z);
    const uint64_t C = pk2(12582912.0f, 12582912.0f);
    const uint64_t r = sub2(z, sub2(add2(z, C), C));
    const uint64_t r2 = mul2(r, r);
    uint64_t p = pk2(-7.3704309762e-03f, -7.3704309762e-03f);
    p = fma2(p, r2, pk2(8.2145884633e-02f, 8.2145884633e-02f));
    p = fma2(p, r2, pk2(-5.9926450253e-01f, -5.9926450253e-01f));
    p = fma2(p, r2, pk2(2.5501639843e+00f, 2.5501639843e+00f));
    p = fma2(p, r2, pk2(-5.1677126884e+00f, -5.1677126884e+00f));
    p = fma2(p, r2, pk2(3.1415927410e+00f, 3.1415927410e+00f));
    const uint64_t sn = mul2(r, p);
    return fma2(z, z, mul2(mul2(pk2(20.0f, 20.0f), sn), sn));
}

// The per-coordinate-sum epilogue splits a row's Np accumulator columns between two threads:
// [0, h) and [h, Np) with h = 32 ceil(Np / 64); the second part's sum is added to the first's. Every
// kernel using this epilogue splits the same way, so a row's fitness does not depend on the kernel.
__host__ __device__ __forceinline__ int epi_split(int Np) { return 32 * ((Np + 63) / 64); }

// sum_j term(scale * z_j) of one 32-column chunk starting at column c (j < D), added to the packed
// pair accumulator two columns per operation, in column order.
__device__ __forceinline__ void row_terms32(uint64_t &acc, const uint32_t (&r)[32], int c, int D, int func,
                                            uint64_t sc)
{
    using namespace tc;
    if (c + 32 <= D) {
#pragma unroll
        for (int j = 0; j < 32; j += 2)
            acc = add2(acc, obj_term2(func, mul2(pk2(__uint_as_float(r[j]), __uint_as_float(r[j + 1])), sc)));
    } else {
#pragma unroll
        for (int j = 0; j < 32; j += 2) {
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
// sum_j term(scale * z_j) over the columns j in [c0, c1), j < D, two columns per packed op, 32
// columns per TMEM load (c0 a multiple of 32).
__device__ __forceinline__ float epilogue_row(uint32_t tmem, int warp, int D, int c0, int c1, int func, float scale)
{
    const uint32_t lane_base = tmem + ((uint32_t)((warp & 3) * 32) << 16);
    const uint64_t sc = tc::pk2(scale, scale);
    uint64_t acc = tc::pk2(0.f, 0.f);
    for (int c = c0; c < c1; c += 32) {
        uint32_t r[32];
        tc::tmem_ld32_nowait(lane_base + (uint32_t)c, r);
        tc::tmem_wait_ld();
        row_terms32(acc, r, c, D, func, sc);
    }
    return pair_sum(acc);
}

}  // namespace tcs
}  // namespace speo
