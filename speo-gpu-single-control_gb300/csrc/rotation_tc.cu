// rotation_tc.cu -- exact evaluation with the rotation on the tcgen05 tensor cores.
//
// Replaces global_ShiftAndRotation + global_f8 (CUDA_EA_library/kernel_CEC2014_CUDA.cu:147-181,
// 557-587), an FP64 16x16 shared-memory GEMM that writes the rotated population back to HBM,
// with one pass per 128-row tile:
//   TMA (cp.async.bulk.tensor.2d) brings the FP32 rows into shared memory (a ring of up to three
//   stages); converter warps subtract o and split y = y_hi + y_lo into BF16, each thread one row,
//   and store the A operand straight into tensor memory (tcgen05.st, double-buffered by tile);
//   M (B operand, [N][K] = M[n][k]) is split the same way once per instance into shared memory;
//   one thread issues, per 16-wide K step, the three products y_hi*M_hi + y_hi*M_lo + y_lo*M_hi
//   (A from tensor memory) into an FP32 accumulator in tensor memory (M = 128 rows, N = D rounded
//   up to 16). The tile is converted and multiplied in two K halves (one converter warp per lane
//   quarter and half); eight warps read the rows back with tcgen05.ld (two per lane quarter, each
//   half of the columns), apply the scale and the objective term and reduce each row in registers.
// Nothing but the fitness is written. D <= 128.
#include <cuda.h>

#include <cmath>

#include "common.cuh"
#include "host.h"
#include "tcgen05.cuh"

SPEO_DEFINE_DEVERR(speo_deverr_tc)

namespace speo {
namespace {

constexpr int kTileM = 128;
constexpr int kTmemCols = 128;   // one accumulator (N <= 128)
// Tensor memory: accumulators b = 0, 1 at columns 128 b (MMA of tile i+1 overlaps the epilogue of
// tile i); A operand of buffer b at 256 + 128 b (hi, <= 64 columns) and 320 + 128 b (lo).
constexpr int kTmemAlloc = 512;
constexpr int kAcolBase = 256;
constexpr long long kWaitBudget = 2000000000LL;  // ~1 s at 2 GHz: any wait longer is a failure
constexpr int kEpiThreads = 256;                 // warps 0-7: epilogue
constexpr int kCvtThreads = 256;                 // warps 8-15: conversion
constexpr int kThreadsTc = kEpiThreads + kCvtThreads + 32;  // warp 16: TMA and MMA issue
constexpr int kIssuerWarp = (kEpiThreads + kCvtThreads) / 32;
constexpr int kMaxStages = 3;

__host__ __device__ __forceinline__ int round16(int x) { return (x + 15) & ~15; }

// Row stride of a staged tile: ld padded so that 8 consecutive rows start in different banks.
__host__ __device__ __forceinline__ int stage_ld(int ld) { return (ld & 7) ? ld : ld + 4; }

struct TcLayout {
    int kmax;         // round16(max D)
    int box_x;        // staged row stride (floats)
    int nstage;       // 1 to kMaxStages
    size_t stage_bytes, b_bytes, off_b, off_o, off_bar, off_psum, total;
};

//   stage[nstage] | B hi, lo | o | barriers | psum[2][kTileM]
__host__ __device__ inline TcLayout tc_layout(int dim_hi, int ld, int nstage)
{
    TcLayout L;
    L.kmax = round16(dim_hi);
    L.box_x = stage_ld(ld);
    L.nstage = nstage;
    L.stage_bytes = (size_t)kTileM * L.box_x * 4;
    L.b_bytes = (size_t)L.kmax * L.kmax * 2;
    L.off_b = ((L.stage_bytes * nstage) + 1023) & ~(size_t)1023;
    L.off_o = L.off_b + 2 * L.b_bytes;
    L.off_bar = (L.off_o + (size_t)L.kmax * 4 + 15) & ~(size_t)15;
    L.off_psum = L.off_bar + 256;
    L.total = L.off_psum + 2 * kTileM * 4;
    return L;
}

struct EvalTcArgs {
    const speo_segment *segs;
    const speo_work_item *items;
    int n_items;
    long long n_rows;
    int ld;
    int dim_hi;
    int nstage;
    float *fit;
};

// Builds B = split(M) for an instance with `nthr` threads (index t): B[n][k] = M[n][k] =
// rot[k*ld_rot + n] (zero past D), and the shift o.
__device__ __forceinline__ void build_b(const speo_segment &s, int Kp, uint8_t *b_hi, uint8_t *b_lo, float *so, int t,
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
        uint4 h, l;
        tc::split8(v, h, l);
        const uint32_t off = tc::kmajor_offset(n, 8 * kc, Kp);
        *reinterpret_cast<uint4 *>(b_hi + off) = h;
        *reinterpret_cast<uint4 *>(b_lo + off) = l;
    }
    for (int k = t; k < Kp; k += nthr) so[k] = k < D ? s.shift[k] : 0.f;
}

// One row's K step of the A operand: y = x - o over the 16 columns k0 .. k0+15 of a staged row
// (zero past D or for a dead row), split into BF16 hi / lo and packed two per 32-bit word (even
// k in the low half), as tcgen05.mma reads A from tensor memory.
__device__ __forceinline__ void convert16(const float *row, const float *so, int k0, int D, bool live,
                                          uint32_t (&hi)[8], uint32_t (&lo)[8])
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
        const __nv_bfloat162 ll = __floats2bfloat162_rn(v[2 * p] - hf.x, v[2 * p + 1] - hf.y);
        hi[p] = *reinterpret_cast<const uint32_t *>(&hh);
        lo[p] = *reinterpret_cast<const uint32_t *>(&ll);
    }
}

// One thread: the 3-term split product over K steps [s0, s1) into the TMEM accumulator (step 0
// overwrites it); A hi / lo in tensor memory at a_hi / a_lo (8 columns per step), B in shared
// memory.
__device__ __forceinline__ void issue_split_mma(uint32_t acc, uint32_t a_hi, uint32_t a_lo, const uint8_t *b_hi,
                                                const uint8_t *b_lo, int Kp, int Np, int s0, int s1)
{
    const uint32_t idesc = tc::idesc_bf16_f32(kTileM, Np);
    const uint32_t sbo = (uint32_t)Kp * 16;  // 8-row groups
    const uint32_t lbo = 128;                // adjacent core matrices along K
    // a K step moves B by two core matrices (256 B: 16 in the descriptor's address field, which
    // holds smem address >> 4 and cannot carry for addresses below 256 KB) and A by 8 columns
    uint64_t dh = tc::smem_desc(tc::smem_u32(b_hi) + (uint32_t)s0 * 256u, lbo, sbo);
    uint64_t dl = tc::smem_desc(tc::smem_u32(b_lo) + (uint32_t)s0 * 256u, lbo, sbo);
    uint32_t ah = a_hi + (uint32_t)s0 * 8u, al = a_lo + (uint32_t)s0 * 8u;
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

// Warps of one TMEM lane quarter (warp % 4), one lane (= tile row) per thread:
// sum_j term(scale * z_j) over the columns j in [c0, c1), j < D, two columns per packed op, 32
// columns per TMEM load (c0 a multiple of 32).
__device__ __forceinline__ float epilogue_row(uint32_t tmem, int warp, int D, int c0, int c1, int func, float scale)
{
    using namespace tc;
    const uint32_t lane_base = tmem + ((uint32_t)((warp & 3) * 32) << 16);
    const uint64_t sc = pk2(scale, scale);
    uint64_t acc = pk2(0.f, 0.f);
    for (int c = c0; c < c1; c += 32) {
        uint32_t r[32];
        tmem_ld32_nowait(lane_base + (uint32_t)c, r);
        tmem_wait_ld();
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
    float a, b;
    upk2(acc, a, b);
    return a + b;
}

// The other rotated CEC2014 bodies (1-7, 11-16), one TMEM lane (= tile row) per thread: the row
// accumulator of the CUDA-core paths (row_push / row_finish) over the row's columns in order, each
// column pushed once its successor is known and the last one with column 0. The function id is a
// template parameter, so each instance carries one body.
template <int FID>
__device__ __noinline__ float epi_generic(uint32_t lane_base, int D, int Np, float scale)
{
    using namespace tc;
    const float fs = func_fixed_shift<float>(FID);
    RowAcc<float> acc;
    float z0 = 0.f, prev = 0.f;
    for (int c = 0; c < Np; c += 32) {
        uint32_t r[32];
        tmem_ld32_nowait(lane_base + (uint32_t)c, r);
        tmem_wait_ld();
#pragma unroll
        for (int j = 0; j < 32; ++j) {
            const int e = c + j;
            if (e < D) {
                const float z = __uint_as_float(r[j]) * scale + fs;
                if (e == 0) z0 = z;
                else row_push(acc, FID, e - 1, prev, z, D);
                prev = z;
            }
        }
    }
    row_push(acc, FID, D - 1, prev, z0, D);
    return row_finish(acc, FID, D);
}

__device__ __forceinline__ float epilogue_row_generic(uint32_t tmem, int warp, int D, int Np, int func, float scale)
{
    const uint32_t lb = tmem + ((uint32_t)((warp & 3) * 32) << 16);
    switch (func) {
    case 1: return epi_generic<1>(lb, D, Np, scale);
    case 2: return epi_generic<2>(lb, D, Np, scale);
    case 3: return epi_generic<3>(lb, D, Np, scale);
    case 4: return epi_generic<4>(lb, D, Np, scale);
    case 5: return epi_generic<5>(lb, D, Np, scale);
    case 6: return epi_generic<6>(lb, D, Np, scale);
    case 7: return epi_generic<7>(lb, D, Np, scale);
    case 11: return epi_generic<11>(lb, D, Np, scale);
    case 12: return epi_generic<12>(lb, D, Np, scale);
    case 13: return epi_generic<13>(lb, D, Np, scale);
    case 14: return epi_generic<14>(lb, D, Np, scale);
    case 15: return epi_generic<15>(lb, D, Np, scale);
    default: return epi_generic<16>(lb, D, Np, scale);
    }
}

__device__ __forceinline__ bool tc_tile_ok(const speo_work_item &it, const speo_segment &s, const EvalTcArgs &a)
{
    // the rotated single-matrix ids (CEC2014 1-7, 9, 11-16 and 31); 8 and 10 do not rotate and
    // 17-30 have several matrices
    return func_supported(s.func_id) && func_rotated(s.func_id) && it.count >= 1 &&
           it.count <= kTileM && s.dim >= 1 && s.dim <= a.dim_hi && s.dim <= kTmemCols &&
           s.ld == a.ld && it.first >= 0 && it.first + it.count <= s.pop_size && s.row0 >= 0 &&
           s.row0 + it.first + it.count <= a.n_rows;
}

// Warp roles: warps 8..15 convert tile i into the A buffer i % 2 in tensor memory (warp 8 + q + 4h:
// lane quarter q, K half h); warp 16 issues the TMA loads and (one thread) the MMAs of each half
// as soon as it is converted; warps 0..7 run the epilogue of tile i-1 from the other accumulator.
//   bar_tma[s]      stage s holds the rows of its tile                 (TMA transaction bytes)
//   bar_afull[b][h] half h of A buffer b is converted (and its stage rows read) (128 arrivals)
//   bar_afree[b]    the products reading A buffer b are done          (tcgen05.commit)
//   bar_mma[b]      accumulator b holds a finished product            (tcgen05.commit)
//   bar_epi[b]      the epilogue is done reading accumulator b        (256 arrivals)
//   bar_fin         every product this block issued is done           (tcgen05.commit, on abort)
// Everything a role needs about one tile is loaded ahead of use (register prefetch of the work
// items and segments of the next tiles).
struct TileInfo {
    int ok, count, D, func, ld_rot;
    long long row;
    const float *rot, *shift;
};

__device__ __forceinline__ TileInfo tile_info(const EvalTcArgs &a, const speo_work_item &it)
{
    const speo_segment &s = a.segs[it.segment];
    TileInfo t;
    t.ok = tc_tile_ok(it, s, a);
    t.count = it.count;
    t.D = t.ok ? s.dim : 16;
    t.func = s.func_id;
    t.ld_rot = s.ld_rot;
    t.row = s.row0 + it.first;
    t.rot = s.rot;
    t.shift = s.shift;
    return t;
}

__global__ void __launch_bounds__(kThreadsTc, 1) k_evaluate_tc(const __grid_constant__ CUtensorMap xmap, EvalTcArgs a)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    const TcLayout L = tc_layout(a.dim_hi, a.ld, a.nstage);
    const int ns = a.nstage;
    float *stage[kMaxStages];
#pragma unroll
    for (int k = 0; k < kMaxStages; ++k) stage[k] = reinterpret_cast<float *>(smem + (size_t)k * L.stage_bytes);
    uint8_t *b_hi = smem + L.off_b, *b_lo = b_hi + L.b_bytes;
    float *so = reinterpret_cast<float *>(smem + L.off_o);
    float *psum = reinterpret_cast<float *>(smem + L.off_psum);
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + L.off_bar);
    uint64_t *bar_tma = bars, *bar_mma = bars + 3, *bar_epi = bars + 5, *bar_afull = bars + 7, *bar_afree = bars + 11,
             *bar_fin = bars + 13;
    volatile int *abort_flag = reinterpret_cast<volatile int *>(bars + 14);
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 15);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    if (warp == 0) {
        tc::tmem_alloc(tmem_slot, kTmemAlloc);
        tc::tmem_relinquish();
    }
    if (tid == 32) {
        for (int k = 0; k < kMaxStages; ++k) tc::mbar_init(&bar_tma[k], 1);
        for (int b = 0; b < 2; ++b) {
            tc::mbar_init(&bar_mma[b], 1);
            tc::mbar_init(&bar_epi[b], kEpiThreads);
            tc::mbar_init(&bar_afull[2 * b], 128);
            tc::mbar_init(&bar_afull[2 * b + 1], 128);
            tc::mbar_init(&bar_afree[b], 1);
        }
        tc::mbar_init(bar_fin, 1);
        *abort_flag = 0;
        tc::fence_mbar_init();
        tc::prefetch_tensormap(&xmap);
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tmem_slot;
    auto a_hi_col = [&](int b) { return tmem + (uint32_t)(kAcolBase + 128 * b); };
    auto a_lo_col = [&](int b) { return tmem + (uint32_t)(kAcolBase + 128 * b + 64); };

    const int my_items = a.n_items > (int)blockIdx.x ? (a.n_items - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    auto item_of = [&](int i) { return a.items[blockIdx.x + (i < my_items ? i : my_items - 1) * gridDim.x]; };
    int tma_issued = 0;      // issuer bookkeeping (warp kIssuerWarp, lane 0)
    bool mma_any = false;

    if (warp == kIssuerWarp) {
        // ---- TMA and MMA issue: the whole warp runs the loop, lane 0 issues ----------------------
        const bool leader = lane == 0;
        auto issue_tma = [&](int i, const TileInfo &t) {
            if (i >= my_items) return;
            if (leader) {
                const int sidx = i % ns;
                tc::mbar_arrive_expect_tx(&bar_tma[sidx], (uint32_t)L.stage_bytes);
                tc::tma_load_2d(stage[sidx], &xmap, 0, t.ok ? (int)t.row : 0, &bar_tma[sidx]);
            }
            tma_issued = i + 1;
        };
        for (int j = 0; j < ns; ++j) issue_tma(j, tile_info(a, item_of(j)));
        TileInfo cur = tile_info(a, item_of(0)), nxt = tile_info(a, item_of(1));
        speo_work_item it_n2 = item_of(2);
        TileInfo tq = tile_info(a, item_of(ns));        // the tile whose TMA follows tile 0
        speo_work_item it_q = item_of(ns + 1);
        for (int i = 0; i < my_items; ++i) {
            // work items a tile ahead of their segments: no dependent load waits in this iteration
            const TileInfo n2 = tile_info(a, it_n2);
            const speo_work_item it_n3 = item_of(i + 3);
            const TileInfo tq_next = tile_info(a, it_q);
            const speo_work_item it_q_next = item_of(i + ns + 2);
            const int b = i & 1, Kp = round16(cur.D), S = Kp / 16, s_half = (S + 1) / 2;
            bool ok = tc::mbar_wait_sleep(&bar_afull[2 * b], (uint32_t)((i >> 1) & 1), kWaitBudget);
            if (i >= 2) ok = ok && tc::mbar_wait_sleep(&bar_epi[b], (uint32_t)(((i - 2) >> 1) & 1), kWaitBudget);
            if (!__all_sync(0xffffffffu, ok && *abort_flag == 0)) { *abort_flag = 1; break; }
            tc::fence_after_sync();
            const uint32_t acc = tmem + (uint32_t)(b * kTmemCols);
            if (leader) {
                issue_split_mma(acc, a_hi_col(b), a_lo_col(b), b_hi, b_lo, Kp, Kp, 0, s_half);
                mma_any = true;
            }
            ok = tc::mbar_wait_sleep(&bar_afull[2 * b + 1], (uint32_t)((i >> 1) & 1), kWaitBudget);
            if (!__all_sync(0xffffffffu, ok && *abort_flag == 0)) { *abort_flag = 1; break; }
            tc::fence_after_sync();
            if (leader) {
                issue_split_mma(acc, a_hi_col(b), a_lo_col(b), b_hi, b_lo, Kp, Kp, s_half, S);
                tc::mma_commit(&bar_mma[b]);
                tc::mma_commit(&bar_afree[b]);
            }
            // both halves' converters have read stage i % ns: it takes tile i + ns
            issue_tma(i + ns, tq);
            __syncwarp();
            cur = nxt;
            nxt = n2;
            it_n2 = it_n3;
            tq = tq_next;
            it_q = it_q_next;
        }
    } else if (warp >= kEpiThreads / 32) {
        // ---- conversion: thread = row 32 q + lane, K half ch -------------------------------------
        const int ct = tid - kEpiThreads, q = warp & 3, ch = (warp - kEpiThreads / 32) >> 2;
        const int m = q * 32 + lane;
        const uint32_t lane_off = (uint32_t)(q * 32) << 16;
        TileInfo cur = tile_info(a, item_of(0));
        TileInfo nxt = tile_info(a, item_of(1));
        speo_work_item it_nn = item_of(2);
        const float *c_rot = nullptr, *c_shift = nullptr;
        int c_dim = -1, c_ldrot = -1;
        for (int i = 0; i < my_items; ++i) {
            const speo_work_item it_n3 = item_of(i + 3);
            const TileInfo nn = tile_info(a, it_nn);
            const int sidx = i % ns, b = i & 1;
            const int D = cur.D, Kp = round16(D), S = Kp / 16, s_half = (S + 1) / 2;
            bool to = !tc::mbar_wait_sleep(&bar_tma[sidx], (uint32_t)((i / ns) & 1), kWaitBudget);
            const bool new_b = cur.ok && (cur.rot != c_rot || cur.shift != c_shift || D != c_dim ||
                                          cur.ld_rot != c_ldrot);
            // B and o are read by every product of the previous tile: rebuild them once those are done
            if (new_b && i >= 1)
                to |= !tc::mbar_wait_sleep(&bar_mma[(i - 1) & 1], (uint32_t)(((i - 1) >> 1) & 1), kWaitBudget);
            // the group's decision to stop is reduced over all converters, so that none waits at
            // named barrier 1 for one that left
            if (tc::named_bar_or(1, kCvtThreads, to || *abort_flag != 0)) { *abort_flag = 1; break; }
            if (new_b) {
                speo_segment sb;
                sb.dim = D; sb.rot = cur.rot; sb.shift = cur.shift; sb.ld_rot = cur.ld_rot;
                build_b(sb, Kp, b_hi, b_lo, so, ct, kCvtThreads);
                c_rot = cur.rot; c_shift = cur.shift; c_dim = D; c_ldrot = cur.ld_rot;
                tc::fence_proxy_async_smem();
                tc::named_bar_sync(1, kCvtThreads);
            }
            if (!cur.ok && ct == 0) atomicOr(&s_deverr, SPEO_DEVERR_BAD_SEGMENT);
            // A buffer b was last read by the products of tile i - 2
            bool ok = i < 2 || tc::mbar_wait_sleep(&bar_afree[b], (uint32_t)(((i - 2) >> 1) & 1), kWaitBudget);
            if (__all_sync(0xffffffffu, ok)) {
                const int s0 = ch == 0 ? 0 : s_half, s1 = ch == 0 ? s_half : S;
                const float *row = stage[sidx] + (size_t)m * L.box_x;
                const bool live = cur.ok && m < cur.count;
                for (int st = s0; st < s1; ++st) {
                    uint32_t hi[8], lo[8];
                    convert16(row, so, 16 * st, D, live, hi, lo);
                    tc::tmem_st32x8(a_hi_col(b) + lane_off + (uint32_t)(8 * st), hi);
                    tc::tmem_st32x8(a_lo_col(b) + lane_off + (uint32_t)(8 * st), lo);
                }
                tc::tmem_wait_st();
                tc::fence_before_sync();
                tc::mbar_arrive(&bar_afull[2 * b + ch]);
            } else {
                *abort_flag = 1;  // the next tile's barrier stops the group
            }
            cur = nxt;
            nxt = nn;
            it_nn = it_n3;
        }
    } else {
        // ---- epilogue group: one TMEM lane (= tile row) per thread, two warps per lane quarter ------
        const int q = warp & 3, ch = warp >> 2;  // lane quarter, column half
        speo_work_item it_next = item_of(1);
        TileInfo cur = tile_info(a, item_of(0));
        for (int i = 0; i < my_items; ++i) {
            // Decisions to stop are reduced over the quarter's two warps (named barrier 2 + q), so
            // that both leave together and neither waits at that barrier for the other; they are
            // then also warp-uniform, as the warp-collective tcgen05.ld below needs.
            if (tc::named_bar_or(2 + q, 64, *abort_flag != 0)) break;
            const speo_work_item it_nn = item_of(i + 2);
            const TileInfo nxt = tile_info(a, it_next);
            const bool got = tc::mbar_wait_sleep(&bar_mma[i & 1], (uint32_t)((i >> 1) & 1), kWaitBudget);
            if (tc::named_bar_or(2 + q, 64, !got)) { *abort_flag = 1; break; }
            tc::fence_after_sync();
            const uint32_t acc_t = tmem + (uint32_t)((i & 1) * kTmemCols);
            const int Np = round16(cur.D), m = q * 32 + lane;
            float f = 0.f;
            bool writer = ch == 0;
            if (func_sum_form(cur.func)) {
                // columns [0, 64) on the first warp of the quarter, [64, Np) on the second; the
                // second warp's partial sums meet the first's through psum[i % 2]
                const int c0 = ch * 64, c1 = ch == 0 ? (Np < 64 ? Np : 64) : Np;
                f = c0 < c1 ? epilogue_row(acc_t, warp, cur.D, c0, c1, cur.func, func_scale(cur.func)) : 0.f;
                float *ps = psum + (i & 1) * kTileM;
                if (ch == 1) ps[m] = f;
                tc::named_bar_sync(2 + q, 64);
                if (ch == 0) f += ps[m];
            } else if (ch == 0) {
                f = epilogue_row_generic(acc_t, warp, cur.D, Np, cur.func, func_scale(cur.func));
            }
            if (writer && cur.ok && m < cur.count) a.fit[cur.row + m] = f;
            tc::fence_before_sync();
            tc::mbar_arrive(&bar_epi[i & 1]);
            cur = nxt;
            it_next = it_nn;
        }
    }
    __syncthreads();
    if (*abort_flag && warp == kIssuerWarp && lane == 0) {
        // Let the copies and products this block started finish (bounded) before its shared and
        // tensor memory are released.
        atomicOr(&s_deverr, SPEO_DEVERR_WAIT_TIMEOUT);
        for (int j = (tma_issued > ns ? tma_issued - ns : 0); j < tma_issued; ++j)
            tc::mbar_wait(&bar_tma[j % ns], (uint32_t)((j / ns) & 1), kWaitBudget);
        if (mma_any) {
            tc::mma_commit(bar_fin);
            tc::mbar_wait(bar_fin, 0, kWaitBudget);
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (warp == 0) tc::tmem_dealloc(tmem, kTmemAlloc);
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no libcuda link).
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn()
{
    static EncodeTiledFn fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    }
    return fn;
}

int max_optin_smem()
{
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    return v;
}

}  // namespace
}  // namespace speo

using namespace speo;

extern "C" int speo_evaluate_tc(const speo_segment *segs, const speo_work_item *items, int n_items, int dim_lo,
                                int dim_hi, const float *pop, int64_t n_rows, int ld, float *fit, void *stream)
{
    if (!segs || !items || !pop || !fit || n_items < 1 || n_rows < 1)
        return fail(SPEO_ERR_INVALID_ARG, "speo_evaluate_tc: bad arguments");
    if (dim_lo < 1 || dim_hi > kTmemCols || dim_lo > dim_hi)
        return fail(SPEO_ERR_UNSUPPORTED, "speo_evaluate_tc: D in [%d, %d]; the tensor-core path takes D <= %d",
                    dim_lo, dim_hi, kTmemCols);
    if (ld < dim_hi || (ld & 3) || stage_ld(ld) > 256 || ((uintptr_t)pop & 15))
        return fail(SPEO_ERR_INVALID_ARG, "speo_evaluate_tc: ld %d / alignment", ld);
    EncodeTiledFn enc = encode_fn();
    if (!enc) return fail(SPEO_ERR_CUDA, "speo_evaluate_tc: cuTensorMapEncodeTiled unavailable");
    CUtensorMap map;
    const cuuint64_t dims[2] = {(cuuint64_t)ld, (cuuint64_t)n_rows};
    const cuuint64_t strides[1] = {(cuuint64_t)ld * sizeof(float)};
    const cuuint32_t box[2] = {(cuuint32_t)stage_ld(ld), (cuuint32_t)kTileM};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult r = enc(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float *>(pop), dims, strides, box, estr,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(SPEO_ERR_CUDA, "speo_evaluate_tc: cuTensorMapEncodeTiled failed (%d)", (int)r);
    const int limit = max_optin_smem();
    int nstage = kMaxStages;
    while (nstage > 1 && (int)tc_layout(dim_hi, ld, nstage).total > limit) --nstage;
    const TcLayout Lay = tc_layout(dim_hi, ld, nstage);
    if ((int)Lay.total > limit) return fail(SPEO_ERR_UNSUPPORTED, "speo_evaluate_tc: needs %zu B of shared memory", Lay.total);
    // At least half of the SM's shared memory per block: one block (one TMEM allocation) per SM.
    const size_t smem = Lay.total > (size_t)limit / 2 + 1024 ? Lay.total : (size_t)limit / 2 + 1024;
    cudaError_t e = cudaFuncSetAttribute(k_evaluate_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return check_cuda(e, "cudaFuncSetAttribute(k_evaluate_tc)");
    EvalTcArgs a{segs, items, n_items, (long long)n_rows, ld, dim_hi, nstage, fit};
    const int grid = n_items < sm_count() ? n_items : sm_count();
    k_evaluate_tc<<<grid, kThreadsTc, smem, static_cast<cudaStream_t>(stream)>>>(map, a);
    return check_launch("k_evaluate_tc");
}

__global__ void k_advance_gen_tc(uint32_t *gen) { gen[0] += 1u; }

extern "C" int speo_generation_tc(const speo_segment *segs, const speo_work_item *items, int n_items, int dim_lo,
                                  int dim_hi, const float *pop_in, const float *fit_in, float *pop_out,
                                  float *fit_out, int64_t n_rows, int ld, uint32_t *d_gen, float *trial,
                                  float *trial_fit, void *stream)
{
    if (!segs || !items || !pop_in || !fit_in || !pop_out || !fit_out || !d_gen || !trial || !trial_fit ||
        n_items < 1 || n_rows < 1)
        return fail(SPEO_ERR_INVALID_ARG, "speo_generation_tc: bad arguments");
    if (pop_in == pop_out || fit_in == fit_out || trial == pop_in || trial == pop_out)
        return fail(SPEO_ERR_INVALID_ARG, "speo_generation_tc: input, output and trial buffers must differ");
    if (int e = speo_make_trials(segs, items, n_items, dim_hi, 1, pop_in, fit_in, trial, d_gen, stream)) return e;
    if (int e = speo_evaluate_tc(segs, items, n_items, dim_lo, dim_hi, trial, n_rows, ld, trial_fit, stream))
        return e;
    if (int e = speo_select_rows(pop_in, fit_in, trial, trial_fit, pop_out, fit_out, n_rows, ld, stream)) return e;
    k_advance_gen_tc<<<1, 1, 0, static_cast<cudaStream_t>(stream)>>>(d_gen);
    return check_launch("k_advance_gen_tc");
}
