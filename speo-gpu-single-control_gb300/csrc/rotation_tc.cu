// rotation_tc.cu -- exact evaluation with the rotation on the tcgen05 tensor cores.
//
// Replaces global_ShiftAndRotation + global_f8 (CUDA_EA_library/kernel_CEC2014_CUDA.cu:147-181,
// 557-587), an FP64 16x16 shared-memory GEMM that writes the rotated population back to HBM,
// with one pass per 128-row tile:
//   TMA (cp.async.bulk.tensor.2d) brings the FP32 rows into shared memory (two stages, the
//   next tile in flight while this one is processed); the block subtracts o and splits
//   y = y_hi + y_lo into BF16 K-major operands; M (B operand, [N][K] = M[n][k]) is split the
//   same way once per instance; one thread issues, per 16-wide K step, the three products
//   y_hi*M_hi + y_hi*M_lo + y_lo*M_hi into an FP32 accumulator in tensor memory
//   (M = 128 rows, N = D rounded up to 16); the tile is converted and multiplied in two K
//   halves, so that the products of one half run while the other half (or the next tile's first
//   half) is converted; eight warps read the rows back with tcgen05.ld (two per TMEM lane
//   quarter, each half of the columns), apply the scale and the objective term and reduce each
//   row in registers.
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
constexpr int kTmemAlloc = 256;  // two accumulators: MMA of tile i+1 overlaps the epilogue of tile i
constexpr long long kWaitBudget = 2000000000LL;  // ~1 s at 2 GHz: any wait longer is a failure
constexpr int kThreadsTc = 512;   // warps 0-7: epilogue; warps 8-15: conversion (+ TMA / MMA issue)
constexpr int kEpiThreads = 256;
constexpr int kCvtThreads = kThreadsTc - kEpiThreads;

__host__ __device__ __forceinline__ int round16(int x) { return (x + 15) & ~15; }

// Row stride of a staged tile: ld padded so that 8 consecutive rows start in different banks.
__host__ __device__ __forceinline__ int stage_ld(int ld) { return (ld & 7) ? ld : ld + 4; }

struct TcLayout {
    int kmax;         // round16(max D)
    int box_x;        // staged row stride (floats)
    int nstage;       // 1 or 2
    size_t stage_bytes, a_bytes, b_bytes, off_a, off_b, off_o, off_bar, off_psum, total;
};

__host__ __device__ inline TcLayout tc_layout(int dim_hi, int ld, int nstage)
{
    TcLayout L;
    L.kmax = round16(dim_hi);
    L.box_x = stage_ld(ld);
    L.nstage = nstage;
    L.stage_bytes = (size_t)kTileM * L.box_x * 4;
    L.a_bytes = (size_t)kTileM * L.kmax * 2;         // one of hi / lo
    L.b_bytes = (size_t)L.kmax * L.kmax * 2;
    L.off_a = ((L.stage_bytes * nstage) + 1023) & ~(size_t)1023;
    L.off_b = L.off_a + 2 * L.a_bytes;
    L.off_o = L.off_b + 2 * L.b_bytes;
    L.off_bar = (L.off_o + (size_t)L.kmax * 4 + 15) & ~(size_t)15;
    L.off_psum = L.off_bar + 128;                      // [2][kTileM] partial row sums
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

// Staged FP32 rows -> y = x - o -> BF16 hi/lo K-major A operand, K chunks [kc0, kc1) of 8
// columns, `nthr` threads (a multiple of kTileM). Thread t converts row m = t % kTileM, chunks
// kc0 + t / kTileM + j * nthr / kTileM: per chunk it reads 8 consecutive floats of its row with
// two 16-byte loads (the staged row stride keeps 8 consecutive rows on distinct banks) and writes
// one 16-byte chunk of each operand, core matrices 128 B apart along K. Rows >= count and columns
// >= D become zero. The loop is unrolled so that the chunks' load-convert-store chains overlap.
__device__ __forceinline__ void build_a(const float *stage, int box_x, int count, int D, int Kp, const float *so,
                                        uint8_t *a_hi, uint8_t *a_lo, int kc0, int kc1, int t, int nthr)
{
    const int m = t % kTileM, kstep = nthr / kTileM;
    const bool live = m < count;
    const float *row = stage + (size_t)m * box_x;
    const uint32_t base = tc::kmajor_offset(m, 0, Kp);
#pragma unroll 4
    for (int kc = kc0 + t / kTileM; kc < kc1; kc += kstep) {
        const int kb = 8 * kc;
        const float4 *src = reinterpret_cast<const float4 *>(row + kb);
        const float4 *o4 = reinterpret_cast<const float4 *>(so + kb);
        const float4 x0 = src[0], x1 = src[1], s0 = o4[0], s1 = o4[1];
        float v[8];
        if (live && kb + 8 <= D) {
            v[0] = __fsub_rn(x0.x, s0.x); v[1] = __fsub_rn(x0.y, s0.y);
            v[2] = __fsub_rn(x0.z, s0.z); v[3] = __fsub_rn(x0.w, s0.w);
            v[4] = __fsub_rn(x1.x, s1.x); v[5] = __fsub_rn(x1.y, s1.y);
            v[6] = __fsub_rn(x1.z, s1.z); v[7] = __fsub_rn(x1.w, s1.w);
        } else {
            v[0] = (live && kb + 0 < D) ? __fsub_rn(x0.x, s0.x) : 0.f;
            v[1] = (live && kb + 1 < D) ? __fsub_rn(x0.y, s0.y) : 0.f;
            v[2] = (live && kb + 2 < D) ? __fsub_rn(x0.z, s0.z) : 0.f;
            v[3] = (live && kb + 3 < D) ? __fsub_rn(x0.w, s0.w) : 0.f;
            v[4] = (live && kb + 4 < D) ? __fsub_rn(x1.x, s1.x) : 0.f;
            v[5] = (live && kb + 5 < D) ? __fsub_rn(x1.y, s1.y) : 0.f;
            v[6] = (live && kb + 6 < D) ? __fsub_rn(x1.z, s1.z) : 0.f;
            v[7] = (live && kb + 7 < D) ? __fsub_rn(x1.w, s1.w) : 0.f;
        }
        uint4 h, l;
        tc::split8(v, h, l);
        const uint32_t off = base + (uint32_t)kc * 128u;
        *reinterpret_cast<uint4 *>(a_hi + off) = h;
        *reinterpret_cast<uint4 *>(a_lo + off) = l;
    }
}

// One thread: the 3-term split product over K steps [s0, s1) into the TMEM accumulator (step 0
// overwrites it).
__device__ __forceinline__ void issue_split_mma(uint32_t tmem, const uint8_t *a_hi, const uint8_t *a_lo,
                                                const uint8_t *b_hi, const uint8_t *b_lo, int Kp, int Np, int s0,
                                                int s1)
{
    const uint32_t idesc = tc::idesc_bf16_f32(kTileM, Np);
    const uint32_t sbo = (uint32_t)Kp * 16;  // 8-row groups
    const uint32_t lbo = 128;                // adjacent core matrices along K
    const uint32_t ah = tc::smem_u32(a_hi), al = tc::smem_u32(a_lo);
    const uint32_t bh = tc::smem_u32(b_hi), bl = tc::smem_u32(b_lo);
    for (int s = s0; s < s1; ++s) {
        const uint32_t koff = (uint32_t)s * 256;  // two core matrices per K step
        tc::mma_bf16(tmem, tc::smem_desc(al + koff, lbo, sbo), tc::smem_desc(bh + koff, lbo, sbo), idesc, s > 0);
        tc::mma_bf16(tmem, tc::smem_desc(ah + koff, lbo, sbo), tc::smem_desc(bl + koff, lbo, sbo), idesc, 1);
        tc::mma_bf16(tmem, tc::smem_desc(ah + koff, lbo, sbo), tc::smem_desc(bh + koff, lbo, sbo), idesc, 1);
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
    for (int c = c0; c < c1; c += 64) {
        // both 32-column loads in flight before the wait (warp-uniform: c, c1 are)
        uint32_t r[2][32];
        const bool two = c + 32 < c1;
        tmem_ld32_nowait(lane_base + (uint32_t)c, r[0]);
        if (two) tmem_ld32_nowait(lane_base + (uint32_t)(c + 32), r[1]);
        tmem_wait_ld();
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            if (u == 1 && !two) break;
            const int cu = c + 32 * u;
            if (cu + 32 <= D) {
#pragma unroll
                for (int j = 0; j < 32; j += 2)
                    acc = add2(acc, obj_term2(func, mul2(pk2(__uint_as_float(r[u][j]), __uint_as_float(r[u][j + 1])), sc)));
            } else {
#pragma unroll
                for (int j = 0; j < 32; j += 2) {
                    if (cu + j < D) {
                        const float z1 = (cu + j + 1 < D) ? __uint_as_float(r[u][j + 1]) : 0.f;
                        acc = add2(acc, obj_term2(func, mul2(pk2(__uint_as_float(r[u][j]), z1), sc)));
                    }
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

// Warp roles: warps 8..15 convert tile i (thread 256 also issues the TMA loads and the MMAs);
// warps 0..7 run the epilogue of tile i-1 from the other TMEM accumulator meanwhile. The A
// operand is converted and multiplied in two K halves: while the products of one half run, the
// other half is converted.
//   bar_tma[s]  stage s holds the rows of its tile         (TMA transaction bytes)
//   bar_ah[h]   the products of half h of the last tile are done: its A half is free (tcgen05.commit)
//   bar_mma[b]  accumulator b holds a finished product     (tcgen05.commit)
//   bar_epi[b]  the epilogue is done reading accumulator b (256 arrivals)
//   bar_fin     every product this block issued is done    (tcgen05.commit, on abort)
// Everything a role needs about one tile, loaded ahead of use (two-stage register prefetch:
// the work item two tiles ahead, its segment one tile ahead).
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
    float *stage[2] = {reinterpret_cast<float *>(smem), reinterpret_cast<float *>(smem + L.stage_bytes)};
    uint8_t *a_hi = smem + L.off_a, *a_lo = a_hi + L.a_bytes;
    uint8_t *b_hi = smem + L.off_b, *b_lo = b_hi + L.b_bytes;
    float *so = reinterpret_cast<float *>(smem + L.off_o);
    float *psum = reinterpret_cast<float *>(smem + L.off_psum);
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + L.off_bar);
    uint64_t *bar_tma = bars, *bar_mma = bars + 2, *bar_epi = bars + 4, *bar_ah = bars + 8, *bar_fin = bars + 10;
    volatile int *abort_flag = reinterpret_cast<volatile int *>(bars + 6);
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 7);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int ns = a.nstage;

    if (warp == 0) {
        tc::tmem_alloc(tmem_slot, kTmemAlloc);
        tc::tmem_relinquish();
    }
    if (tid == 32) {
        tc::mbar_init(&bar_tma[0], 1);
        tc::mbar_init(&bar_tma[1], 1);
        tc::mbar_init(&bar_mma[0], 1);
        tc::mbar_init(&bar_mma[1], 1);
        tc::mbar_init(&bar_epi[0], kEpiThreads);
        tc::mbar_init(&bar_epi[1], kEpiThreads);
        tc::mbar_init(&bar_ah[0], 1);
        tc::mbar_init(&bar_ah[1], 1);
        tc::mbar_init(bar_fin, 1);
        *abort_flag = 0;
        tc::fence_mbar_init();
        tc::prefetch_tensormap(&xmap);
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tmem_slot;

    const int my_items = a.n_items > (int)blockIdx.x ? (a.n_items - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    auto item_of = [&](int i) { return a.items[blockIdx.x + i * gridDim.x]; };
    int tma_issued = 0;      // issuer bookkeeping (thread kEpiThreads)
    bool mma_any = false;
    // t: the tile's information, loaded a tile ahead (no dependent global load on the issuer's path)
    auto issue_tma = [&](int i, const TileInfo &t) {
        if (i >= my_items) return;
        const int sidx = i % ns;
        tc::mbar_arrive_expect_tx(&bar_tma[sidx], (uint32_t)L.stage_bytes);
        tc::tma_load_2d(stage[sidx], &xmap, 0, t.ok ? (int)t.row : 0, &bar_tma[sidx]);
        tma_issued = i + 1;
    };

    if (warp >= kEpiThreads / 32) {
        // ---- conversion group ---------------------------------------------------------------------
        const int ct = tid - kEpiThreads;
        const bool issuer = ct == 0;
        // three-deep prefetch: tile i's information (cur), tile i+1's (nxt), tile i+2's work item
        TileInfo cur = tile_info(a, item_of(0));
        TileInfo nxt = tile_info(a, item_of(my_items > 1 ? 1 : 0));
        speo_work_item it_nn = item_of(my_items > 2 ? 2 : 0);
        if (issuer) {
            issue_tma(0, cur);
            if (ns > 1) issue_tma(1, nxt);
        }
        const float *c_rot = nullptr, *c_shift = nullptr;
        int c_dim = -1, c_ldrot = -1;
        bool stop = false;
        for (int i = 0; i < my_items && !stop; ++i) {
            const speo_work_item it_n3 = item_of(i + 3 < my_items ? i + 3 : i);
            const TileInfo nn = tile_info(a, it_nn);  // tile i+2
            const int D = cur.D, Kp = round16(D), S = Kp / 16, s_half = (S + 1) / 2;
            bool to = !tc::mbar_wait_sleep(&bar_tma[i % ns], (uint32_t)((i / ns) & 1), kWaitBudget);
            const bool new_b = cur.ok && (cur.rot != c_rot || cur.shift != c_shift || D != c_dim ||
                                          cur.ld_rot != c_ldrot);
            // B and o are read by every product of the previous tile: rebuild them once those are done
            if (new_b && i >= 1)
                to |= !tc::mbar_wait_sleep(&bar_mma[(i - 1) & 1], (uint32_t)(((i - 1) >> 1) & 1), kWaitBudget);
            if (tc::named_bar_or(1, kCvtThreads, to || *abort_flag != 0)) { *abort_flag = 1; break; }
            if (new_b) {
                speo_segment sb;
                sb.dim = D; sb.rot = cur.rot; sb.shift = cur.shift; sb.ld_rot = cur.ld_rot;
                build_b(sb, Kp, b_hi, b_lo, so, ct, kCvtThreads);
                c_rot = cur.rot; c_shift = cur.shift; c_dim = D; c_ldrot = cur.ld_rot;
                tc::named_bar_sync(1, kCvtThreads);
            }
            if (!cur.ok && ct == 0) atomicOr(&s_deverr, SPEO_DEVERR_BAD_SEGMENT);
            for (int h = 0; h < 2; ++h) {
                const int s0 = h == 0 ? 0 : s_half, s1 = h == 0 ? s_half : S;
                // the products of half h of the previous tile must be done before its A half is rewritten
                bool th = i >= 1 && !tc::mbar_wait_sleep(&bar_ah[h], (uint32_t)((i - 1) & 1), kWaitBudget);
                if (cur.ok && !th) build_a(stage[i % ns], L.box_x, cur.count, D, Kp, so, a_hi, a_lo, 2 * s0, 2 * s1, ct,
                                           kCvtThreads);
                tc::fence_proxy_async_smem();
                if (tc::named_bar_or(1, kCvtThreads, th || *abort_flag != 0)) {
                    *abort_flag = 1;
                    stop = true;
                    break;
                }
                if (issuer) {
                    bool free_acc = true;
                    if (h == 0 && i >= 2)
                        free_acc = tc::mbar_wait_sleep(&bar_epi[i & 1], (uint32_t)(((i - 2) >> 1) & 1), kWaitBudget);
                    if (!free_acc) {
                        *abort_flag = 1;
                    } else {
                        tc::fence_after_sync();
                        issue_split_mma(tmem + (uint32_t)((i & 1) * kTmemCols), a_hi, a_lo, b_hi, b_lo, Kp, Kp, s0, s1);
                        mma_any = true;
                        tc::mma_commit(&bar_ah[h]);
                        if (h == 1) {
                            tc::mma_commit(&bar_mma[i & 1]);
                            // every converter has read the stage: it takes tile i + ns
                            issue_tma(i + ns, ns > 1 ? nn : nxt);
                        }
                    }
                }
            }
            cur = nxt;
            nxt = nn;
            it_nn = it_n3;
        }
    } else {
        // ---- epilogue group: one TMEM lane (= tile row) per thread, two warps per lane quarter ------
        const int q = warp & 3, ch = warp >> 2;  // lane quarter, column half
        speo_work_item it_next = item_of(my_items > 1 ? 1 : 0);
        TileInfo cur = tile_info(a, item_of(0));
        for (int i = 0; i < my_items; ++i) {
            // Decisions to stop are reduced over the quarter's two warps (named barrier 2 + q), so
            // that both leave together and neither waits at that barrier for the other; they are
            // then also warp-uniform, as the warp-collective tcgen05.ld below needs.
            if (tc::named_bar_or(2 + q, 64, *abort_flag != 0)) break;
            const speo_work_item it_nn = item_of(i + 2 < my_items ? i + 2 : i);
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
    if (*abort_flag && tid == kEpiThreads) {
        // Let the copies and products this block started finish (bounded) before its shared and
        // tensor memory are released.
        atomicOr(&s_deverr, SPEO_DEVERR_WAIT_TIMEOUT);
        for (int j = (tma_issued > ns ? tma_issued - ns : 0); j < tma_issued; ++j)
            tc::mbar_wait_sleep(&bar_tma[j % ns], (uint32_t)((j / ns) & 1), kWaitBudget);
        if (mma_any) {
            tc::mma_commit(bar_fin);
            tc::mbar_wait_sleep(bar_fin, 0, kWaitBudget);
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
    int nstage = 2;
    if ((int)tc_layout(dim_hi, ld, 2).total > limit) nstage = 1;
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
