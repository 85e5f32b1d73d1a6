// rotation_tc.cu -- exact evaluation with the rotation on the tcgen05 tensor cores.
//
// Replaces global_ShiftAndRotation + global_f8 (CUDA_EA_library/kernel_CEC2014_CUDA.cu:147-181,
// 557-587), an FP64 16x16 shared-memory GEMM that writes the rotated population back to HBM,
// with one pass per 128-row tile:
//   TMA (cp.async.bulk.tensor.2d) brings the FP32 rows into shared memory (a ring of up to three
//   stages); two groups of four converter warps take alternate tiles, a thread per row: it
//   subtracts o, finds the row's largest |y|, scales y = x - o by the row's power of two and splits
//   it two ways into FP16 (tc_split.cuh), and stores the A operand straight into tensor memory
//   (tcgen05.st, a ring of K-half slots); M (B operand, [N][K] = M[n][k]) is scaled and split the
//   same way once per instance into shared memory; one thread issues, per 16-wide K step, the three
//   products of tc_split.cuh (A from tensor memory) into an FP32 accumulator in tensor memory
//   (M = 128 rows, N = D rounded up to 16, three accumulators): the fitness is as exact as the
//   CUDA-core FP32 rotation's. Each K half is handed to the products as soon as it is converted;
//   eight warps read the rows back with tcgen05.ld (two per lane quarter, each half of the
//   columns), apply the row's scale and the objective term and reduce each row in registers.
// Nothing but the fitness is written. D <= 128.
#include <cuda.h>

#include <cmath>

#include "common.cuh"
#include "host.h"
#include "tc_split.cuh"
#include "tcgen05.cuh"

SPEO_DEFINE_DEVERR(speo_deverr_tc)

namespace speo {
namespace {

using tcs::kTileM;
using tcs::round16;
using tcs::build_b;
using tcs::issue_split_mma;
using tcs::epilogue_row;
constexpr int kTmemCols = 128;   // widest accumulator (N <= 128)
// Tensor memory (kmax = round16(largest D) columns per accumulator): accumulators b = 0, 1, 2 at
// columns kmax b (tile i uses accumulator i % 3: the products of tiles i + 1 and i + 2 run while
// the epilogue of tile i reads its accumulator); then two A slots of kSlotCols columns from
// 3 kmax, one per K half: a slot holds the hi and lo parts of one K half (<= 4 steps: 32 columns
// each) kApart = 32 columns apart, and K half h of tile i is converted once the products of K
// half h of tile i - 1 have read the slot.
constexpr int kTmemAlloc = 512;
constexpr int kApart = 32;
constexpr int kSlotCols = tcs::kParts * kApart;
constexpr int kAcc = 3;
constexpr int kSlots = 2;
// The ring of four row-scale buffers (rmul, bar_rs) relies on this layout: the converters of tile
// i + 4 pass their first slot wait only after the products of tile i + 3, which start after the
// epilogue of tile i.
static_assert(kAcc * kTmemCols + kSlots * kSlotCols <= kTmemAlloc, "three accumulators and two A slots");
constexpr long long kWaitBudget = 2000000000LL;  // ~1 s at 2 GHz: any wait longer is a failure
constexpr int kEpiThreads = 256;                 // warps 0-7: epilogue
constexpr int kCvtThreads = 256;                 // warps 8-15: conversion
constexpr int kThreadsTc = kEpiThreads + kCvtThreads + 64;  // warp 16: MMA issue, warp 17: TMA issue
constexpr int kIssuerWarp = (kEpiThreads + kCvtThreads) / 32;
constexpr int kTmaWarp = kIssuerWarp + 1;
constexpr int kMaxStages = 3;

// Row stride of a staged tile: ld padded so that 8 consecutive rows start in different banks.
__host__ __device__ __forceinline__ int stage_ld(int ld) { return (ld & 7) ? ld : ld + 4; }

struct TcLayout {
    int kmax;         // round16(max D)
    int box_x;        // staged row stride (floats)
    int nstage;       // 1 to kMaxStages
    size_t stage_bytes, b_bytes, off_b, off_o, off_bar, off_psum, off_rmul, total;
};

//   stage[nstage] | B hi, lo | o[2][kmax] (each converter group's copy) | barriers | psum[2][kTileM] |
//   rmul[4][kTileM]
// rmul[i % 4][m]: the objective's scale times 2^-(k_row + k_M) of row m in tile i (written by the
// converters, read by the epilogue).
__host__ __device__ inline TcLayout tc_layout(int dim_hi, int ld, int nstage)
{
    TcLayout L;
    L.kmax = round16(dim_hi);
    L.box_x = stage_ld(ld);
    L.nstage = nstage;
    L.stage_bytes = (size_t)kTileM * L.box_x * 4;
    L.b_bytes = (size_t)L.kmax * L.kmax * 2;
    L.off_b = ((L.stage_bytes * nstage) + 1023) & ~(size_t)1023;
    L.off_o = L.off_b + tcs::kParts * L.b_bytes;
    L.off_bar = (L.off_o + 2 * (size_t)L.kmax * 4 + 15) & ~(size_t)15;
    L.off_psum = L.off_bar + 256;
    L.off_rmul = L.off_psum + 2 * kTileM * 4;
    L.total = L.off_rmul + 4 * kTileM * 4;
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
        tmem_ld32(lane_base + (uint32_t)c, r);
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

// Warp roles: warps 8..11 convert the even tiles and warps 12..15 the odd ones into the A slots in
// tensor memory (warp 8 + q + 4g: lane quarter q, group g; each group with its own copy of o and
// named barrier 1 or 6); warp 16 (one thread) issues the MMAs of each half as soon as it is
// converted and the accumulator is free; warp 17 (one thread) issues the TMA loads, each stage
// once the converters of the tile before are done with it; warps 0..7 run the epilogue. B is
// rebuilt by the group whose tile is the first of a new instance, once the previous tile's
// products are done.
//   bar_tma[s]      stage s holds the rows of its tile                 (TMA transaction bytes)
//   bar_afull[s]    slot s holds its K half (and its stage rows are read)       (128 arrivals)
//   bar_afree[s]    the products reading slot s are done                        (tcgen05.commit)
//   bar_mma[b]      accumulator b holds a finished product                      (tcgen05.commit)
//   bar_epi[b]      the epilogue is done reading accumulator b                  (256 arrivals)
//   bar_sfree[s]    the converters are done with stage s                        (128 arrivals)
//   bar_fin         every product this block issued is done           (tcgen05.commit, on abort)
//   bar_rs[i % 4]   rmul of tile i is written (its converter group)                (128 arrivals)
// The converters and the epilogue load what they need about a tile a tile ahead (register prefetch
// of the work items and segments); the MMA warp reads each tile's D from s_dim, written by the
// converters.
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

// An mbarrier wait that also gives up once another role has raised the abort flag (checked between
// suspend-hinted tests), or after the wait budget.
__device__ __forceinline__ bool wait_or_abort(uint64_t *bar, uint32_t parity, volatile int *abort_flag)
{
    const long long t0 = clock64();
    while (!tc::mbar_try_wait_sleep(bar, parity, 20000u))
        if (*abort_flag != 0 || clock64() - t0 > kWaitBudget) return false;
    return true;
}

__global__ void __launch_bounds__(kThreadsTc, 1) k_evaluate_tc(const __grid_constant__ CUtensorMap xmap, EvalTcArgs a)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    const TcLayout L = tc_layout(a.dim_hi, a.ld, a.nstage);
    const int ns = a.nstage;
    float *stage[kMaxStages];
#pragma unroll
    for (int k = 0; k < kMaxStages; ++k) stage[k] = reinterpret_cast<float *>(smem + (size_t)k * L.stage_bytes);
    uint8_t *b_hi = smem + L.off_b;
    float *so = reinterpret_cast<float *>(smem + L.off_o);
    float *psum = reinterpret_cast<float *>(smem + L.off_psum);
    float *rmul = reinterpret_cast<float *>(smem + L.off_rmul);
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + L.off_bar);
    uint64_t *bar_tma = bars, *bar_mma = bars + 3, *bar_epi = bars + 6, *bar_afull = bars + 9, *bar_afree = bars + 11,
             *bar_fin = bars + 15, *bar_rs = bars + 18, *bar_sfree = bars + 26;
    // tile i's D, written by its converters before their first A half is handed over (ring of 4)
    int *s_dim = reinterpret_cast<int *>(bars + 29);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(bars + 16);
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 17);
    float *red = reinterpret_cast<float *>(bars + 22);  // 2 x 4 floats: each converter group's |M| maxima
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    if (warp == 0) {
        tc::tmem_alloc(tmem_slot, kTmemAlloc);
        tc::tmem_relinquish();
    }
    if (tid == 32) {
        for (int k = 0; k < kMaxStages; ++k) {
            tc::mbar_init(&bar_tma[k], 1);
            tc::mbar_init(&bar_sfree[k], 128);
        }
        for (int b = 0; b < kAcc; ++b) {
            tc::mbar_init(&bar_mma[b], 1);
            tc::mbar_init(&bar_epi[b], kEpiThreads);
        }
        for (int k = 0; k < kSlots; ++k) {
            tc::mbar_init(&bar_afull[k], 128);
            tc::mbar_init(&bar_afree[k], 1);
        }
        tc::mbar_init(bar_fin, 1);
        for (int k = 0; k < 4; ++k) tc::mbar_init(&bar_rs[k], 128);
        *abort_flag = 0;
        tc::fence_mbar_init();
        tc::prefetch_tensormap(&xmap);
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tmem_slot;
    const int nslot = kSlots;
    // K half h of tile i: its slot, the slot's column, and how often the slot was used before
    auto slot_of = [&](int i, int h) { return (2 * i + h) % nslot; };
    auto use_of = [&](int i, int h) { return (2 * i + h) / nslot; };
    auto slot_col = [&](int sl) { return tmem + (uint32_t)(kAcc * L.kmax + kSlotCols * sl); };

    const int my_items = a.n_items > (int)blockIdx.x ? (a.n_items - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    auto item_of = [&](int i) { return a.items[blockIdx.x + (i < my_items ? i : my_items - 1) * gridDim.x]; };
    int tma_issued = 0;      // TMA bookkeeping (warp kTmaWarp, lane 0)
    bool mma_any = false;

    if (warp == kTmaWarp) {
        // ---- TMA issue, lane 0: tile i into stage i % ns once the converters of tile i - ns have
        // finished with that stage --------------------------------------------------------------
        if (lane == 0) {
            for (int i = 0; i < my_items; ++i) {
                const int sidx = i % ns;
                const TileInfo t = tile_info(a, item_of(i));
                if (i >= ns && !wait_or_abort(&bar_sfree[sidx], (uint32_t)((i / ns - 1) & 1), abort_flag)) {
                    *abort_flag = 1;
                    break;
                }
                tc::mbar_arrive_expect_tx(&bar_tma[sidx], (uint32_t)L.stage_bytes);
                tc::tma_load_2d(stage[sidx], &xmap, 0, t.ok ? (int)t.row : 0, &bar_tma[sidx]);
                tma_issued = i + 1;
            }
        }
    } else if (warp == kIssuerWarp) {
        // ---- MMA issue: the whole warp runs the loop, lane 0 issues ------------------------------
        const bool leader = lane == 0;
        for (int i = 0; i < my_items; ++i) {
            const int b = i % kAcc;
            const int sl0 = slot_of(i, 0), sl1 = slot_of(i, 1);
            bool ok = tc::mbar_wait_sleep(&bar_afull[sl0], (uint32_t)(use_of(i, 0) & 1), kWaitBudget);
            if (i >= kAcc)
                ok = ok && tc::mbar_wait_sleep(&bar_epi[b], (uint32_t)((i / kAcc - 1) & 1), kWaitBudget);
            if (!__all_sync(0xffffffffu, ok && *abort_flag == 0)) { *abort_flag = 1; break; }
            tc::fence_after_sync();
            const int Kp = round16(s_dim[i & 3]), S = Kp / 16, s_half = (S + 1) / 2;
            const uint32_t acc = tmem + (uint32_t)(b * L.kmax);
            if (leader) {
                issue_split_mma(acc, slot_col(sl0), kApart, b_hi, L.b_bytes, Kp, Kp, 0, s_half);
                tc::mma_commit(&bar_afree[sl0]);
                mma_any = true;
            }
            ok = tc::mbar_wait_sleep(&bar_afull[sl1], (uint32_t)(use_of(i, 1) & 1), kWaitBudget);
            if (!__all_sync(0xffffffffu, ok && *abort_flag == 0)) { *abort_flag = 1; break; }
            tc::fence_after_sync();
            if (leader) {
                // the slot holds steps s_half .. S - 1 from its first column
                issue_split_mma(acc, slot_col(sl1) - (uint32_t)(8 * s_half), kApart, b_hi, L.b_bytes, Kp, Kp, s_half,
                                S);
                tc::mma_commit(&bar_mma[b]);
                tc::mma_commit(&bar_afree[sl1]);
            }
            __syncwarp();
        }
    } else if (warp >= kEpiThreads / 32) {
        // ---- conversion: group g = tiles g, g + 2, ...; thread = row 32 q + lane, both K halves ----
        const int g = (warp - kEpiThreads / 32) >> 2, q = warp & 3, gt = q * 32 + lane;
        const int gbar = g == 0 ? 1 : 6;  // the group's named barrier (128 threads)
        const int m = q * 32 + lane;
        const uint32_t lane_off = (uint32_t)(q * 32) << 16;
        float *so_g = so + g * L.kmax;
        float *red_g = red + 4 * g;
        const float *g_rot = nullptr, *g_shift = nullptr;
        int g_dim = -1, g_ldrot = -1, g_km = 0;
        auto same_inst = [](const TileInfo &x, const TileInfo &y) {
            return x.rot == y.rot && x.shift == y.shift && x.D == y.D && x.ld_rot == y.ld_rot;
        };
        TileInfo prv = tile_info(a, item_of(g > 0 ? g - 1 : 0)), cur = tile_info(a, item_of(g));
        for (int i = g; i < my_items; i += 2) {
            const TileInfo prv_n = tile_info(a, item_of(i + 1)), cur_n = tile_info(a, item_of(i + 2));
            const int sidx = i % ns;
            const int D = cur.D, Kp = round16(D), S = Kp / 16, s_half = (S + 1) / 2;
            float *row = stage[sidx] + (size_t)m * L.box_x;
            const bool live = cur.ok && m < cur.count;
            bool to = !tc::mbar_wait_sleep(&bar_tma[sidx], (uint32_t)((i / ns) & 1), kWaitBudget);
            const bool new_inst = cur.ok && (cur.rot != g_rot || cur.shift != g_shift || D != g_dim ||
                                             cur.ld_rot != g_ldrot);
            // B holds the instance of tile i - 1 when that tile was valid
            const bool new_b = cur.ok && (i == 0 || !prv.ok || !same_inst(cur, prv));
            // B is read by every product of the previous tile: rebuild it once those are done
            if (new_b && i >= 1)
                to |= !tc::mbar_wait_sleep(&bar_mma[(i - 1) % kAcc], (uint32_t)(((i - 1) / kAcc) & 1), kWaitBudget);
            // the group's decision to stop is reduced over its threads, so that none waits at its
            // named barrier for one that left
            if (tc::named_bar_or(gbar, 128, to || *abort_flag != 0)) { *abort_flag = 1; break; }
            if (new_inst || new_b) {
                speo_segment sb;
                sb.dim = D; sb.rot = cur.rot; sb.shift = cur.shift; sb.ld_rot = cur.ld_rot;
                if (new_inst) {
                    // a new instance for this group: o, and k_M from the largest |M|; when B changes
                    // too, one pass over M builds it with 2^14 while finding that value (b_exp keeps
                    // 14 for the usual range; a second pass otherwise)
                    float bm = new_b ? build_b(sb, Kp, b_hi, L.b_bytes, so_g, gt, 128, tcs::pow2i(14))
                                     : tcs::b_absmax(sb, gt, 128);
                    for (int o = 16; o > 0; o >>= 1) bm = fmaxf(bm, __shfl_xor_sync(0xffffffffu, bm, o));
                    if (lane == 0) red_g[q] = bm;
                    for (int k = gt; k < Kp; k += 128) so_g[k] = k < D ? cur.shift[k] : 0.f;
                    tc::named_bar_sync(gbar, 128);
                    bm = fmaxf(fmaxf(red_g[0], red_g[1]), fmaxf(red_g[2], red_g[3]));
                    g_km = tcs::b_exp(bm);
                    g_rot = cur.rot; g_shift = cur.shift; g_dim = D; g_ldrot = cur.ld_rot;
                    if (new_b && g_km != 14) build_b(sb, Kp, b_hi, L.b_bytes, so_g, gt, 128, tcs::pow2i(g_km));
                } else {
                    // B changed under this group (the other group's tile), the instance did not
                    build_b(sb, Kp, b_hi, L.b_bytes, so_g, gt, 128, tcs::pow2i(g_km));
                }
                if (new_b) tc::fence_proxy_async_smem();
                tc::named_bar_sync(gbar, 128);  // B, o and red are complete
            }
            if (!cur.ok && gt == 0) atomicOr(&s_deverr, SPEO_DEVERR_BAD_SEGMENT);
            // y = x - o replaces x in the staged row (columns < D) while the largest |y| is found;
            // the conversion then reads y
            float mx = 0.f;
            if (live) {
                for (int k = 0; k < D; k += 4) {
                    const float4 x = *reinterpret_cast<const float4 *>(row + k);
                    const float4 o = *reinterpret_cast<const float4 *>(so_g + k);
                    float4 y;
                    tc::upk2(tc::sub2(tc::pk2(x.x, x.y), tc::pk2(o.x, o.y)), y.x, y.y);
                    tc::upk2(tc::sub2(tc::pk2(x.z, x.w), tc::pk2(o.z, o.w)), y.z, y.w);
                    if (k + 4 > D) {  // the row's own padding past D: zero, as the conversion reads it
                        if (k + 1 >= D) y.y = 0.f;
                        if (k + 2 >= D) y.z = 0.f;
                        y.w = 0.f;
                    }
                    mx = fmaxf(fmaxf(mx, fabsf(y.x)), fmaxf(fabsf(y.y), fmaxf(fabsf(y.z), fabsf(y.w))));
                    *reinterpret_cast<float4 *>(row + k) = y;
                }
            }
            const int k_row = tcs::scale_exp(mx);
            const float rs = tcs::pow2i(k_row);
            bool ok = true;
            for (int h = 0; h < 2 && ok; ++h) {
                // the slot of this K half was last read by the products of the half four half-steps back
                const int sl = slot_of(i, h), u = use_of(i, h);
                ok = u < 1 || tc::mbar_wait_sleep(&bar_afree[sl], (uint32_t)((u - 1) & 1), kWaitBudget);
                if (!__all_sync(0xffffffffu, ok)) { ok = false; break; }
                if (h == 0) {
                    // the epilogue of tile i - 4, the last reader of rmul[i % 4], finished before
                    // the products that freed this slot were issued
                    rmul[(i & 3) * kTileM + m] = tcs::row_scale(func_scale(cur.func), g_km, k_row);
                    tc::mbar_arrive(&bar_rs[i & 3]);
                    if (gt == 0) s_dim[i & 3] = D;
                }
                const int s0 = h == 0 ? 0 : s_half, s1 = h == 0 ? s_half : S;
                for (int st = s0; st < s1; ++st) {
                    uint32_t hi[8], lo[8];
                    float v[16];
#pragma unroll
                    for (int q4 = 0; q4 < 4; ++q4) {
                        const int k = 16 * st + 4 * q4;
                        const float4 y = (live && k < D) ? *reinterpret_cast<const float4 *>(row + k)
                                                         : make_float4(0.f, 0.f, 0.f, 0.f);
                        v[4 * q4 + 0] = y.x; v[4 * q4 + 1] = y.y; v[4 * q4 + 2] = y.z; v[4 * q4 + 3] = y.w;
                    }
                    tcs::split16(v, rs, hi, lo);
                    const uint32_t col = slot_col(sl) + lane_off + (uint32_t)(8 * (st - s0));
                    tc::tmem_st32x8(col, hi);
                    tc::tmem_st32x8(col + (uint32_t)kApart, lo);
                }
                tc::tmem_wait_st();
                tc::fence_before_sync();
                tc::mbar_arrive(&bar_afull[sl]);
            }
            if (!ok) *abort_flag = 1;  // the next tile's barrier stops the group
            else tc::mbar_arrive(&bar_sfree[sidx]);  // this group's reads of the staged tile are done
            prv = prv_n;
            cur = cur_n;
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
            const bool got = tc::mbar_wait_sleep(&bar_mma[i % kAcc], (uint32_t)((i / kAcc) & 1), kWaitBudget) &&
                             tc::mbar_wait_sleep(&bar_rs[i & 3], (uint32_t)((i >> 2) & 1), kWaitBudget);
            if (tc::named_bar_or(2 + q, 64, !got)) { *abort_flag = 1; break; }
            tc::fence_after_sync();
            const uint32_t acc_t = tmem + (uint32_t)((i % kAcc) * L.kmax);
            const int Np = round16(cur.D), m = q * 32 + lane;
            const float rsc = rmul[(i & 3) * kTileM + m];
            float f = 0.f;
            bool writer = ch == 0;
            if (func_sum_form(cur.func)) {
                // columns [0, h) on the first warp of the quarter, [h, D) on the second
                // (tcs::epi_split); the second warp's partial sums meet the first's through psum[i % 2]
                const int h = tcs::epi_split(cur.D);
                const int c0 = ch == 0 ? 0 : h, c1 = ch == 0 ? (cur.D < h ? cur.D : h) : cur.D;
                f = c0 < c1 ? epilogue_row(acc_t, warp, cur.D, c0, c1, cur.func, rsc) : 0.f;
                float *ps = psum + (i & 1) * kTileM;
                if (ch == 1) ps[m] = f;
                tc::named_bar_sync(2 + q, 64);
                if (ch == 0) f += ps[m];
            } else if (ch == 0) {
                f = epilogue_row_generic(acc_t, warp, cur.D, Np, cur.func, rsc);
            }
            if (writer && cur.ok && m < cur.count) a.fit[cur.row + m] = f;
            tc::fence_before_sync();
            tc::mbar_arrive(&bar_epi[i % kAcc]);
            cur = nxt;
            it_next = it_nn;
        }
    }
    __syncthreads();
    if (*abort_flag && lane == 0) {
        // Let the copies and products this block started finish (bounded) before its shared and
        // tensor memory are released.
        if (warp == kTmaWarp) {
            atomicOr(&s_deverr, SPEO_DEVERR_WAIT_TIMEOUT);
            for (int j = (tma_issued > ns ? tma_issued - ns : 0); j < tma_issued; ++j)
                tc::mbar_wait(&bar_tma[j % ns], (uint32_t)((j / ns) & 1), kWaitBudget);
        }
        if (warp == kIssuerWarp && mma_any) {
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
