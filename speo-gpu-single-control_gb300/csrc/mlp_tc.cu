// mlp_tc.cu -- the surrogate MLP's screening forward pass on the tcgen05 tensor cores.
//
// No counterpart in the reference. y = w3 . relu(W2 relu(W1 x' + b1) + b2) + b3 with
// x' = (x - mu) * isig, BF16 operands and FP32 accumulation:
//   * W1 (H x din, K padded to 64) and W2 (H x H) are packed once per call into BF16 images laid
//     out exactly as the K-major no-swizzle shared-memory operands, so one bulk copy per image
//     brings them into shared memory, where they stay for every tile the block processes;
//   * per 128-row tile: the block standardises and converts the rows into the A operand, one
//     thread issues layer 1 (M = 128, N = H, K = 64) into tensor memory, all 16 warps read the
//     accumulators back (bias, ReLU, BF16; four warps per TMEM lane quarter, each a quarter of
//     the columns) into the layer-2 A operand, layer 2 (K = H) reuses the same tensor-memory
//     columns, and the epilogue folds bias, ReLU and the H -> 1 head into per-row dot products
//     of each column quarter, added in a fixed order.
// H is 64, 128 or 256 (tensor-memory columns = H). Every wait is bounded; a timeout sets the
// device error word and the block returns after releasing its tensor memory.
#include <cuda_bf16.h>

#include "common.cuh"
#include "host.h"
#include "tcgen05.cuh"

SPEO_DEFINE_DEVERR(speo_deverr_mlp)

namespace speo {
namespace {

constexpr int kRows = 128;                       // rows per tile (MMA M)
constexpr int kK1 = 64;                          // layer-1 K (din padded)
constexpr long long kWaitBudget = 2000000000LL;  // ~1 s at 2 GHz
constexpr int kFwdThreads = 512;                 // screening forward: 16 warps
constexpr int kFwdParts = 4;                     // column parts of a row in its epilogues (H >= 128)

__host__ __device__ constexpr size_t w1_bytes(int H) { return (size_t)H * kK1 * 2; }
__host__ __device__ constexpr size_t w2_bytes(int H) { return (size_t)H * H * 2; }
__host__ __device__ constexpr size_t a_bytes(int H) { return (size_t)kRows * (H > kK1 ? H : kK1) * 2; }
__host__ __device__ constexpr size_t smem_total(int H)
{
    return w1_bytes(H) + w2_bytes(H) + a_bytes(H) + kFwdParts * kRows * sizeof(float) + 64;
}

__device__ __forceinline__ uint32_t bf2(float a, float b)
{
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t *>(&h);
}

// Weight images: chunk (n, kc) = 8 consecutive K elements of row n, as one 16-byte core-matrix row.
// Image 1: W1 (n = hidden unit, k = input); image 2: W2 (n = output unit i, k = input unit j);
// image 3 (with_t): W2^T (n = j, k = i), the B operand of dZ1 = dZ2 W2.
template <int H>
__global__ void k_pack_mlp(const float *__restrict__ theta, int din, uint8_t *__restrict__ img, int with_t)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    constexpr int c1 = H * (kK1 / 8), c2 = H * (H / 8);
    if (t >= c1 + c2 + (with_t ? c2 : 0)) return;
    const float *W1 = theta;
    const float *W2 = theta + (size_t)H * din + H;
    float v[8];
    uint32_t off;
    if (t < c1) {
        const int n = t / (kK1 / 8), k0 = (t % (kK1 / 8)) * 8;
#pragma unroll
        for (int j = 0; j < 8; ++j) v[j] = k0 + j < din ? W1[(size_t)n * din + k0 + j] : 0.f;
        off = tc::kmajor_offset(n, k0, kK1);
    } else if (t < c1 + c2) {
        const int u = t - c1, n = u / (H / 8), k0 = (u % (H / 8)) * 8;
#pragma unroll
        for (int j = 0; j < 8; ++j) v[j] = W2[(size_t)n * H + k0 + j];
        off = (uint32_t)w1_bytes(H) + tc::kmajor_offset(n, k0, H);
    } else {
        const int u = t - c1 - c2, n = u / (H / 8), k0 = (u % (H / 8)) * 8;
#pragma unroll
        for (int j = 0; j < 8; ++j) v[j] = W2[(size_t)(k0 + j) * H + n];
        off = (uint32_t)(w1_bytes(H) + w2_bytes(H)) + tc::kmajor_offset(n, k0, H);
    }
    *reinterpret_cast<uint4 *>(img + off) =
        make_uint4(bf2(v[0], v[1]), bf2(v[2], v[3]), bf2(v[4], v[5]), bf2(v[6], v[7]));
}

__device__ __forceinline__ void bulk_load(void *dst, const void *src, uint32_t bytes, uint64_t *bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     tc::smem_u32(dst)),
                 "l"((uint64_t)src), "r"(bytes), "r"(tc::smem_u32(bar))
                 : "memory");
}

struct MlpArgs {
    const uint8_t *img;   // packed W1 | W2 images
    const float *b1, *b2, *w3, *b3;
    const float *mu, *isig;
    const float *X;
    long long n;
    int ldx, din, vec;    // vec: rows 16-byte aligned (X aligned, ldx % 4 == 0)
    float *y;
};

template <int H>
__global__ void __launch_bounds__(kFwdThreads, 1) k_mlp_fwd_tc(MlpArgs a)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t *sw1 = smem, *sw2 = smem + w1_bytes(H), *sa = sw2 + w2_bytes(H);
    float *red = reinterpret_cast<float *>(sa + a_bytes(H));
    uint64_t *bars = reinterpret_cast<uint64_t *>(red + kFwdParts * kRows);
    uint64_t *bar_w = bars, *bar_mma = bars + 1;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 2);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    if (warp == 0) {
        tc::tmem_alloc(tmem_slot, H);
        tc::tmem_relinquish();
    }
    if (tid == 32) {
        tc::mbar_init(bar_w, 1);
        tc::mbar_init(bar_mma, 1);
        tc::fence_mbar_init();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tmem_slot;
    if (tid == 0) {
        const uint32_t total = (uint32_t)(w1_bytes(H) + w2_bytes(H));
        tc::mbar_arrive_expect_tx(bar_w, total);
        for (uint32_t o = 0; o < total; o += 32768u)
            bulk_load(smem + o, a.img + o, total - o < 32768u ? total - o : 32768u, bar_w);
    }
    bool ok = tc::mbar_wait(bar_w, 0, kWaitBudget);
    bool abort = __syncthreads_or(!ok) != 0;

    constexpr uint32_t idesc = tc::idesc_bf16_f32(kRows, H);
    const uint32_t sa_u = tc::smem_u32(sa), sw1_u = tc::smem_u32(sw1), sw2_u = tc::smem_u32(sw2);
    // TMEM lane quadrant and column part (H / kParts columns; H = 64 uses two parts of 32)
    constexpr int kParts = H >= 128 ? kFwdParts : 2, kPartCols = H / kParts;
    const int q = warp & 3, part = warp >> 2;
    const int row_l = 32 * q + lane;                // tile row this thread reads back
    const uint32_t t_row = tmem + ((uint32_t)(32 * q) << 16);
    const long long ntiles = (a.n + kRows - 1) / kRows;
    uint32_t phase = 0;
    int mma_pending = 0;  // a commit whose wait gave up

    // This thread's share of a tile's inputs: rows r = tid % 128 (lanes = consecutive rows, so
    // each 8-lane phase of the shared-memory stores covers 128 contiguous bytes), 16-byte chunks
    // k0 = 8 ((tid + 512 j) / 128). The next tile's rows are loaded into registers before the
    // current tile's products start, so their latency overlaps the tensor-core work.
    constexpr int kItems = kRows * (kK1 / 8) / kFwdThreads;
    float xin[kItems][8];
    auto load_rows = [&](long long r0) {
#pragma unroll
        for (int j = 0; j < kItems; ++j) {
            const int item = tid + kFwdThreads * j;
            const int r = item % kRows, k0 = (item / kRows) * 8;
            const long long gr = r0 + r;
#pragma unroll
            for (int e = 0; e < 8; ++e) xin[j][e] = 0.f;
            if (gr < a.n) {
                const float *xr = a.X + gr * a.ldx;
                if (a.vec && k0 + 8 <= a.din) {
                    const float4 p = *reinterpret_cast<const float4 *>(xr + k0);
                    const float4 q = *reinterpret_cast<const float4 *>(xr + k0 + 4);
                    xin[j][0] = p.x; xin[j][1] = p.y; xin[j][2] = p.z; xin[j][3] = p.w;
                    xin[j][4] = q.x; xin[j][5] = q.y; xin[j][6] = q.z; xin[j][7] = q.w;
                } else {
#pragma unroll
                    for (int e = 0; e < 8; ++e) xin[j][e] = k0 + e < a.din ? xr[k0 + e] : 0.f;
                }
            }
        }
    };
    if (blockIdx.x < ntiles) load_rows((long long)blockIdx.x * kRows);

    for (long long tile = blockIdx.x; tile < ntiles && !abort; tile += gridDim.x) {
        const long long r0 = tile * kRows;
        // ---- A1 = bf16((x - mu) * isig), zero past din and past n ----------------------------
#pragma unroll
        for (int j = 0; j < kItems; ++j) {
            const int item = tid + kFwdThreads * j;
            const int r = item % kRows, k0 = (item / kRows) * 8;
            float v[8];
#pragma unroll
            for (int e = 0; e < 8; ++e)
                v[e] = (k0 + e < a.din && r0 + r < a.n) ? __fmul_rn(__fsub_rn(xin[j][e], a.mu[k0 + e]), a.isig[k0 + e])
                                                        : 0.f;
            *reinterpret_cast<uint4 *>(sa + tc::kmajor_offset(r, k0, kK1)) =
                make_uint4(bf2(v[0], v[1]), bf2(v[2], v[3]), bf2(v[4], v[5]), bf2(v[6], v[7]));
        }
        if (tile + gridDim.x < ntiles) load_rows((tile + gridDim.x) * kRows);
        tc::fence_proxy_async_smem();
        tc::fence_before_sync();
        __syncthreads();
        if (tid == 0) {
            tc::fence_after_sync();
#pragma unroll
            for (int kk = 0; kk < kK1 / 16; ++kk)
                tc::mma_bf16(tmem, tc::smem_desc(sa_u + kk * 256, 128, kK1 * 16),
                             tc::smem_desc(sw1_u + kk * 256, 128, kK1 * 16), idesc, kk > 0);
            tc::mma_commit(bar_mma);
        }
        ok = tc::mbar_wait(bar_mma, phase, kWaitBudget);
        if (__syncthreads_or(!ok)) { abort = true; mma_pending = 1; break; }
        phase ^= 1u;
        tc::fence_after_sync();
        // ---- H1 = bf16(relu(acc + b1)) into the layer-2 A operand ------------------------------
#pragma unroll 1
        for (int c0 = part * kPartCols; part < kParts && c0 < (part + 1) * kPartCols; c0 += 32) {
            uint32_t r[32];
            tc::tmem_ld32(t_row + (uint32_t)c0, r);
#pragma unroll
            for (int g = 0; g < 4; ++g) {
                float v[8];
#pragma unroll
                for (int e = 0; e < 8; ++e) v[e] = fmaxf(__fadd_rn(__uint_as_float(r[8 * g + e]), a.b1[c0 + 8 * g + e]), 0.f);
                *reinterpret_cast<uint4 *>(sa + tc::kmajor_offset(row_l, c0 + 8 * g, H)) =
                    make_uint4(bf2(v[0], v[1]), bf2(v[2], v[3]), bf2(v[4], v[5]), bf2(v[6], v[7]));
            }
        }
        tc::fence_proxy_async_smem();
        tc::fence_before_sync();
        __syncthreads();
        if (tid == 0) {
            tc::fence_after_sync();
#pragma unroll 4
            for (int kk = 0; kk < H / 16; ++kk)
                tc::mma_bf16(tmem, tc::smem_desc(sa_u + kk * 256, 128, H * 16),
                             tc::smem_desc(sw2_u + kk * 256, 128, H * 16), idesc, kk > 0);
            tc::mma_commit(bar_mma);
        }
        ok = tc::mbar_wait(bar_mma, phase, kWaitBudget);
        if (__syncthreads_or(!ok)) { abort = true; mma_pending = 1; break; }
        phase ^= 1u;
        tc::fence_after_sync();
        // ---- y = b3 + sum_c relu(acc + b2) w3 ----------------------------------------------------
        float s = 0.f;
#pragma unroll 1
        for (int c0 = part * kPartCols; part < kParts && c0 < (part + 1) * kPartCols; c0 += 32) {
            uint32_t r[32];
            tc::tmem_ld32(t_row + (uint32_t)c0, r);
#pragma unroll
            for (int e = 0; e < 32; ++e)
                s = __fmaf_rn(fmaxf(__fadd_rn(__uint_as_float(r[e]), a.b2[c0 + e]), 0.f), a.w3[c0 + e], s);
        }
        if (part < kParts) red[part * kRows + row_l] = s;
        tc::fence_before_sync();
        __syncthreads();
        if (tid < kRows && r0 + tid < a.n) {
            float y = red[tid];
#pragma unroll
            for (int p = 1; p < kParts; ++p) y = __fadd_rn(y, red[p * kRows + tid]);
            a.y[r0 + tid] = __fadd_rn(y, a.b3[0]);
        }
    }
    if (abort && tid == 0) {
        // let the copy and the products this block started finish (bounded) before its shared and
        // tensor memory are released
        atomicOr(&s_deverr, SPEO_DEVERR_WAIT_TIMEOUT);
        tc::mbar_wait(bar_w, 0, kWaitBudget);
        if (mma_pending) tc::mbar_wait(bar_mma, phase, kWaitBudget);
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (warp == 0) tc::tmem_dealloc(tmem, H);
}

template <int H>
int launch_fwd(const MlpArgs &a, cudaStream_t st)
{
    const size_t smem = smem_total(H);
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if ((size_t)optin < smem) return fail(SPEO_ERR_UNSUPPORTED, "mlp forward (H = %d): needs %zu B of shared memory", H, smem);
    cudaError_t e = cudaFuncSetAttribute(k_mlp_fwd_tc<H>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return check_cuda(e, "cudaFuncSetAttribute(k_mlp_fwd_tc)");
    // blocks per SM bounded by shared memory and by tensor memory (512 columns)
    int per_sm = (int)((size_t)optin / smem);
    if (per_sm > 512 / H) per_sm = 512 / H;
    if (per_sm < 1) per_sm = 1;
    const long long ntiles = (a.n + kRows - 1) / kRows;
    const long long cap = (long long)sm_count() * per_sm;
    const int grid = (int)(ntiles < cap ? ntiles : cap);
    k_mlp_fwd_tc<H><<<grid, kFwdThreads, smem, st>>>(a);
    return check_launch("k_mlp_fwd_tc");
}

template <int H>
int pack(const float *theta, int din, uint8_t *img, cudaStream_t st, int with_t = 0)
{
    const int total = H * (kK1 / 8) + H * (H / 8) * (with_t ? 2 : 1);
    k_pack_mlp<H><<<(total + 255) / 256, 256, 0, st>>>(theta, din, img, with_t);
    return check_launch("k_pack_mlp");
}

// ================================ training (one Adam step's gradient) ================================
// Batch rows are padded to rp (a multiple of 128); padded rows have dy = 0 and contribute nothing.
// k_mlp_train_tc, one block per 128-row tile:
//   A1 = bf16(x') -> Z1 = A1 W1^T (TMEM) -> H1 = bf16(relu(Z1 + b1)) -> Z2 = H1 W2^T (TMEM)
//   -> y, dy = 2 (y - t) / n -> dZ2 = bf16(dy w3 1[Z2 + b2 > 0]) -> dZ1 = (dZ2 W2) 1[Z1 + b1 > 0]
// writing the transposed BF16 operands of the weight gradients (x'^T, H1^T, H2^T, dZ2^T, dZ1^T,
// each [features][rp]) and dy. W2^T replaces W2 in shared memory once layer 2 has finished.
struct TrainArgs {
    const uint8_t *img;  // W1 | W2 | W2^T images
    const float *b1, *b2, *w3, *b3, *mu, *isig;
    const float *X, *T;  // batch rows, or null: drawn from the archive (arch)
    MlpArchive arch;
    int n, ldx, din, vec;
    long long rp;
    float two_over_n;
    uint16_t *xnT, *h1T, *h2T, *dz2T, *dz1T;
    float *dy, *loss;
};

__host__ __device__ constexpr size_t train_smem(int H)
{
    return w1_bytes(H) + w2_bytes(H) + a_bytes(H) + 3 * kRows * sizeof(float) + 64;
}

__device__ __forceinline__ uint16_t lo16(uint32_t p) { return (uint16_t)(p & 0xffffu); }
__device__ __forceinline__ uint16_t hi16(uint32_t p) { return (uint16_t)(p >> 16); }

template <int H>
__global__ void __launch_bounds__(256, 1) k_mlp_train_tc(TrainArgs a)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t *sw1 = smem, *sw2 = smem + w1_bytes(H), *sa = sw2 + w2_bytes(H);
    float *red = reinterpret_cast<float *>(sa + a_bytes(H));
    float *dys = red + 2 * kRows;
    uint64_t *bars = reinterpret_cast<uint64_t *>(dys + kRows);
    uint64_t *bar_w = bars, *bar_wt = bars + 1, *bar_mma = bars + 2;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 3);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    if (warp == 0) {
        tc::tmem_alloc(tmem_slot, H);
        tc::tmem_relinquish();
    }
    if (tid == 32) {
        tc::mbar_init(bar_w, 1);
        tc::mbar_init(bar_wt, 1);
        tc::mbar_init(bar_mma, 1);
        tc::fence_mbar_init();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tmem_slot;
    if (tid == 0) {
        const uint32_t total = (uint32_t)(w1_bytes(H) + w2_bytes(H));
        tc::mbar_arrive_expect_tx(bar_w, total);
        for (uint32_t o = 0; o < total; o += 32768u)
            bulk_load(smem + o, a.img + o, total - o < 32768u ? total - o : 32768u, bar_w);
    }
    const long long r0 = (long long)blockIdx.x * kRows;
    const long long rp = a.rp;
    // this thread's batch row (tid % 128) and, when drawn from the archive, its slot
    const float *xrow = nullptr, *trow = nullptr;
    {
        const long long gr = r0 + (tid % kRows);
        if (gr < a.n) {
            if (a.X) {
                xrow = a.X + gr * a.ldx;
                trow = a.T + gr;
            } else {
                const uint4 w = philox(make_uint4((uint32_t)(gr >> 2), a.arch.st->step, 0u, kTagSample),
                                       make_uint2(a.arch.key0, a.arch.key1));
                const long long slot = (long long)(pick(w, (uint32_t)(gr & 3)) % (uint32_t)a.arch.st->count);
                xrow = a.arch.AX + slot * a.arch.lda;
                trow = a.arch.AT + slot;
            }
        }
    }
    // ---- A1 and x'^T (lanes = consecutive rows: coalesced transposed writes) --------------------
#pragma unroll
    for (int j = 0; j < kRows * (kK1 / 8) / 256; ++j) {
        const int item = tid + 256 * j;
        const int r = item % kRows, k0 = (item / kRows) * 8;
        const long long gr = r0 + r;
        float v[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) v[e] = 0.f;
        if (gr < a.n) {
            const float *xr = xrow;
            if (a.vec && k0 + 8 <= a.din) {
                const float4 p = *reinterpret_cast<const float4 *>(xr + k0);
                const float4 q = *reinterpret_cast<const float4 *>(xr + k0 + 4);
                v[0] = p.x; v[1] = p.y; v[2] = p.z; v[3] = p.w; v[4] = q.x; v[5] = q.y; v[6] = q.z; v[7] = q.w;
            } else {
#pragma unroll
                for (int e = 0; e < 8; ++e) v[e] = k0 + e < a.din ? xr[k0 + e] : 0.f;
            }
#pragma unroll
            for (int e = 0; e < 8; ++e)
                v[e] = k0 + e < a.din ? __fmul_rn(__fsub_rn(v[e], a.mu[k0 + e]), a.isig[k0 + e]) : 0.f;
        }
        const uint32_t p0 = bf2(v[0], v[1]), p1 = bf2(v[2], v[3]), p2 = bf2(v[4], v[5]), p3 = bf2(v[6], v[7]);
        *reinterpret_cast<uint4 *>(sa + tc::kmajor_offset(r, k0, kK1)) = make_uint4(p0, p1, p2, p3);
        uint16_t *xt = a.xnT + (size_t)k0 * rp + gr;
        xt[0] = lo16(p0); xt[rp] = hi16(p0); xt[2 * rp] = lo16(p1); xt[3 * rp] = hi16(p1);
        xt[4 * rp] = lo16(p2); xt[5 * rp] = hi16(p2); xt[6 * rp] = lo16(p3); xt[7 * rp] = hi16(p3);
    }
    tc::fence_proxy_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    bool ok = tc::mbar_wait(bar_w, 0, kWaitBudget);
    int stage = 0;  // 1: MMA1 pending, 2: MMA2 pending, 3: W2^T copy pending, 4: MMA3 pending
    bool abort = __syncthreads_or(!ok) != 0;
    constexpr uint32_t idesc = tc::idesc_bf16_f32(kRows, H);
    const uint32_t sa_u = tc::smem_u32(sa), sw1_u = tc::smem_u32(sw1), sw2_u = tc::smem_u32(sw2);
    const int q = warp & 3, half = warp >> 2;
    const int row_l = 32 * q + lane;
    const long long grow = r0 + row_l;
    const uint32_t t_row = tmem + ((uint32_t)(32 * q) << 16);
    uint32_t m1[H / 64];  // 1[Z1 + b1 > 0] over this thread's H/2 columns
    do {
        if (abort) break;
        if (tid == 0) {
            tc::fence_after_sync();
#pragma unroll
            for (int kk = 0; kk < kK1 / 16; ++kk)
                tc::mma_bf16(tmem, tc::smem_desc(sa_u + kk * 256, 128, kK1 * 16),
                             tc::smem_desc(sw1_u + kk * 256, 128, kK1 * 16), idesc, kk > 0);
            tc::mma_commit(bar_mma);
        }
        stage = 1;
        ok = tc::mbar_wait(bar_mma, 0, kWaitBudget);
        if (__syncthreads_or(!ok)) { abort = true; break; }
        stage = 0;
        tc::fence_after_sync();
        // ---- H1 -> layer-2 A operand and H1^T --------------------------------------------------
#pragma unroll
        for (int ci = 0; ci < H / 64; ++ci) {
            const int c0 = half * (H / 2) + 32 * ci;
            uint32_t r[32];
            tc::tmem_ld32(t_row + (uint32_t)c0, r);
            uint32_t bits = 0;
#pragma unroll
            for (int g = 0; g < 4; ++g) {
                float v[8];
#pragma unroll
                for (int e = 0; e < 8; ++e) {
                    v[e] = fmaxf(__fadd_rn(__uint_as_float(r[8 * g + e]), a.b1[c0 + 8 * g + e]), 0.f);
                    bits |= (v[e] > 0.f ? 1u : 0u) << (8 * g + e);
                }
                const uint32_t p0 = bf2(v[0], v[1]), p1 = bf2(v[2], v[3]), p2 = bf2(v[4], v[5]), p3 = bf2(v[6], v[7]);
                *reinterpret_cast<uint4 *>(sa + tc::kmajor_offset(row_l, c0 + 8 * g, H)) = make_uint4(p0, p1, p2, p3);
                uint16_t *ht = a.h1T + (size_t)(c0 + 8 * g) * rp + grow;
                ht[0] = lo16(p0); ht[rp] = hi16(p0); ht[2 * rp] = lo16(p1); ht[3 * rp] = hi16(p1);
                ht[4 * rp] = lo16(p2); ht[5 * rp] = hi16(p2); ht[6 * rp] = lo16(p3); ht[7 * rp] = hi16(p3);
            }
            m1[ci] = bits;
        }
        tc::fence_proxy_async_smem();
        tc::fence_before_sync();
        __syncthreads();
        if (tid == 0) {
            tc::fence_after_sync();
#pragma unroll 4
            for (int kk = 0; kk < H / 16; ++kk)
                tc::mma_bf16(tmem, tc::smem_desc(sa_u + kk * 256, 128, H * 16),
                             tc::smem_desc(sw2_u + kk * 256, 128, H * 16), idesc, kk > 0);
            tc::mma_commit(bar_mma);
        }
        stage = 2;
        ok = tc::mbar_wait(bar_mma, 1, kWaitBudget);
        if (__syncthreads_or(!ok)) { abort = true; break; }
        stage = 3;
        tc::fence_after_sync();
        if (tid == 0) {  // layer 2 is done with W2: bring W2^T into its place
            const uint32_t total = (uint32_t)w2_bytes(H);
            tc::mbar_arrive_expect_tx(bar_wt, total);
            for (uint32_t o = 0; o < total; o += 32768u)
                bulk_load(sw2 + o, a.img + w1_bytes(H) + w2_bytes(H) + o, total - o < 32768u ? total - o : 32768u,
                          bar_wt);
        }
        // ---- y and dy ---------------------------------------------------------------------------
        float s = 0.f;
#pragma unroll 1
        for (int c0 = half * (H / 2); c0 < (half + 1) * (H / 2); c0 += 32) {
            uint32_t r[32];
            tc::tmem_ld32(t_row + (uint32_t)c0, r);
#pragma unroll
            for (int e = 0; e < 32; ++e)
                s = __fmaf_rn(fmaxf(__fadd_rn(__uint_as_float(r[e]), a.b2[c0 + e]), 0.f), a.w3[c0 + e], s);
        }
        red[half * kRows + row_l] = s;
        __syncthreads();
        if (tid < kRows) {
            const long long gr = r0 + tid;
            float e = 0.f;
            if (gr < a.n) e = __fsub_rn(__fadd_rn(__fadd_rn(red[tid], red[kRows + tid]), a.b3[0]), *trow);
            const float d = __fmul_rn(e, a.two_over_n);
            dys[tid] = d;
            a.dy[gr] = d;
            float e2 = e * e;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) e2 += __shfl_xor_sync(0xffffffffu, e2, o);
            if (lane == 0) atomicAdd(a.loss, e2);
        }
        __syncthreads();
        // ---- dZ2 -> layer-3 A operand, dZ2^T and H2^T --------------------------------------------
        const float dyr = dys[row_l];
#pragma unroll 1
        for (int c0 = half * (H / 2); c0 < (half + 1) * (H / 2); c0 += 32) {
            uint32_t r[32];
            tc::tmem_ld32(t_row + (uint32_t)c0, r);
#pragma unroll
            for (int g = 0; g < 4; ++g) {
                float dz[8], h2[8];
#pragma unroll
                for (int e = 0; e < 8; ++e) {
                    const int c = c0 + 8 * g + e;
                    const float z = __fadd_rn(__uint_as_float(r[8 * g + e]), a.b2[c]);
                    h2[e] = fmaxf(z, 0.f);
                    dz[e] = z > 0.f ? __fmul_rn(dyr, a.w3[c]) : 0.f;
                }
                const uint32_t p0 = bf2(dz[0], dz[1]), p1 = bf2(dz[2], dz[3]), p2 = bf2(dz[4], dz[5]), p3 = bf2(dz[6], dz[7]);
                *reinterpret_cast<uint4 *>(sa + tc::kmajor_offset(row_l, c0 + 8 * g, H)) = make_uint4(p0, p1, p2, p3);
                uint16_t *dt = a.dz2T + (size_t)(c0 + 8 * g) * rp + grow;
                dt[0] = lo16(p0); dt[rp] = hi16(p0); dt[2 * rp] = lo16(p1); dt[3 * rp] = hi16(p1);
                dt[4 * rp] = lo16(p2); dt[5 * rp] = hi16(p2); dt[6 * rp] = lo16(p3); dt[7 * rp] = hi16(p3);
                const uint32_t u0 = bf2(h2[0], h2[1]), u1 = bf2(h2[2], h2[3]), u2 = bf2(h2[4], h2[5]), u3 = bf2(h2[6], h2[7]);
                uint16_t *h2t = a.h2T + (size_t)(c0 + 8 * g) * rp + grow;
                h2t[0] = lo16(u0); h2t[rp] = hi16(u0); h2t[2 * rp] = lo16(u1); h2t[3 * rp] = hi16(u1);
                h2t[4 * rp] = lo16(u2); h2t[5 * rp] = hi16(u2); h2t[6 * rp] = lo16(u3); h2t[7 * rp] = hi16(u3);
            }
        }
        tc::fence_proxy_async_smem();
        tc::fence_before_sync();
        __syncthreads();
        ok = tc::mbar_wait(bar_wt, 0, kWaitBudget);
        if (__syncthreads_or(!ok)) { abort = true; break; }
        stage = 4;
        if (tid == 0) {
            tc::fence_after_sync();
#pragma unroll 4
            for (int kk = 0; kk < H / 16; ++kk)
                tc::mma_bf16(tmem, tc::smem_desc(sa_u + kk * 256, 128, H * 16),
                             tc::smem_desc(sw2_u + kk * 256, 128, H * 16), idesc, kk > 0);
            tc::mma_commit(bar_mma);
        }
        ok = tc::mbar_wait(bar_mma, 0, kWaitBudget);
        if (__syncthreads_or(!ok)) { abort = true; break; }
        stage = 0;
        tc::fence_after_sync();
        // ---- dZ1^T = ((dZ2 W2) 1[Z1 > 0])^T -----------------------------------------------------
#pragma unroll
        for (int ci = 0; ci < H / 64; ++ci) {
            const int c0 = half * (H / 2) + 32 * ci;
            uint32_t r[32];
            tc::tmem_ld32(t_row + (uint32_t)c0, r);
#pragma unroll
            for (int g = 0; g < 4; ++g) {
                float v[8];
#pragma unroll
                for (int e = 0; e < 8; ++e) v[e] = (m1[ci] >> (8 * g + e)) & 1u ? __uint_as_float(r[8 * g + e]) : 0.f;
                const uint32_t p0 = bf2(v[0], v[1]), p1 = bf2(v[2], v[3]), p2 = bf2(v[4], v[5]), p3 = bf2(v[6], v[7]);
                uint16_t *dt = a.dz1T + (size_t)(c0 + 8 * g) * rp + grow;
                dt[0] = lo16(p0); dt[rp] = hi16(p0); dt[2 * rp] = lo16(p1); dt[3 * rp] = hi16(p1);
                dt[4 * rp] = lo16(p2); dt[5 * rp] = hi16(p2); dt[6 * rp] = lo16(p3); dt[7 * rp] = hi16(p3);
            }
        }
    } while (false);
    if (abort && tid == 0) {
        atomicOr(&s_deverr, SPEO_DEVERR_WAIT_TIMEOUT);
        tc::mbar_wait(bar_w, 0, kWaitBudget);
        if (stage == 1) tc::mbar_wait(bar_mma, 0, kWaitBudget);
        if (stage == 2) tc::mbar_wait(bar_mma, 1, kWaitBudget);
        if (stage == 3) tc::mbar_wait(bar_wt, 0, kWaitBudget);
        if (stage == 4) tc::mbar_wait(bar_mma, 0, kWaitBudget);
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (warp == 0) tc::tmem_dealloc(tmem, H);
}

// k_mlp_wgrad_tc, block (z, mh): rows chunk z (128 batch rows) and output half mh of the weight
// gradients, as two tcgen05 products with K = the 128 rows:
//   gW2[i][j] (+)= sum_r dZ2^T[i][r] H1^T[j][r]   (M = 128 rows i, N = H)
//   gW1[i][d] (+)= sum_r dZ1^T[i][r] x'^T[d][r]   (M = 128 rows i, N = 64)
// written to the chunk's partial-gradient vector (summed over chunks in a fixed order later).
struct WgradArgs {
    const uint16_t *xnT, *h1T, *dz2T, *dz1T;
    long long rp;
    int din, np;  // np: stride of the partial vectors (n_params rounded up to 4)
    float *gpart;
};

__host__ __device__ constexpr int wg_tmem_cols(int H) { return H + 64 <= 128 ? 128 : H + 64 <= 256 ? 256 : 512; }
__host__ __device__ constexpr size_t wg_smem(int H)
{
    return (size_t)kRows * 128 * 2 * 2 + (size_t)H * 128 * 2 + (size_t)kK1 * 128 * 2 + 64;
}

// Rows [row0, row0 + R) x columns [col0, col0 + 128) of a BF16 [*][ld] matrix into a K-major
// (K = the 128 columns) operand. A warp moves 8 rows x 4 chunks per step: 64 contiguous bytes per
// row from global memory, 128 contiguous bytes per 8 lanes into shared memory.
__device__ __forceinline__ void load_kmajor128(uint8_t *dst, const uint16_t *src, long long ld, int row0, long long col0,
                                               int R, int warp, int lane)
{
    const int r8 = lane & 7, kq = lane >> 3;
    for (int t = warp; t < (R / 8) * 4; t += 8 * 4) {
        uint4 v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int tt = t + 8 * u;
            if (tt < (R / 8) * 4) {
                const int row = 8 * (tt >> 2) + r8, kc = 4 * (tt & 3) + kq;
                v[u] = *reinterpret_cast<const uint4 *>(src + (size_t)(row0 + row) * ld + col0 + 8 * kc);
            }
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int tt = t + 8 * u;
            if (tt < (R / 8) * 4) {
                const int row = 8 * (tt >> 2) + r8, kc = 4 * (tt & 3) + kq;
                *reinterpret_cast<uint4 *>(dst + tc::kmajor_offset(row, 8 * kc, 128)) = v[u];
            }
        }
    }
}

template <int H>
__global__ void __launch_bounds__(256, 1) k_mlp_wgrad_tc(WgradArgs a)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t *sA2 = smem, *sA1 = smem + kRows * 128 * 2, *sB2 = sA1 + kRows * 128 * 2, *sB1 = sB2 + H * 128 * 2;
    uint64_t *bar_mma = reinterpret_cast<uint64_t *>(sB1 + kK1 * 128 * 2);
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bar_mma + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    constexpr int kCols = wg_tmem_cols(H);
    if (warp == 0) {
        tc::tmem_alloc(tmem_slot, kCols);
        tc::tmem_relinquish();
    }
    if (tid == 32) {
        tc::mbar_init(bar_mma, 1);
        tc::fence_mbar_init();
    }
    const int z = blockIdx.x, mh = blockIdx.y;
    const long long c0 = (long long)z * 128;
    const int ra = H - 128 * mh < kRows ? H - 128 * mh : kRows;  // valid rows i of this half (H = 64: 64)
    load_kmajor128(sA2, a.dz2T, a.rp, 128 * mh, c0, ra, warp, lane);
    load_kmajor128(sA1, a.dz1T, a.rp, 128 * mh, c0, ra, warp, lane);
    for (int o = ra * 256 + 16 * tid; o < kRows * 256; o += 16 * 256) {  // rows ra..127: zero
        *reinterpret_cast<uint4 *>(sA2 + o) = make_uint4(0u, 0u, 0u, 0u);
        *reinterpret_cast<uint4 *>(sA1 + o) = make_uint4(0u, 0u, 0u, 0u);
    }
    load_kmajor128(sB2, a.h1T, a.rp, 0, c0, H, warp, lane);
    load_kmajor128(sB1, a.xnT, a.rp, 0, c0, kK1, warp, lane);
    tc::fence_proxy_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tmem_slot;
    if (tid == 0) {
        const uint32_t a2 = tc::smem_u32(sA2), a1 = tc::smem_u32(sA1), b2 = tc::smem_u32(sB2), b1 = tc::smem_u32(sB1);
#pragma unroll
        for (int kk = 0; kk < 8; ++kk)
            tc::mma_bf16(tmem, tc::smem_desc(a2 + kk * 256, 128, 128 * 16), tc::smem_desc(b2 + kk * 256, 128, 128 * 16),
                         tc::idesc_bf16_f32(kRows, H), kk > 0);
#pragma unroll
        for (int kk = 0; kk < 8; ++kk)
            tc::mma_bf16(tmem + H, tc::smem_desc(a1 + kk * 256, 128, 128 * 16),
                         tc::smem_desc(b1 + kk * 256, 128, 128 * 16), tc::idesc_bf16_f32(kRows, kK1), kk > 0);
        tc::mma_commit(bar_mma);
    }
    const bool ok = tc::mbar_wait(bar_mma, 0, kWaitBudget);
    const bool abort = __syncthreads_or(!ok) != 0;
    if (!abort) {
        tc::fence_after_sync();
        const int q = warp & 3, half = warp >> 2;
        const int i = 128 * mh + 32 * q + lane;
        const bool live = i < H;
        const uint32_t t_row = tmem + ((uint32_t)(32 * q) << 16);
        float *g = a.gpart + (size_t)z * a.np;
        float *gW2 = g + (size_t)H * a.din + H + (size_t)(live ? i : 0) * H;
#pragma unroll 1
        for (int cc = half * (H / 2); cc < (half + 1) * (H / 2); cc += 32) {
            uint32_t r[32];
            tc::tmem_ld32(t_row + (uint32_t)cc, r);
#pragma unroll
            for (int e = 0; e < 32; e += 4)
                if (live) *reinterpret_cast<float4 *>(gW2 + cc + e) =
                    make_float4(__uint_as_float(r[e]), __uint_as_float(r[e + 1]), __uint_as_float(r[e + 2]),
                                __uint_as_float(r[e + 3]));
        }
        {
            uint32_t r[32];
            tc::tmem_ld32(t_row + (uint32_t)(H + 32 * half), r);
            float *gW1 = g + (size_t)(live ? i : 0) * a.din;
#pragma unroll
            for (int e = 0; e < 32; ++e)
                if (live && 32 * half + e < a.din) gW1[32 * half + e] = __uint_as_float(r[e]);
        }
    } else if (tid == 0) {
        atomicOr(&s_deverr, SPEO_DEVERR_WAIT_TIMEOUT);
        tc::mbar_wait(bar_mma, 0, kWaitBudget);
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (warp == 0) tc::tmem_dealloc(tmem, kCols);
}

// Column sums of chunk z: gb1 = sum dZ1, gb2 = sum dZ2, gw3 = sum dy H2, gb3 = sum dy (one warp per
// feature, lanes over the 128 rows, fixed-order reduction).
template <int H>
__global__ void k_mlp_colsum(const uint16_t *dz1T, const uint16_t *dz2T, const uint16_t *h2T, const float *dy,
                             long long rp, int din, int np, float *gpart)
{
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int c = blockIdx.x * (blockDim.x >> 5) + warp, z = blockIdx.y;
    if (c > H) return;
    const long long r = (long long)z * 128 + 4 * lane;
    float *g = gpart + (size_t)z * np;
    float d[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) d[e] = dy[r + e];
    if (c == H) {
        float s = (d[0] + d[1]) + (d[2] + d[3]);
        s = warp_sum(s);
        if (lane == 0) g[(size_t)H * din + H + (size_t)H * H + H + H] = s;
        return;
    }
    auto bf = [](uint16_t b) { return __uint_as_float((uint32_t)b << 16); };
    const uint2 u1 = *reinterpret_cast<const uint2 *>(dz1T + (size_t)c * rp + r);
    const uint2 u2 = *reinterpret_cast<const uint2 *>(dz2T + (size_t)c * rp + r);
    const uint2 u3 = *reinterpret_cast<const uint2 *>(h2T + (size_t)c * rp + r);
    float s1 = (bf(lo16(u1.x)) + bf(hi16(u1.x))) + (bf(lo16(u1.y)) + bf(hi16(u1.y)));
    float s2 = (bf(lo16(u2.x)) + bf(hi16(u2.x))) + (bf(lo16(u2.y)) + bf(hi16(u2.y)));
    float s3 = (d[0] * bf(lo16(u3.x)) + d[1] * bf(hi16(u3.x))) + (d[2] * bf(lo16(u3.y)) + d[3] * bf(hi16(u3.y)));
    s1 = warp_sum(s1);
    s2 = warp_sum(s2);
    s3 = warp_sum(s3);
    if (lane == 0) {
        const size_t ob1 = (size_t)H * din, ob2 = ob1 + H + (size_t)H * H, ow3 = ob2 + H;
        g[ob1 + c] = s1;
        g[ob2 + c] = s2;
        g[ow3 + c] = s3;
    }
}

template <int H>
int launch_train(const TrainArgs &ta, const WgradArgs &wa, int splits, cudaStream_t st)
{
    const size_t s1 = train_smem(H), s2 = wg_smem(H);
    cudaError_t e = cudaFuncSetAttribute(k_mlp_train_tc<H>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s1);
    if (e != cudaSuccess) return check_cuda(e, "cudaFuncSetAttribute(k_mlp_train_tc)");
    e = cudaFuncSetAttribute(k_mlp_wgrad_tc<H>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s2);
    if (e != cudaSuccess) return check_cuda(e, "cudaFuncSetAttribute(k_mlp_wgrad_tc)");
    k_mlp_train_tc<H><<<splits, 256, s1, st>>>(ta);
    if (int r = check_launch("k_mlp_train_tc")) return r;
    k_mlp_wgrad_tc<H><<<dim3(splits, (H + kRows - 1) / kRows), 256, s2, st>>>(wa);
    if (int r = check_launch("k_mlp_wgrad_tc")) return r;
    k_mlp_colsum<H><<<dim3((H + 1 + 7) / 8, splits), 256, 0, st>>>(wa.dz1T, wa.dz2T, ta.h2T, ta.dy, ta.rp, ta.din,
                                                                   wa.np, wa.gpart);
    return check_launch("k_mlp_colsum");
}

}  // namespace

bool mlp_bf16_supported(int din, int h) { return din >= 1 && din <= kK1 && (h == 64 || h == 128 || h == 256); }

size_t mlp_bf16_image_bytes(int h) { return w1_bytes(h) + 2 * w2_bytes(h); }

int mlp_forward_bf16(const float *theta, int din, int h, const float *mu, const float *isig, const float *X,
                     long long n, int ldx, float *y, uint8_t *img, cudaStream_t st)
{
    if (!mlp_bf16_supported(din, h)) return fail(SPEO_ERR_UNSUPPORTED, "mlp forward: din %d, hidden %d", din, h);
    if (n <= 0) return SPEO_OK;
    if (((uintptr_t)img & 15) != 0) return fail(SPEO_ERR_INVALID_ARG, "mlp forward: weight image alignment");
    const float *b1 = theta + (size_t)h * din;
    const float *b2 = b1 + h + (size_t)h * h;
    const float *w3 = b2 + h;
    MlpArgs a{img, b1, b2, w3, w3 + h, mu, isig, X, n, ldx, din, (((uintptr_t)X & 15) == 0 && (ldx & 3) == 0) ? 1 : 0, y};
    int e = 0;
    switch (h) {
    case 64: e = pack<64>(theta, din, img, st); return e ? e : launch_fwd<64>(a, st);
    case 128: e = pack<128>(theta, din, img, st); return e ? e : launch_fwd<128>(a, st);
    default: e = pack<256>(theta, din, img, st); return e ? e : launch_fwd<256>(a, st);
    }
}

size_t mlp_img_w2_offset(int h) { return w1_bytes(h); }
size_t mlp_img_w2t_offset(int h) { return w1_bytes(h) + w2_bytes(h); }

int mlp_grad_bf16(const float *theta, int din, int h, const float *mu, const float *isig, const float *X, int n,
                  int ldx, const float *T, const MlpArchive *arch, uint8_t *img, bool pack_weights,
                  const MlpTrainBufs &b, float *gpart, float *loss, cudaStream_t st)
{
    if (!X && !arch) return fail(SPEO_ERR_INVALID_ARG, "mlp gradient: no batch");
    if (!mlp_bf16_supported(din, h)) return fail(SPEO_ERR_UNSUPPORTED, "mlp gradient: din %d, hidden %d", din, h);
    if (n < 1 || (long long)n > b.rp || (b.rp % kRows) != 0)
        return fail(SPEO_ERR_INVALID_ARG, "mlp gradient: %d rows, %lld padded", n, b.rp);
    const int np = h * din + h + h * h + h + h + 1;
    const int gs = (np + 3) & ~3;  // partial-vector stride: 16-byte aligned for the float4 stores
    const float *b1 = theta + (size_t)h * din;
    const float *b2 = b1 + h + (size_t)h * h;
    const float *w3 = b2 + h;
    const int splits = (int)((n + kRows - 1) / kRows);
    const MlpArchive none{nullptr, nullptr, 0, nullptr, 0u, 0u};
    const int vec = X ? ((((uintptr_t)X & 15) == 0 && (ldx & 3) == 0) ? 1 : 0)
                      : ((((uintptr_t)arch->AX & 15) == 0 && (arch->lda & 3) == 0) ? 1 : 0);
    TrainArgs ta{img, b1, b2, w3, w3 + h, mu, isig, X, T, X ? none : *arch, n, ldx, din, vec, b.rp, 2.f / (float)n,
                 b.xnT, b.h1T, b.h2T, b.dz2T, b.dz1T, b.dy, loss};
    WgradArgs wa{b.xnT, b.h1T, b.dz2T, b.dz1T, b.rp, din, gs, gpart};
    int e = 0;
    switch (h) {
    case 64: e = pack_weights ? pack<64>(theta, din, img, st, 1) : 0; return e ? e : launch_train<64>(ta, wa, splits, st);
    case 128: e = pack_weights ? pack<128>(theta, din, img, st, 1) : 0; return e ? e : launch_train<128>(ta, wa, splits, st);
    default: e = pack_weights ? pack<256>(theta, din, img, st, 1) : 0; return e ? e : launch_train<256>(ta, wa, splits, st);
    }
}

}  // namespace speo
