// mlp_tc.cu -- the surrogate MLP's screening forward pass on the tcgen05 tensor cores.
//
// No counterpart in the reference. y = w3 . relu(W2 relu(W1 x' + b1) + b2) + b3 with
// x' = (x - mu) * isig, BF16 operands and FP32 accumulation:
//   * W1 (H x din, K padded to 64) and W2 (H x H) are packed once per call into BF16 images laid
//     out exactly as the K-major no-swizzle shared-memory operands, so one bulk copy per image
//     brings them into shared memory, where they stay for every tile the block processes;
//   * per 128-row tile: the block standardises and converts the rows into the A operand, one
//     thread issues layer 1 (M = 128, N = H, K = 64) into tensor memory, all 8 warps read the
//     accumulators back (bias, ReLU, BF16) into the layer-2 A operand, layer 2 (K = H) reuses
//     the same tensor-memory columns, and the epilogue folds bias, ReLU and the H -> 1 head into
//     a per-row dot product.
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

__host__ __device__ constexpr size_t w1_bytes(int H) { return (size_t)H * kK1 * 2; }
__host__ __device__ constexpr size_t w2_bytes(int H) { return (size_t)H * H * 2; }
__host__ __device__ constexpr size_t a_bytes(int H) { return (size_t)kRows * (H > kK1 ? H : kK1) * 2; }
__host__ __device__ constexpr size_t smem_total(int H)
{
    return w1_bytes(H) + w2_bytes(H) + a_bytes(H) + 2 * kRows * sizeof(float) + 64;
}

__device__ __forceinline__ uint32_t bf2(float a, float b)
{
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t *>(&h);
}

// Weight images: chunk (n, kc) = 8 consecutive K elements of row n, as one 16-byte core-matrix row.
template <int H>
__global__ void k_pack_mlp(const float *__restrict__ theta, int din, uint8_t *__restrict__ img)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    constexpr int c1 = H * (kK1 / 8), c2 = H * (H / 8);
    if (t >= c1 + c2) return;
    const float *W1 = theta;
    const float *W2 = theta + (size_t)H * din + H;
    float v[8];
    uint32_t off;
    if (t < c1) {
        const int n = t / (kK1 / 8), k0 = (t % (kK1 / 8)) * 8;
#pragma unroll
        for (int j = 0; j < 8; ++j) v[j] = k0 + j < din ? W1[(size_t)n * din + k0 + j] : 0.f;
        off = tc::kmajor_offset(n, k0, kK1);
    } else {
        const int u = t - c1, n = u / (H / 8), k0 = (u % (H / 8)) * 8;
#pragma unroll
        for (int j = 0; j < 8; ++j) v[j] = W2[(size_t)n * H + k0 + j];
        off = (uint32_t)w1_bytes(H) + tc::kmajor_offset(n, k0, H);
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
__global__ void __launch_bounds__(256, 1) k_mlp_fwd_tc(MlpArgs a)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t *sw1 = smem, *sw2 = smem + w1_bytes(H), *sa = sw2 + w2_bytes(H);
    float *red = reinterpret_cast<float *>(sa + a_bytes(H));
    uint64_t *bars = reinterpret_cast<uint64_t *>(red + 2 * kRows);
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
    const int q = warp & 3, half = warp >> 2;       // TMEM lane quadrant, column half
    const int row_l = 32 * q + lane;                // tile row this thread reads back
    const uint32_t t_row = tmem + ((uint32_t)(32 * q) << 16);
    const long long ntiles = (a.n + kRows - 1) / kRows;
    uint32_t phase = 0;
    int mma_pending = 0;  // a commit whose wait gave up

    for (long long tile = blockIdx.x; tile < ntiles && !abort; tile += gridDim.x) {
        const long long r0 = tile * kRows;
        // ---- A1 = bf16((x - mu) * isig), zero past din and past n ----------------------------
#pragma unroll
        for (int j = 0; j < kRows * (kK1 / 8) / 256; ++j) {
            const int item = tid + 256 * j;
            const int r = item / (kK1 / 8), k0 = (item % (kK1 / 8)) * 8;
            const long long gr = r0 + r;
            float v[8];
#pragma unroll
            for (int e = 0; e < 8; ++e) v[e] = 0.f;
            if (gr < a.n) {
                const float *xr = a.X + gr * a.ldx;
                if (a.vec && k0 + 8 <= a.din) {
                    const float4 p = *reinterpret_cast<const float4 *>(xr + k0);
                    const float4 s = *reinterpret_cast<const float4 *>(xr + k0 + 4);
                    v[0] = p.x; v[1] = p.y; v[2] = p.z; v[3] = p.w; v[4] = s.x; v[5] = s.y; v[6] = s.z; v[7] = s.w;
                } else {
#pragma unroll
                    for (int e = 0; e < 8; ++e) v[e] = k0 + e < a.din ? xr[k0 + e] : 0.f;
                }
#pragma unroll
                for (int e = 0; e < 8; ++e)
                    v[e] = k0 + e < a.din ? __fmul_rn(__fsub_rn(v[e], a.mu[k0 + e]), a.isig[k0 + e]) : 0.f;
            }
            *reinterpret_cast<uint4 *>(sa + tc::kmajor_offset(r, k0, kK1)) =
                make_uint4(bf2(v[0], v[1]), bf2(v[2], v[3]), bf2(v[4], v[5]), bf2(v[6], v[7]));
        }
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
        for (int c0 = half * (H / 2); c0 < (half + 1) * (H / 2); c0 += 32) {
            uint32_t r[32];
            tc::tmem_ld32_nowait(t_row + (uint32_t)c0, r);
            tc::tmem_wait_ld();
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
        for (int c0 = half * (H / 2); c0 < (half + 1) * (H / 2); c0 += 32) {
            uint32_t r[32];
            tc::tmem_ld32_nowait(t_row + (uint32_t)c0, r);
            tc::tmem_wait_ld();
#pragma unroll
            for (int e = 0; e < 32; ++e)
                s = __fmaf_rn(fmaxf(__fadd_rn(__uint_as_float(r[e]), a.b2[c0 + e]), 0.f), a.w3[c0 + e], s);
        }
        red[half * kRows + row_l] = s;
        tc::fence_before_sync();
        __syncthreads();
        if (tid < kRows && r0 + tid < a.n) a.y[r0 + tid] = __fadd_rn(__fadd_rn(red[tid], red[kRows + tid]), a.b3[0]);
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
    k_mlp_fwd_tc<H><<<grid, 256, smem, st>>>(a);
    return check_launch("k_mlp_fwd_tc");
}

template <int H>
int pack(const float *theta, int din, uint8_t *img, cudaStream_t st)
{
    const int total = H * (kK1 / 8) + H * (H / 8);
    k_pack_mlp<H><<<(total + 255) / 256, 256, 0, st>>>(theta, din, img);
    return check_launch("k_pack_mlp");
}

}  // namespace

bool mlp_bf16_supported(int din, int h) { return din >= 1 && din <= kK1 && (h == 64 || h == 128 || h == 256); }

size_t mlp_bf16_image_bytes(int h) { return w1_bytes(h) + w2_bytes(h); }

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

}  // namespace speo
