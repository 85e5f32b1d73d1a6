// surrogate.cu -- the online MLP surrogate that pre-screens DE trials.
//
// No counterpart in the reference (it evaluates every trial exactly). Per generation:
//   1. every target gets k trial vectors (DE/<strategy>/bin, Philox streams tagged with the trial
//      number, so they are independent of the plain DE draws);
//   2. the MLP (din -> h -> h -> 1, ReLU) predicts a transformed fitness for all k trials;
//   3. the trial with the lowest prediction is evaluated exactly and goes through the usual
//      strict-`<` greedy selection;
//   4. the exact evaluations are appended to a ring-buffer archive;
//   5. Adam trains the MLP on batches sampled from the archive.
// Exact evaluation stays the arbiter: the surrogate only chooses which trial is evaluated.
#include <cmath>
#include <cstring>
#include <new>

#include "eval_simt.cuh"
#include "host.h"
#include "tcgen05.cuh"

SPEO_DEFINE_DEVERR(speo_deverr_surrogate)

namespace speo {
namespace {

constexpr float kTargetFloor = 1e-8f;  // target = log(f + floor)
constexpr int kSplitRows = 128;        // batch rows per split-K chunk of the weight gradients

// ---- generic strided SIMT GEMM ---------------------------------------------------------------
// C[m][n] = epi(alpha * sum_k A(m,k) B(k,n) + bias[n]),  A(m,k) = A[m*sam + k*sak],
// B(k,n) = B[k*sbk + n*sbn]. epi: 0 = identity, 1 = ReLU (Z receives the pre-activation when
// non-null), 2 = multiply by 1[Z[m][n] > 0] (ReLU backward). 64x64 tiles, 4x4 per thread.
// Split-K: blockIdx.z sums k in [z*kc, (z+1)*kc) into C + z*cz (partial sums, reduced later in a
// fixed order, so the result does not depend on scheduling).
constexpr int BM = 64, BN = 64, BK = 16;

template <int EPI>
__global__ void __launch_bounds__(256) k_gemm(const float *__restrict__ A, long long sam, long long sak,
                                              const float *__restrict__ B, long long sbk, long long sbn,
                                              const float *__restrict__ bias, float *__restrict__ C, int ldc,
                                              float *__restrict__ Z, int M, int N, int K, float alpha, int kc,
                                              long long cz)
{
    __shared__ float As[BK][BM + 4];
    __shared__ float Bs[BK][BN + 4];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
    const int kbeg = blockIdx.z * kc;
    const int kend = min(K, kbeg + kc);
    C += blockIdx.z * cz;
    float acc[4][4] = {};
    for (int k0 = kbeg; k0 < kend; k0 += BK) {
        for (int i = threadIdx.x; i < BK * BM; i += 256) {
            int kk, mm;
            if (sak == 1) { kk = i % BK; mm = i / BK; } else { mm = i % BM; kk = i / BM; }
            const int m = m0 + mm, k = k0 + kk;
            As[kk][mm] = (m < M && k < kend) ? A[m * sam + k * sak] : 0.f;
        }
        for (int i = threadIdx.x; i < BK * BN; i += 256) {
            int kk, nn;
            if (sbn == 1) { nn = i % BN; kk = i / BN; } else { kk = i % BK; nn = i / BK; }
            const int n = n0 + nn, k = k0 + kk;
            Bs[kk][nn] = (n < N && k < kend) ? B[k * sbk + n * sbn] : 0.f;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < BK; ++kk) {
            float a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = As[kk][ty * 4 + i];
#pragma unroll
            for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx * 4 + j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int m = m0 + ty * 4 + i;
        if (m >= M) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int n = n0 + tx * 4 + j;
            if (n >= N) continue;
            float v = alpha * acc[i][j] + (bias ? bias[n] : 0.f);
            const size_t o = (size_t)m * ldc + n;
            if (EPI == 1) {
                if (Z) Z[o] = v;
                v = fmaxf(v, 0.f);
            } else if (EPI == 2) {
                v = Z[o] > 0.f ? v : 0.f;
            }
            C[o] = v;
        }
    }
}

template <int EPI>
int gemm(cudaStream_t st, const float *A, long long sam, long long sak, const float *B, long long sbk, long long sbn,
         const float *bias, float *C, int ldc, float *Z, int M, int N, int K, float alpha, int splits = 1,
         long long cz = 0)
{
    const int kc = (((K + splits - 1) / splits) + BK - 1) / BK * BK;
    const dim3 grid((N + BN - 1) / BN, (M + BM - 1) / BM, splits);
    k_gemm<EPI><<<grid, 256, 0, st>>>(A, sam, sak, B, sbk, sbn, bias, C, ldc, Z, M, N, K, alpha, kc, cz);
    return check_launch("k_gemm");
}

// out[i] = sum_z P[z * stride + i], z ascending.
__global__ void k_reduce_splits(const float *P, int splits, int n, long long stride, float *out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float s = 0.f;
    for (int z = 0; z < splits; ++z) s += P[(size_t)z * stride + i];
    out[i] = s;
}

// y[i] = b3 + sum_j H2[i][j] w3[j]: one warp per row.
__global__ void k_head(const float *H2, int h, const float *w3, const float *b3, float *y, int n)
{
    const int row = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (row >= n) return;
    float s = 0.f;
    for (int j = lane; j < h; j += 32) s = fmaf(H2[(size_t)row * h + j], w3[j], s);
    s = warp_sum(s);
    if (lane == 0) y[row] = s + b3[0];
}

// dy[i] = 2 (y[i] - t[i]) / n; loss_sum += (y - t)^2.
__global__ void k_mse(const float *y, const float *t, int n, float *dy, float *loss_sum)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    float e2 = 0.f;
    if (i < n) {
        const float e = y[i] - t[i];
        dy[i] = 2.f * e / (float)n;
        e2 = e * e;
    }
    e2 = warp_sum(e2);
    if ((threadIdx.x & 31) == 0 && loss_sum) atomicAdd(loss_sum, e2);
}

// dZ2[i][j] = 1[Z2 > 0] dy[i] w3[j]
__global__ void k_head_back(const float *dy, const float *w3, const float *Z2, float *dZ2, int n, int h)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)n * h) return;
    const int i = (int)(t / h), j = (int)(t - (long long)i * h);
    dZ2[t] = Z2[t] > 0.f ? dy[i] * w3[j] : 0.f;
}

__global__ void k_archive_advance(SurrDev *st, long long n, long long cap)
{
    st->head = (st->head + n) % cap;
    st->count = st->count + n < cap ? st->count + n : cap;
}

// Adam (Kingma & Ba, 2015) at step t = st->step + 1 with the bias corrections st->c1, st->c2.
// The gradient is the fixed-order sum of `splits` partial vectors (stride pstride). With `img`,
// the BF16 weight images of the tensor-core passes are refreshed from the new parameters. The last
// block to finish advances the step and the next step's bias corrections, so a captured sequence
// of steps replays correctly.
__global__ void k_adam(float *theta, float *m, float *v, const float *P, int splits, long long pstride, int n,
                       float lr, float b1, float b2, float eps, SurrDev *st, uint8_t *img, int din, int h)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const float c1 = st->c1, c2 = st->c2;
    if (i < n) {
        float gi = 0.f;
        for (int z = 0; z < splits; ++z) gi += P[(size_t)z * pstride + i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float th = theta[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
        theta[i] = th;
        if (img) {
            const long long o2 = (long long)h * din + h;
            const __nv_bfloat16 hb = __float2bfloat16_rn(th);
            if (i < h * din) {
                *reinterpret_cast<__nv_bfloat16 *>(img + tc::kmajor_offset(i / din, i % din, 64)) = hb;
            } else if (i >= o2 && i < o2 + (long long)h * h) {
                const int a = (int)((i - o2) / h), b = (int)((i - o2) % h);
                *reinterpret_cast<__nv_bfloat16 *>(img + (size_t)h * 64 * 2 + tc::kmajor_offset(a, b, h)) = hb;
                *reinterpret_cast<__nv_bfloat16 *>(img + (size_t)h * 64 * 2 + (size_t)h * h * 2 +
                                                   tc::kmajor_offset(b, a, h)) = hb;
            }
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(&st->done, 1u) == gridDim.x - 1) {
            const uint32_t s = st->step + 1u;
            st->step = s;
            st->c1 = (float)(1.0 - pow((double)b1, (double)s + 1.0));
            st->c2 = (float)(1.0 - pow((double)b2, (double)s + 1.0));
            st->done = 0u;
        }
    }
}


// Archive append: rows [0, n) of X (stride ldx, din used) and their exact fitness at slots
// (head + i) mod cap, target = log(f + floor).
__global__ void k_archive_append(const float *X, int ldx, const float *f, int n, int din, float *AX, int lda, float *AT,
                                 const SurrDev *st, long long cap)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)n * lda) return;
    const int i = (int)(t / lda), d = (int)(t - (long long)i * lda);
    const long long slot = (st->head + i) % cap;
    AX[slot * lda + d] = d < din ? X[(size_t)i * ldx + d] : 0.f;
    if (d == 0) AT[slot] = logf(fmaxf(f[i], 0.f) + kTargetFloor);
}

// Batch sampling: index i at Adam step `step` is philox({i/4, step, 0, SAMPLE})[i%4] mod count.
__global__ void k_archive_sample(const float *AX, int lda, const float *AT, const SurrDev *st, int batch, uint2 key,
                                 float *X, float *T)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)batch * lda) return;
    const int i = (int)(t / lda), d = (int)(t - (long long)i * lda);
    const uint4 w = philox(make_uint4((uint32_t)(i >> 2), st->step, 0u, kTagSample), key);
    const long long slot = (long long)(pick(w, (uint32_t)(i & 3)) % (uint32_t)st->count);
    X[t] = AX[slot * lda + d];
    if (d == 0) T[i] = AT[slot];
}

// ---- k trials per target ----------------------------------------------------------------------
// Trial t of the row `row` uses Philox tags TAG_IDX | (t+1) << 8 and TAG_CR | (t+1) << 8.
// Each warp takes up to 32 (row, trial) pairs of a work item (fewer when the item has few pairs,
// so that all warps of the block work), its lanes drawing the pairs' donors in parallel; the
// batch's (pair, 4-element chunk) tasks are then dealt to all 32 lanes. Output:
// T[(row * k + t) * ld + e].
__device__ __forceinline__ int ndon(int st)
{
    switch (st) {
    case 0: case 2: case 6: return 2;
    case 3: case 4: case 8: return 3;
    case 1: case 7: return 4;
    default: return 5;
    }
}

__global__ void __launch_bounds__(256) k_make_trials(const speo_segment *segs, const speo_work_item *items, int n_items,
                                                     int k, const float *pop, const float *fit, float *T,
                                                     const uint32_t *gen_ctr)
{
    const uint32_t gen = *(volatile const uint32_t *)gen_ctr;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int t_item = blockIdx.x; t_item < n_items; t_item += gridDim.x) {
        const speo_work_item it = items[t_item];
        const speo_segment &s = segs[it.segment];
        const int D = s.dim, P = s.pop_size, ld = s.ld, nch = (D + 3) >> 2;
        if (it.count < 1 || it.first + it.count > P || P < 2 || (ld & 3) || ld < D) {
            if (threadIdx.x == 0) atomicOr(&s_deverr, SPEO_DEVERR_BAD_SEGMENT);
            continue;
        }
        const uint2 key = seed_key(s.seed);
        const int st = s.strategy, nd = ndon(st);
        // the segment's fields in registers: the trial stores below may alias `segs` for the
        // compiler, which would otherwise load them again after every store
        const long long row0 = s.row0;
        const float sF = s.F, sCR = s.CR, slb = s.lb, sub = s.ub;
        long long best_row = -1;
        if (strategy_uses_best(st)) {  // argmin of the segment's fitness (every lane, small P)
            float bf = __int_as_float(0x7f800000);
            for (int i = 0; i < P; ++i) {
                const float f = rank_key(fit[row0 + i]);
                if (f < bf) { bf = f; best_row = row0 + i; }
            }
            if (best_row < 0) best_row = row0;
        }
        const int pairs = it.count * k;
        // pairs per warp: up to 32, fewer when the item has few pairs, so that every warp works
        const int nwarps = (int)(blockDim.x >> 5);
        int ppw = (pairs + nwarps - 1) / nwarps;
        ppw = ppw > 32 ? 32 : ppw;
        for (int pb = warp * ppw; pb < pairs; pb += nwarps * ppw) {
            // lane < ppw draws for pair pb + lane
            int d0 = 0, d1 = 0, d2 = 0, d3 = 0, d4 = 0, jr = 0;
            {
                const int p = pb + lane;
                if (lane < ppw && p < pairs) {
                    const int lr = p / k, tt = p - lr * k;
                    const long long row = row0 + it.first + lr;
                    IdxStream is(key, (uint32_t)row, gen, kTagIdx | ((uint32_t)(tt + 1) << 8));
                    int r[5];
                    if (!draw_donors(is, P, r)) atomicOr(&s_deverr, SPEO_DEVERR_REDRAW_LIMIT);
                    d0 = r[0]; d1 = r[1]; d2 = r[2]; d3 = r[3]; d4 = r[4];
                    jr = is.index(D);
                }
            }
            bool ok_bound = true;
            // the batch's (pair, 4-element chunk) tasks dealt to all 32 lanes; a task reads its
            // pair's draws from the drawing lane
            const int np = pairs - pb < ppw ? pairs - pb : ppw, tasks = np * nch;
            for (int t0 = 0; t0 < tasks; t0 += 32) {
                const int t = t0 + lane;
                const int src = t < tasks ? t / nch : 0, c = t - src * nch;
                const int rd[5] = {__shfl_sync(0xffffffffu, d0, src), __shfl_sync(0xffffffffu, d1, src),
                                   __shfl_sync(0xffffffffu, d2, src), __shfl_sync(0xffffffffu, d3, src),
                                   __shfl_sync(0xffffffffu, d4, src)};
                const int rjr = __shfl_sync(0xffffffffu, jr, src);
                if (t >= tasks) continue;
                const int p = pb + src;
                const int lr = p / k, tt = p - lr * k;
                const long long row = row0 + it.first + lr;
                const float *xi = pop + row * ld;
                const float *xb = pop + (best_row >= 0 ? best_row : row) * ld;
                float *out = T + (row * k + tt) * (long long)ld;
                {
                    const int e0 = 4 * c;
                    const float4 ti = *reinterpret_cast<const float4 *>(xi + e0);
                    const float4 tb = best_row >= 0 ? *reinterpret_cast<const float4 *>(xb + e0) : ti;
                    float4 tr[5];
#pragma unroll
                    for (int q = 0; q < 5; ++q)
                        tr[q] = q < nd ? *reinterpret_cast<const float4 *>(pop + (row0 + rd[q]) * ld + e0) : ti;
                    const uint4 w = philox(make_uint4((uint32_t)c, (uint32_t)row, gen,
                                                      kTagCr | ((uint32_t)(tt + 1) << 8)), key);
                    float o[4] = {0.f, 0.f, 0.f, 0.f};
                    const float tiv[4] = {ti.x, ti.y, ti.z, ti.w}, tbv[4] = {tb.x, tb.y, tb.z, tb.w};
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        const int e = e0 + q;
                        if (e >= D) continue;
                        const float u = u01(pick(w, (uint32_t)q));
                        float x;
                        if (e == rjr || u < sCR) {
                            float xr[5];
#pragma unroll
                            for (int z = 0; z < 5; ++z)
                                xr[z] = q == 0 ? tr[z].x : q == 1 ? tr[z].y : q == 2 ? tr[z].z : tr[z].w;
                            x = mutant<float>(st, sF, tiv[q], tbv[q], xr);
                        } else {
                            x = tiv[q];
                        }
                        o[q] = check_bound<float>(x, slb, sub, ok_bound);
                    }
                    *reinterpret_cast<float4 *>(out + e0) = make_float4(o[0], o[1], o[2], o[3]);
                }
            }
            if (!ok_bound) atomicOr(&s_deverr, SPEO_DEVERR_BOUND_LIMIT);
        }
    }
}

// Per row: the trial with the lowest prediction (NaN as +inf, ties lowest trial) -> sel row.
// An `explore` fraction of rows instead takes a uniformly drawn trial: those exact evaluations are
// an unbiased sample of the trial distribution, which keeps the archive from holding only the
// points the model under-predicts. Draw for row r at generation g:
// u = u01(philox({0, r, g, PICK}, key)[0]); explore if u < explore, trial = word 1 mod k.
constexpr uint32_t kTagPick = 5u;

__global__ void k_pick(const float *T, const float *pred, int k, float *sel, long long rows, int ld, int max_dim,
                       float explore, uint2 key, const uint32_t *gen_ctr)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int nch = (max_dim + 3) >> 2;
    if (t >= rows * nch) return;
    const long long row = t / nch;
    const int c = (int)(t - row * nch);
    int bt = 0;
    const uint4 w = philox(make_uint4(0u, (uint32_t)row, *gen_ctr, kTagPick), key);
    if (u01(w.x) < explore) {
        bt = (int)(w.y % (uint32_t)k);
    } else {
        float bp = rank_key(pred[row * k]);
        for (int q = 1; q < k; ++q) {
            const float v = rank_key(pred[row * k + q]);
            if (v < bp) { bp = v; bt = q; }
        }
    }
    if (4 * c < ld)
        *reinterpret_cast<float4 *>(sel + row * ld + 4 * c) =
            *reinterpret_cast<const float4 *>(T + (row * k + bt) * (long long)ld + 4 * c);
}

// Greedy selection over a flat segment-layout buffer, double-buffered; also writes the chosen
// trial's exact fitness into `tf_out` order (caller's trial_fit).
__global__ void k_select_flat(const float *pop_in, const float *fit_in, const float *sel, const float *fsel,
                              float *pop_out, float *fit_out, long long rows, int ld, int nch)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= rows * nch) return;
    const long long row = t / nch;
    const int c = (int)(t - row * nch);
    const bool win = fsel[row] < fit_in[row];
    const float *src = win ? sel : pop_in;
    *reinterpret_cast<float4 *>(pop_out + row * ld + 4 * c) = *reinterpret_cast<const float4 *>(src + row * ld + 4 * c);
    if (c == 0) fit_out[row] = win ? fsel[row] : fit_in[row];
}

__global__ void k_advance_gen(uint32_t *gen, uint32_t n) { gen[0] += n; }

// Per input dimension d: mean and 1/std over `rows` rows of pop (stride ld), FP64 sums; one block
// per dimension. The MLP then sees the population's region at unit scale.
__global__ void k_input_stats(const float *pop, long long rows, int ld, int din, float *mu, float *isig)
{
    __shared__ double s1[256], s2[256];
    const int d = blockIdx.x;
    double a = 0.0, b = 0.0;
    for (long long i = threadIdx.x; i < rows; i += blockDim.x) {
        const double x = pop[i * ld + d];
        a += x;
        b += x * x;
    }
    s1[threadIdx.x] = a;
    s2[threadIdx.x] = b;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) { s1[threadIdx.x] += s1[threadIdx.x + o]; s2[threadIdx.x] += s2[threadIdx.x + o]; }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const double m = s1[0] / (double)rows;
        const double var = fmax(s2[0] / (double)rows - m * m, 0.0);
        mu[d] = (float)m;
        isig[d] = (float)(1.0 / (sqrt(var) + 1e-6));
        (void)din;
    }
}

// Y[i][d] = (X[i][d] - mu[d]) * isig[d] for d < din (zero in the padding up to ldy).
__global__ void k_normalize(const float *X, int ldx, long long n, int din, const float *mu, const float *isig, float *Y,
                            int ldy)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n * ldy) return;
    const long long i = t / ldy;
    const int d = (int)(t - i * ldy);
    Y[t] = d < din ? (X[i * ldx + d] - mu[d]) * isig[d] : 0.f;
}

}  // namespace

// ---- host object --------------------------------------------------------------------------------
struct Surrogate {
    int din, h, lda, batch, np;
    long long cap, count = 0, head = 0;
    float lr, in_scale, beta1 = 0.9f, beta2 = 0.999f, eps = 1e-8f;
    uint64_t seed;
    int step = 0;                             // host mirrors of the device state (exact: advanced in
                                              // the same order); used for sizes and first-call checks
    SurrDev *dst = nullptr;                   // device state: archive head / count, Adam step
    float *theta = nullptr, *m = nullptr, *v = nullptr, *grad = nullptr;
    float *AX = nullptr, *AT = nullptr;       // archive
    float *Xb = nullptr, *Tb = nullptr;       // training batch
    float *Z1 = nullptr, *H1 = nullptr, *Z2 = nullptr, *H2 = nullptr, *yb = nullptr, *dy = nullptr;
    float *dZ2 = nullptr, *dZ1 = nullptr, *loss = nullptr, *one = nullptr;
    float *gpart = nullptr;                   // split-K partial gradients, ceil(batch / 128) x np
    float *mu = nullptr, *isig = nullptr;     // input standardisation (default: 0 and in_scale)
    float *Xbn = nullptr;                     // standardised training batch
    long long nrm_rows = 0;
    float *Xn = nullptr;                      // standardised screening inputs
    uint8_t *wimg = nullptr;                  // packed BF16 weight images of the tensor-core passes
    MlpTrainBufs tb{};                        // tensor-core training scratch
    int mode = 0;                             // SPEO_SURROGATE_BF16_SCREEN | SPEO_SURROGATE_BF16_TRAIN
    // screening scratch (grown on demand)
    long long scr_rows = 0;
    float *sH1 = nullptr, *sH2 = nullptr;
    long long trial_cap = 0;
    float *T = nullptr, *pred = nullptr, *sel = nullptr, *fsel = nullptr;

    long long gstride() const { return (np + 3) & ~3; }  // partial-gradient vector stride (16-byte rows)
    float *W1() { return theta; }
    float *b1() { return theta + (size_t)h * din; }
    float *W2() { return b1() + h; }
    float *b2() { return W2() + (size_t)h * h; }
    float *w3() { return b2() + h; }
    float *b3() { return w3() + h; }
};

namespace {

// Inputs standardised into `Xn` (n x lda) first: x' = (x - mu) * isig.
int standardise(Surrogate *S, cudaStream_t st, const float *X, int n, int ldx, float *Xn)
{
    const long long total = (long long)n * S->lda;
    k_normalize<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(X, ldx, n, S->din, S->mu, S->isig, Xn, S->lda);
    return check_launch("k_normalize");
}

// Forward on standardised inputs Xn (stride lda).
int mlp_forward(Surrogate *S, cudaStream_t st, const float *X, int n, int ldx, float *y, float *Z1, float *H1, float *Z2,
                float *H2)
{
    const int h = S->h;
    if (int e = gemm<1>(st, X, ldx, 1, S->W1(), 1, S->din, S->b1(), H1, h, Z1, n, h, S->din, 1.f)) return e;
    if (int e = gemm<1>(st, H1, h, 1, S->W2(), 1, h, S->b2(), H2, h, Z2, n, h, h, 1.f)) return e;
    k_head<<<(n + 7) / 8, 256, 0, st>>>(H2, h, S->w3(), S->b3(), y, n);
    return check_launch("k_head");
}

// Gradient of the mean squared error over the batch (X raw, T) into S->grad; loss into S->loss.
int mlp_grad(Surrogate *S, cudaStream_t st, const float *Xraw, int n, int ldxraw, const float *T)
{
    const int h = S->h, din = S->din;
    if (int e = standardise(S, st, Xraw, n, ldxraw, S->Xbn)) return e;
    const float *X = S->Xbn;
    const int ldx = S->lda;
    if (int e = mlp_forward(S, st, X, n, ldx, S->yb, S->Z1, S->H1, S->Z2, S->H2)) return e;
    if (int e = check_cuda(cudaMemsetAsync(S->loss, 0, sizeof(float), st), "memset loss")) return e;
    k_mse<<<(n + 255) / 256, 256, 0, st>>>(S->yb, T, n, S->dy, S->loss);
    // Weight and bias gradients are sums over the batch rows: split-K over chunks of kSplitRows
    // rows into the partial buffer (one full gradient vector per chunk), then one fixed-order sum.
    const int splits = (n + kSplitRows - 1) / kSplitRows;
    const long long np = S->gstride();
    float *g = S->gpart;
    float *gW1 = g, *gb1 = gW1 + (size_t)h * din, *gW2 = gb1 + h, *gb2 = gW2 + (size_t)h * h, *gw3 = gb2 + h,
          *gb3 = gw3 + h;
    // head: gw3 = dy^T H2, gb3 = sum dy, dZ2 = 1[Z2>0] dy w3
    if (int e = gemm<0>(st, S->dy, 0, 1, S->H2, h, 1, nullptr, gw3, h, nullptr, 1, h, n, 1.f, splits, np)) return e;
    if (int e = gemm<0>(st, S->one, 0, 0, S->dy, 1, 0, nullptr, gb3, 1, nullptr, 1, 1, n, 1.f, splits, np)) return e;
    k_head_back<<<(unsigned)(((long long)n * h + 255) / 256), 256, 0, st>>>(S->dy, S->w3(), S->Z2, S->dZ2, n, h);
    // layer 2: gW2 = dZ2^T H1, gb2 = 1^T dZ2, dZ1 = (dZ2 W2) * 1[Z1 > 0]
    if (int e = gemm<0>(st, S->dZ2, 1, h, S->H1, h, 1, nullptr, gW2, h, nullptr, h, h, n, 1.f, splits, np)) return e;
    if (int e = gemm<0>(st, S->one, 0, 0, S->dZ2, h, 1, nullptr, gb2, h, nullptr, 1, h, n, 1.f, splits, np)) return e;
    if (int e = gemm<2>(st, S->dZ2, h, 1, S->W2(), h, 1, nullptr, S->dZ1, h, S->Z1, n, h, h, 1.f)) return e;
    // layer 1: gW1 = dZ1^T X', gb1 = 1^T dZ1 (X' standardised)
    if (int e = gemm<0>(st, S->dZ1, 1, h, X, ldx, 1, nullptr, gW1, din, nullptr, h, din, n, 1.f, splits, np)) return e;
    if (int e = gemm<0>(st, S->one, 0, 0, S->dZ1, h, 1, nullptr, gb1, h, nullptr, 1, h, n, 1.f, splits, np)) return e;
    k_reduce_splits<<<(unsigned)((S->np + 255) / 256), 256, 0, st>>>(S->gpart, splits, S->np, np, S->grad);
    return check_launch("k_reduce_splits");
}

// One batch's gradient on the tensor cores: partial vectors per 128-row chunk into S->gpart, summed
// into S->grad when `reduce` (the training loop lets the Adam kernel sum them instead). The batch is
// X/T, or drawn from the archive inside the kernel when X is null.
int grad_bf16(Surrogate *S, cudaStream_t st, const float *X, int n, int ldx, const float *T, bool pack_weights,
              bool reduce)
{
    if (int e = check_cuda(cudaMemsetAsync(S->loss, 0, sizeof(float), st), "memset loss")) return e;
    const MlpArchive arch{S->AX, S->AT, S->lda, S->dst, (uint32_t)S->seed, (uint32_t)(S->seed >> 32)};
    if (int e = mlp_grad_bf16(S->theta, S->din, S->h, S->mu, S->isig, X, n, ldx, T, X ? nullptr : &arch, S->wimg,
                              pack_weights, S->tb, S->gpart, S->loss, st))
        return e;
    if (!reduce) return SPEO_OK;
    const int splits = (n + kSplitRows - 1) / kSplitRows;
    k_reduce_splits<<<(unsigned)((S->np + 255) / 256), 256, 0, st>>>(S->gpart, splits, S->np, S->gstride(), S->grad);
    return check_launch("k_reduce_splits");
}

// One Adam step from `splits` partial gradient vectors (stride pstride); refreshes the BF16 weight
// images when `img` is set.
int adam(Surrogate *S, cudaStream_t st, const float *P, int splits, long long pstride, uint8_t *img)
{
    k_adam<<<(S->np + 255) / 256, 256, 0, st>>>(S->theta, S->m, S->v, P, splits, pstride, S->np, S->lr, S->beta1,
                                                S->beta2, S->eps, S->dst, img, S->din, S->h);
    S->step += 1;
    return check_launch("k_adam");
}

template <typename T>
int dalloc(T **p, size_t n)
{
    return check_cuda(cudaMalloc(reinterpret_cast<void **>(p), sizeof(T) * (n ? n : 1)), "cudaMalloc");
}

}  // namespace
}  // namespace speo

using namespace speo;

extern "C" int speo_surrogate_create(speo_surrogate **out, int din, int hidden, long long archive_cap, int batch,
                                     float lr, float in_scale, uint64_t seed)
{
    if (!out || din < 1 || din > SPEO_MAX_DIM || hidden < 1 || hidden > 1024 || archive_cap < 1 || batch < 1)
        return fail(SPEO_ERR_INVALID_ARG, "speo_surrogate_create: bad arguments");
    Surrogate *S = new (std::nothrow) Surrogate();
    if (!S) return fail(SPEO_ERR_INVALID_ARG, "speo_surrogate_create: out of host memory");
    S->din = din; S->h = hidden; S->lda = (din + 3) & ~3; S->batch = batch; S->cap = archive_cap; S->lr = lr;
    S->in_scale = in_scale; S->seed = seed;
    S->np = hidden * din + hidden + hidden * hidden + hidden + hidden + 1;
    int e = 0;
    e = e ? e : dalloc(&S->theta, S->np);
    e = e ? e : dalloc(&S->m, S->np);
    e = e ? e : dalloc(&S->v, S->np);
    e = e ? e : dalloc(&S->grad, S->np);
    e = e ? e : dalloc(&S->dst, 1);
    if (!e) {
        SurrDev d0{};
        d0.c1 = (float)(1.0 - (double)S->beta1);
        d0.c2 = (float)(1.0 - (double)S->beta2);
        e = check_cuda(cudaMemcpy(S->dst, &d0, sizeof d0, cudaMemcpyHostToDevice), "surrogate state");
    }
    e = e ? e : dalloc(&S->gpart, (size_t)S->gstride() * ((batch + kSplitRows - 1) / kSplitRows));
    e = e ? e : dalloc(&S->AX, (size_t)archive_cap * S->lda);
    e = e ? e : dalloc(&S->AT, (size_t)archive_cap);
    e = e ? e : dalloc(&S->Xb, (size_t)batch * S->lda);
    e = e ? e : dalloc(&S->Tb, (size_t)batch);
    for (float **p : {&S->Z1, &S->H1, &S->Z2, &S->H2, &S->dZ2, &S->dZ1}) e = e ? e : dalloc(p, (size_t)batch * hidden);
    e = e ? e : dalloc(&S->yb, (size_t)batch);
    e = e ? e : dalloc(&S->dy, (size_t)batch);
    e = e ? e : dalloc(&S->loss, 1);
    e = e ? e : dalloc(&S->one, 1);
    e = e ? e : dalloc(&S->mu, (size_t)S->lda);
    e = e ? e : dalloc(&S->isig, (size_t)S->lda);
    e = e ? e : dalloc(&S->Xbn, (size_t)batch * S->lda);
    if (mlp_bf16_supported(din, hidden)) {
        const long long rp = ((long long)batch + 127) / 128 * 128;
        S->tb.rp = rp;
        e = e ? e : dalloc(&S->wimg, mlp_bf16_image_bytes(hidden));
        e = e ? e : dalloc(&S->tb.xnT, (size_t)64 * rp);
        for (uint16_t **p : {&S->tb.h1T, &S->tb.h2T, &S->tb.dz2T, &S->tb.dz1T}) e = e ? e : dalloc(p, (size_t)hidden * rp);
        e = e ? e : dalloc(&S->tb.dy, (size_t)rp);
        S->mode = SPEO_SURROGATE_BF16_SCREEN | SPEO_SURROGATE_BF16_TRAIN;
    }
    if (e) { speo_surrogate_destroy(reinterpret_cast<speo_surrogate *>(S)); return e; }
    // He-style initialisation from Philox on the host side of the stream: uniform(-a, a)
    float *h_theta = new float[S->np];
    const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
    auto uni = [&](uint32_t i) {
        // Philox is device code; a host SplitMix64 stream seeds the weights
        uint64_t z = ((uint64_t)k1 << 32 | k0) + 0x9E3779B97F4A7C15ULL * (uint64_t)(i + 1);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
        z ^= z >> 31;
        return (float)((z >> 40) * (1.0 / 16777216.0)) * 2.f - 1.f;
    };
    size_t o = 0;
    const float a1 = sqrtf(6.f / din), a2 = sqrtf(6.f / hidden);
    for (int i = 0; i < hidden * din; ++i, ++o) h_theta[o] = a1 * uni((uint32_t)o);
    for (int i = 0; i < hidden; ++i, ++o) h_theta[o] = 0.f;
    for (int i = 0; i < hidden * hidden; ++i, ++o) h_theta[o] = a2 * uni((uint32_t)o);
    for (int i = 0; i < hidden; ++i, ++o) h_theta[o] = 0.f;
    for (int i = 0; i < hidden; ++i, ++o) h_theta[o] = a2 * uni((uint32_t)o);
    h_theta[o++] = 0.f;
    const float one = 1.f;
    e = check_cuda(cudaMemcpy(S->theta, h_theta, sizeof(float) * S->np, cudaMemcpyHostToDevice), "init theta");
    delete[] h_theta;
    e = e ? e : check_cuda(cudaMemset(S->m, 0, sizeof(float) * S->np), "memset m");
    e = e ? e : check_cuda(cudaMemset(S->v, 0, sizeof(float) * S->np), "memset v");
    e = e ? e : check_cuda(cudaMemcpy(S->one, &one, sizeof(float), cudaMemcpyHostToDevice), "one");
    {   // default standardisation: x' = x * in_scale
        float *h_mu = new float[S->lda], *h_is = new float[S->lda];
        for (int d = 0; d < S->lda; ++d) { h_mu[d] = 0.f; h_is[d] = in_scale; }
        e = e ? e : check_cuda(cudaMemcpy(S->mu, h_mu, sizeof(float) * S->lda, cudaMemcpyHostToDevice), "mu");
        e = e ? e : check_cuda(cudaMemcpy(S->isig, h_is, sizeof(float) * S->lda, cudaMemcpyHostToDevice), "isig");
        delete[] h_mu;
        delete[] h_is;
    }
    if (e) { speo_surrogate_destroy(reinterpret_cast<speo_surrogate *>(S)); return e; }
    *out = reinterpret_cast<speo_surrogate *>(S);
    return SPEO_OK;
}

extern "C" int speo_surrogate_destroy(speo_surrogate *sp)
{
    Surrogate *S = reinterpret_cast<Surrogate *>(sp);
    if (!S) return SPEO_OK;
    for (float *p : {S->theta, S->m, S->v, S->grad, S->gpart, S->AX, S->AT, S->Xb, S->Tb, S->Z1, S->H1, S->Z2, S->H2, S->yb,
                     S->dy, S->dZ2, S->dZ1, S->loss, S->one, S->sH1, S->sH2, S->T, S->pred, S->sel, S->fsel, S->mu,
                     S->isig, S->Xbn, S->Xn})
        if (p) cudaFree(p);
    if (S->wimg) cudaFree(S->wimg);
    if (S->dst) cudaFree(S->dst);
    for (void *p : {(void *)S->tb.xnT, (void *)S->tb.h1T, (void *)S->tb.h2T, (void *)S->tb.dz2T, (void *)S->tb.dz1T,
                    (void *)S->tb.dy})
        if (p) cudaFree(p);
    delete S;
    return SPEO_OK;
}

extern "C" int speo_surrogate_params(speo_surrogate *sp, float **d_theta, float **d_grad, int *n_params)
{
    Surrogate *S = reinterpret_cast<Surrogate *>(sp);
    if (!S) return fail(SPEO_ERR_INVALID_ARG, "speo_surrogate_params: null");
    if (d_theta) *d_theta = S->theta;
    if (d_grad) *d_grad = S->grad;
    if (n_params) *n_params = S->np;
    return SPEO_OK;
}

extern "C" int speo_surrogate_forward(speo_surrogate *sp, const float *X, int n, int ldx, float *y, void *stream)
{
    Surrogate *S = reinterpret_cast<Surrogate *>(sp);
    if (!S || !X || !y || n < 0 || ldx < S->din) return fail(SPEO_ERR_INVALID_ARG, "speo_surrogate_forward: bad arguments");
    if (n == 0) return SPEO_OK;
    if (S->scr_rows < n) {
        if (S->sH1) cudaFree(S->sH1);
        if (S->sH2) cudaFree(S->sH2);
        S->sH1 = S->sH2 = nullptr;
        S->scr_rows = 0;
        if (int e = dalloc(&S->sH1, (size_t)n * S->h)) return e;
        if (int e = dalloc(&S->sH2, (size_t)n * S->h)) return e;
        S->scr_rows = n;
    }
    if (S->nrm_rows < n) {
        if (S->Xn) cudaFree(S->Xn);
        S->Xn = nullptr;
        S->nrm_rows = 0;
        if (int e = dalloc(&S->Xn, (size_t)n * S->lda)) return e;
        S->nrm_rows = n;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (int e = standardise(S, st, X, n, ldx, S->Xn)) return e;
    return mlp_forward(S, st, S->Xn, n, S->lda, y, nullptr, S->sH1, nullptr, S->sH2);
}

// The same network on the tensor cores: BF16 operands (inputs standardised in FP32 first, weights
// and hidden activations rounded to BF16), FP32 accumulation, FP32 head.
extern "C" int speo_surrogate_forward_bf16(speo_surrogate *sp, const float *X, long long n, int ldx, float *y,
                                           void *stream)
{
    Surrogate *S = reinterpret_cast<Surrogate *>(sp);
    if (!S || !X || !y || n < 0 || ldx < S->din)
        return fail(SPEO_ERR_INVALID_ARG, "speo_surrogate_forward_bf16: bad arguments");
    if (!S->wimg)
        return fail(SPEO_ERR_UNSUPPORTED, "speo_surrogate_forward_bf16: din %d, hidden %d (takes din <= 64, hidden "
                                          "64 / 128 / 256)", S->din, S->h);
    return mlp_forward_bf16(S->theta, S->din, S->h, S->mu, S->isig, X, n, ldx, y, S->wimg,
                            static_cast<cudaStream_t>(stream));
}

// Standardise the MLP's inputs by the per-dimension mean and standard deviation of `rows` rows of
// pop (stride ld); later forward passes and training batches use these statistics.
extern "C" int speo_surrogate_standardize(speo_surrogate *sp, const float *pop, long long rows, int ld, void *stream)
{
    Surrogate *S = reinterpret_cast<Surrogate *>(sp);
    if (!S || !pop || rows < 1 || ld < S->din) return fail(SPEO_ERR_INVALID_ARG, "speo_surrogate_standardize: bad arguments");
    k_input_stats<<<S->din, 256, 0, static_cast<cudaStream_t>(stream)>>>(pop, rows, ld, S->din, S->mu, S->isig);
    return check_launch("k_input_stats");
}

extern "C" int speo_surrogate_grad(speo_surrogate *sp, const float *X, int n, int ldx, const float *T, float *loss_out,
                                   void *stream)
{
    Surrogate *S = reinterpret_cast<Surrogate *>(sp);
    if (!S || !X || !T || n < 1 || n > S->batch || ldx < S->din)
        return fail(SPEO_ERR_INVALID_ARG, "speo_surrogate_grad: bad arguments");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (int e = mlp_grad(S, st, X, n, ldx, T)) return e;
    if (loss_out) {
        float l = 0.f;
        if (int e = check_cuda(cudaMemcpyAsync(&l, S->loss, sizeof(float), cudaMemcpyDeviceToHost, st), "loss")) return e;
        if (int e = check_cuda(cudaStreamSynchronize(st), "loss sync")) return e;
        *loss_out = l / n;
    }
    return SPEO_OK;
}

extern "C" int speo_surrogate_grad_bf16(speo_surrogate *sp, const float *X, int n, int ldx, const float *T,
                                        float *loss_out, void *stream)
{
    Surrogate *S = reinterpret_cast<Surrogate *>(sp);
    if (!S || !X || !T || n < 1 || n > S->batch || ldx < S->din)
        return fail(SPEO_ERR_INVALID_ARG, "speo_surrogate_grad_bf16: bad arguments");
    if (!S->wimg) return fail(SPEO_ERR_UNSUPPORTED, "speo_surrogate_grad_bf16: din %d, hidden %d", S->din, S->h);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (int e = grad_bf16(S, st, X, n, ldx, T, true, true)) return e;
    if (loss_out) {
        float l = 0.f;
        if (int e = check_cuda(cudaMemcpyAsync(&l, S->loss, sizeof(float), cudaMemcpyDeviceToHost, st), "loss")) return e;
        if (int e = check_cuda(cudaStreamSynchronize(st), "loss sync")) return e;
        *loss_out = l / n;
    }
    return SPEO_OK;
}

extern "C" int speo_surrogate_set_mode(speo_surrogate *sp, int mode)
{
    Surrogate *S = reinterpret_cast<Surrogate *>(sp);
    if (!S || (mode & ~(SPEO_SURROGATE_BF16_SCREEN | SPEO_SURROGATE_BF16_TRAIN)))
        return fail(SPEO_ERR_INVALID_ARG, "speo_surrogate_set_mode: bad arguments");
    if (mode && !S->wimg)
        return fail(SPEO_ERR_UNSUPPORTED, "speo_surrogate_set_mode: the tensor-core passes take din <= 64 and hidden "
                                          "64 / 128 / 256 (din %d, hidden %d)", S->din, S->h);
    S->mode = mode;
    return SPEO_OK;
}

extern "C" int speo_surrogate_adam_step(speo_surrogate *sp, void *stream)
{
    Surrogate *S = reinterpret_cast<Surrogate *>(sp);
    if (!S) return fail(SPEO_ERR_INVALID_ARG, "speo_surrogate_adam_step: null");
    return adam(S, static_cast<cudaStream_t>(stream), S->grad, 1, 0, S->wimg);
}

extern "C" int speo_surrogate_archive_append(speo_surrogate *sp, const float *X, int n, int ldx, const float *f,
                                             void *stream)
{
    Surrogate *S = reinterpret_cast<Surrogate *>(sp);
    if (!S || !X || !f || n < 0 || ldx < S->din) return fail(SPEO_ERR_INVALID_ARG, "speo_surrogate_archive_append: bad arguments");
    if (n == 0) return SPEO_OK;
    const long long total = (long long)n * S->lda;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    k_archive_append<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(X, ldx, f, n, S->din, S->AX, S->lda, S->AT,
                                                                      S->dst, S->cap);
    if (int e = check_launch("k_archive_append")) return e;
    k_archive_advance<<<1, 1, 0, st>>>(S->dst, n, S->cap);
    S->head = (S->head + n) % S->cap;
    S->count = S->count + n < S->cap ? S->count + n : S->cap;
    return check_launch("k_archive_advance");
}

// `steps` Adam steps on batches sampled from the archive; the mean batch loss of the last step
// goes to *loss_out when non-null (synchronises). The batch holds min(archive rows, batch) rows
// (drawn with replacement from the rows present when the step runs); under stream capture that
// size is the one at capture time.
extern "C" int speo_surrogate_train(speo_surrogate *sp, int steps, float *loss_out, void *stream)
{
    Surrogate *S = reinterpret_cast<Surrogate *>(sp);
    if (!S || steps < 0) return fail(SPEO_ERR_INVALID_ARG, "speo_surrogate_train: bad arguments");
    if (S->count == 0 || steps == 0) return SPEO_OK;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int n = (int)(S->count < S->batch ? S->count : S->batch);
    const bool bf16 = (S->mode & SPEO_SURROGATE_BF16_TRAIN) != 0;
    for (int i = 0; i < steps; ++i) {
        if (bf16) {  // batch drawn inside the gradient kernel; Adam sums the chunk partials
            if (int e = grad_bf16(S, st, nullptr, n, S->lda, nullptr, i == 0, false)) return e;
            if (int e = adam(S, st, S->gpart, (n + kSplitRows - 1) / kSplitRows, S->gstride(), S->wimg)) return e;
        } else {
            const long long total = (long long)n * S->lda;
            k_archive_sample<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(
                S->AX, S->lda, S->AT, S->dst, n, make_uint2((uint32_t)S->seed, (uint32_t)(S->seed >> 32)), S->Xb,
                S->Tb);
            if (int e = check_launch("k_archive_sample")) return e;
            if (int e = mlp_grad(S, st, S->Xb, n, S->lda, S->Tb)) return e;
            if (int e = adam(S, st, S->grad, 1, 0, nullptr)) return e;
        }
    }
    if (loss_out) {
        float l = 0.f;
        if (int e = check_cuda(cudaMemcpyAsync(&l, S->loss, sizeof(float), cudaMemcpyDeviceToHost, st), "loss")) return e;
        if (int e = check_cuda(cudaStreamSynchronize(st), "loss sync")) return e;
        *loss_out = l / n;
    }
    return SPEO_OK;
}

extern "C" int speo_make_trials(const speo_segment *segs, const speo_work_item *items, int n_items, int dim_hi, int k,
                                const float *pop, const float *fit, float *T, const uint32_t *d_gen, void *stream)
{
    if (!segs || !items || !pop || !fit || !T || !d_gen || n_items < 1 || k < 1 || k > 64)
        return fail(SPEO_ERR_INVALID_ARG, "speo_make_trials: bad arguments");
    (void)dim_hi;
    const int grid = n_items < 4 * sm_count() ? n_items : 4 * sm_count();
    k_make_trials<<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(segs, items, n_items, k, pop, fit, T, d_gen);
    return check_launch("k_make_trials");
}

// One surrogate-screened generation over a flat population of `rows` rows (stride ld, all
// segments D <= dim_hi): k trials per target, MLP screening, exact evaluation of the chosen
// trial, strict-`<` selection into (pop_out, fit_out), archive append, `train_steps` Adam steps.
// *d_gen advances by one (the caller's generation counter, shared with speo_generation).
extern "C" int speo_surrogate_generation(speo_surrogate *sp, const speo_segment *segs, const speo_work_item *items,
                                         int n_items, int dim_lo, int dim_hi, long long rows, int ld, int k,
                                         const float *pop_in, const float *fit_in, float *pop_out, float *fit_out,
                                         uint32_t *d_gen, int train_steps, float explore, void *stream)
{
    Surrogate *S = reinterpret_cast<Surrogate *>(sp);
    if (!S || !segs || !items || !pop_in || !fit_in || !pop_out || !fit_out || !d_gen || rows < 1 || k < 1 ||
        ld < dim_hi || (ld & 3) || dim_hi > S->din)
        return fail(SPEO_ERR_INVALID_ARG, "speo_surrogate_generation: bad arguments");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (S->trial_cap < rows * k) {
        for (float **p : {&S->T, &S->pred, &S->sel, &S->fsel})
            if (*p) { cudaFree(*p); *p = nullptr; }
        S->trial_cap = 0;
        if (int e = dalloc(&S->T, (size_t)rows * k * ld)) return e;
        if (int e = dalloc(&S->pred, (size_t)rows * k)) return e;
        if (int e = dalloc(&S->sel, (size_t)rows * ld)) return e;
        if (int e = dalloc(&S->fsel, (size_t)rows)) return e;
        // padding columns of the trial rows are never written: keep them zero
        if (int e = check_cuda(cudaMemsetAsync(S->T, 0, sizeof(float) * (size_t)rows * k * ld, st), "memset T")) return e;
        if (int e = check_cuda(cudaMemsetAsync(S->sel, 0, sizeof(float) * (size_t)rows * ld, st), "memset sel")) return e;
        S->trial_cap = rows * k;
    }
    if (S->count == 0) {  // first screened generation: the exact-evaluated parents seed the archive
        if (int e = speo_surrogate_archive_append(sp, pop_in, (int)rows, ld, fit_in, stream)) return e;
    }
    if (int e = speo_surrogate_standardize(sp, pop_in, rows, ld, stream)) return e;
    if (int e = speo_make_trials(segs, items, n_items, dim_hi, k, pop_in, fit_in, S->T, d_gen, stream)) return e;
    if (S->mode & SPEO_SURROGATE_BF16_SCREEN) {  // screening on the tensor cores
        if (int e = speo_surrogate_forward_bf16(sp, S->T, rows * k, ld, S->pred, stream)) return e;
    } else {
        if (int e = speo_surrogate_forward(sp, S->T, (int)(rows * k), ld, S->pred, stream)) return e;
    }
    const int nch = (dim_hi + 3) / 4;
    k_pick<<<(unsigned)((rows * nch + 255) / 256), 256, 0, st>>>(
        S->T, S->pred, k, S->sel, rows, ld, dim_hi, explore, make_uint2((uint32_t)S->seed, (uint32_t)(S->seed >> 32)),
        d_gen);
    if (int e = check_launch("k_pick")) return e;
    if (int e = speo_evaluate(segs, items, n_items, dim_lo, dim_hi, S->sel, S->fsel, stream)) return e;
    const int nchl = ld / 4;
    k_select_flat<<<(unsigned)((rows * nchl + 255) / 256), 256, 0, st>>>(pop_in, fit_in, S->sel, S->fsel, pop_out,
                                                                          fit_out, rows, ld, nchl);
    if (int e = check_launch("k_select_flat")) return e;
    // advance the generation counter (one thread, after every reader above on this stream)
    k_advance_gen<<<1, 1, 0, st>>>(d_gen, 1u);
    if (int e = check_launch("k_advance_gen")) return e;
    if (int e = speo_surrogate_archive_append(sp, S->sel, (int)rows, ld, S->fsel, stream)) return e;
    return speo_surrogate_train(sp, train_steps, nullptr, stream);
}

extern "C" int speo_select_rows(const float *pop_in, const float *fit_in, const float *trial, const float *trial_fit,
                                float *pop_out, float *fit_out, long long rows, int ld, void *stream)
{
    if (!pop_in || !fit_in || !trial || !trial_fit || !pop_out || !fit_out || rows < 1 || ld < 4 || (ld & 3))
        return fail(SPEO_ERR_INVALID_ARG, "speo_select_rows: bad arguments");
    const int nchl = ld / 4;
    k_select_flat<<<(unsigned)((rows * nchl + 255) / 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        pop_in, fit_in, trial, trial_fit, pop_out, fit_out, rows, ld, nchl);
    return check_launch("k_select_flat");
}
