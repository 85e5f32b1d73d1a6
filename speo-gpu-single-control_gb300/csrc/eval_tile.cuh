// eval_tile.cuh -- the tile descriptor of the CUDA-core evaluation kernels and the tile body of
// the multi-component CEC2014 functions (17-30), shared by the drop-in and segment kernels.
#pragma once

#include "cec_multi.cuh"
#include "eval_simt.cuh"

namespace speo {

constexpr int kChunk = 32;  // rows of M^T staged per step

struct TileDesc {
    const void *x;        // first row of the tile
    long long ldx;        // row stride (elements)
    int count;            // rows in the tile (<= kEvalTile)
    int D, func, ld_rot;
    const void *shift, *rot;
    void *fit;            // fitness of the first row of the tile
    // ids 17-30: component c's shift / matrix / shuffle start c * *_cs elements after the first
    long long shift_cs, rot_cs, shuf_cs;
    const int *shuf;      // 1-based shuffles (ids 17-22, 29, 30)
};

template <typename T, int TILE = kEvalTile>
__device__ __forceinline__ TileDesc ref_tile(int t, const T *X, int ldx, int P, int D, int func, const T *shift,
                                             const T *rot, T *fit)
{
    TileDesc d;
    d.x = X + (size_t)t * TILE * ldx;
    d.ldx = ldx;
    d.count = min(TILE, P - t * TILE);
    d.D = D;
    d.func = func;
    d.ld_rot = D;
    d.shift = shift;
    d.rot = rot;
    d.fit = fit + (size_t)t * TILE;
    d.shift_cs = d.rot_cs = d.shuf_cs = 0;
    d.shuf = nullptr;
    return d;
}

// The reference's device layout of the multi-component data (CUDA_EA_library/CEC2014_CUDA.cc:
// 160-281): component c's shift at c * np2, its M^T (np2 rows of D) at c * np2 * D, its shuffle
// at c * np2, np2 = max(32, next power of two >= D).
template <typename T, int TILE>
__device__ __forceinline__ TileDesc ref_tile_multi(int t, const T *X, int ldx, int P, int D, int func,
                                                   const T *shift, const T *rot, const int *shuf, T *fit)
{
    TileDesc d = ref_tile<T, TILE>(t, X, ldx, P, D, func, shift, rot, fit);
    d.shift_cs = ldx;
    d.rot_cs = (long long)ldx * D;
    d.shuf_cs = ldx;
    d.shuf = shuf;
    return d;
}

// Ids 17-30 on one tile: per component, stage x - o_c (and the 0-based shuffle), accumulate the
// squared distance of the composition weights, rotate by M_c from shared-memory chunks, evaluate
// the component's body (a hybrid reads its rotated row back from the warp's own rows of Ys,
// gathered through the shuffle) and keep the result per row in shared memory; then mix.
constexpr int kMaxComp = 5;

// Ampere-style asynchronous global -> shared copies (cp.async), element-sized.
template <typename T>
__device__ __forceinline__ void cp_async_elem(T *smem, const T *gmem)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    if constexpr (sizeof(T) == 4)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait()
{
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// The chunks of M_c^T the tile consumes, in order: (component, first row) for every rotated
// component below cend, kChunk rows at a time. Returns false past the last one.
__device__ __forceinline__ bool multi_next_chunk(int func, int D, int cend, int &c, int &kc, bool started)
{
    if (started && kc + kChunk < D) {
        kc += kChunk;
        return true;
    }
    for (int n = started ? c + 1 : c; n < cend; ++n)
        if (multi_hybrid(func, n) >= 0 || comp_piece(func, n).rotated) {
            c = n;
            kc = 0;
            return true;
        }
    return false;
}

template <typename T, int Q>
__device__ __forceinline__ void issue_chunk(const TileDesc &d, int c, int kc, T *Mb)
{
    constexpr int W = 32 * Q;
    const T *rot = static_cast<const T *>(d.rot) + c * d.rot_cs;
    const int D = d.D, rows = min(kc + kChunk, D) - kc, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int r = warp; r < rows; r += blockDim.x >> 5) {
        const T *src = rot + (size_t)(kc + r) * d.ld_rot;
        for (int j = lane; j < D; j += 32) cp_async_elem<T>(Mb + r * W + j, src + j);
    }
    cp_async_commit();
}

// Ids 17-30 on one tile of 8 * RPW rows, components [cbeg, cend): the x rows are staged once
// (cp.async); per component,
// x - o_c is formed in shared memory, the squared distance for the composition weights is
// accumulated, M_c^T streams through two shared-memory chunk buffers (the next chunk, of this or
// the next rotated component, is in flight while the current one is used), the component's body
// runs (a hybrid reads its rotated row back from the warp's own rows of Ys, gathered through the
// shuffle), and the result per row stays in shared memory (fbuf / sbuf [row][component], on lane 0
// of the row's warp); with `finish` the components are then mixed and the fitness written.
template <typename T, int Q, int RPW = kRowsPerWarp>
__device__ __noinline__ void eval_multi_tile(const TileDesc &d, T *Ys, T *Ms, T *Xs, int *Ss, T *fbuf, T *sbuf,
                                             unsigned int *err, int cbeg, int cend, bool finish)
{
    constexpr int W = 32 * Q, kRows = 8 * RPW;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, row0 = warp * RPW;
    const T *X = static_cast<const T *>(d.x);
    const int D = d.D;
    const bool comp = func_composition(d.func);
    T *Mbuf[2] = {Ms, Ms + kChunk * W};
    __syncthreads();  // the previous tile is done with every buffer
    for (int r = warp; r < kChunk; r += blockDim.x >> 5)  // zero columns D..W-1
        for (int j = D + lane; j < W; j += 32) {
            Mbuf[0][r * W + j] = T(0);
            Mbuf[1][r * W + j] = T(0);
        }
    for (int i = threadIdx.x; i < kRows * W; i += blockDim.x) {
        const int r = i / W, k = i - r * W;
        if (r < d.count && k < D) cp_async_elem<T>(Xs + i, X + (size_t)r * d.ldx + k);
        else Xs[i] = T(0);
    }
    cp_async_commit();
    int cc = cbeg, ck = 0;
    bool pending = multi_next_chunk(d.func, D, cend, cc, ck, false);
    if (pending) issue_chunk<T, Q>(d, cc, ck, Mbuf[0]);
    int buf = 0;
    for (int c = cbeg; c < cend; ++c) {
        const int h = multi_hybrid(d.func, c);
        const T *o = static_cast<const T *>(d.shift) + c * d.shift_cs;
        if (c == cbeg) {
            if (pending) cp_async_wait<1>();
            else cp_async_wait<0>();
        }
        __syncthreads();  // x rows arrived; the previous component is done with Ys / Ss
        for (int i = threadIdx.x; i < kRows * W; i += blockDim.x) {
            const int k = i % W;
            Ys[i] = k < D ? Xs[i] - o[k] : T(0);
        }
        if (h >= 0) {
            for (int k = threadIdx.x; k < W; k += blockDim.x) {
                int v = 0;
                if (k < D) {
                    v = d.shuf ? d.shuf[c * d.shuf_cs + k] - 1 : -1;
                    if (v < 0 || v >= D) {
                        atomicOr(err, SPEO_DEVERR_BAD_SEGMENT);
                        v = 0;
                    }
                }
                Ss[k] = v;
            }
        }
        __syncthreads();
        if (comp) {
#pragma unroll 1
            for (int rr = 0; rr < RPW; ++rr) {
                T sq = T(0);
#pragma unroll
                for (int q = 0; q < Q; ++q) {
                    const T v = Ys[(row0 + rr) * W + lane + 32 * q];
                    sq += v * v;
                }
                sq = warp_sum(sq);
                if (lane == 0) sbuf[(row0 + rr) * kMaxComp + c] = sq;
            }
        }
        const bool rotated = h >= 0 || comp_piece(d.func, c).rotated;
        T acc[RPW][Q];
#pragma unroll
        for (int rr = 0; rr < RPW; ++rr)
#pragma unroll
            for (int q = 0; q < Q; ++q) acc[rr][q] = T(0);
        if (rotated) {
            for (int kc = 0; kc < D; kc += kChunk) {  // (cc, ck) == (c, kc) here
                int nc2 = cc, nk = ck;
                const bool more = multi_next_chunk(d.func, D, cend, nc2, nk, true);
                if (more) {
                    issue_chunk<T, Q>(d, nc2, nk, Mbuf[buf ^ 1]);
                    cp_async_wait<1>();
                } else {
                    cp_async_wait<0>();
                }
                __syncthreads();  // chunk (c, kc) visible to every thread
                eval_accumulate<T, Q>(acc, Ys, W, row0, Mbuf[buf], W, kc, min(kc + kChunk, D), lane);
                __syncthreads();  // everyone is done with this buffer before it is refilled
                buf ^= 1;
                cc = nc2;
                ck = nk;
            }
        } else {
            eval_identity<T, Q>(acc, Ys, W, row0, D, lane);
        }
        if (h >= 0) {
            __syncwarp();
#pragma unroll
            for (int rr = 0; rr < RPW; ++rr)
#pragma unroll
                for (int q = 0; q < Q; ++q) Ys[(row0 + rr) * W + lane + 32 * q] = acc[rr][q];
            __syncwarp();
#pragma unroll 1
            for (int rr = 0; rr < RPW; ++rr) {
                const T f = hybrid_row_warp<T>(Ys + (row0 + rr) * W, Ss, h, D, lane);
                if (lane == 0) fbuf[(row0 + rr) * kMaxComp + c] = f;
            }
        } else {
            const CompPiece pc = comp_piece(d.func, c);
            const T scale = rate_of<T>(pc.fid), fs = func_fixed_shift<T>(pc.fid);
#pragma unroll 1
            for (int rr = 0; rr < RPW; ++rr) {
                ZRow<T, Q> z;
#pragma unroll
                for (int q = 0; q < Q; ++q) z.v[q] = acc[rr][q] * scale + fs;
                T f = row_objective_warp<T, Q>(z, D, pc.fid, lane);
                if (pc.den != 0.0) f = (T)pc.num * f / (T)pc.den;
                if (lane == 0) fbuf[(row0 + rr) * kMaxComp + c] = f;
            }
        }
    }
    if (finish && lane == 0) {
        T *fit = static_cast<T *>(d.fit);
#pragma unroll 1
        for (int rr = 0; rr < RPW; ++rr) {
            const int r = row0 + rr;
            if (r < d.count)
                fit[r] = comp ? comp_combine<T>(d.func, D, fbuf + r * kMaxComp, sbuf + r * kMaxComp)
                              : fbuf[r * kMaxComp];
        }
    }
}

// Tiles of 8 * RPW rows (one warp per RPW rows, 256 threads). Layout: Ys (tile), Ms (two chunk
// buffers; the first is where the single-matrix kernels keep their chunk), Xs (tile), fbuf,
// sbuf (per row and component), Ss (shuffle).
template <typename T, int Q, int RPW = kRowsPerWarp>
constexpr size_t multi_smem_bytes()
{
    return sizeof(T) * ((size_t)(2 * 8 * RPW + 2 * kChunk) * 32 * Q + 2 * 8 * RPW * kMaxComp) +
           sizeof(int) * 32 * Q;
}

template <typename T, int Q, int RPW = kRowsPerWarp>
__device__ __forceinline__ void multi_smem(unsigned char *raw, T *&Ys, T *&Ms, T *&Xs, T *&fbuf, T *&sbuf, int *&Ss)
{
    Ys = reinterpret_cast<T *>(raw);
    Ms = Ys + 8 * RPW * 32 * Q;
    Xs = Ms + 2 * kChunk * 32 * Q;
    fbuf = Xs + 8 * RPW * 32 * Q;
    sbuf = fbuf + 8 * RPW * kMaxComp;
    Ss = reinterpret_cast<int *>(sbuf + 8 * RPW * kMaxComp);
}

}  // namespace speo
