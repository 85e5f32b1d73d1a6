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
template <typename T, int Q, int RPW = kRowsPerWarp>
__device__ __noinline__ void eval_multi_tile(const TileDesc &d, T *Ys, T *Ms, int *Ss, T *fbuf, T *sbuf,
                                             unsigned int *err)
{
    constexpr int W = 32 * Q;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, row0 = warp * RPW;
    const T *X = static_cast<const T *>(d.x);
    const int nc = func_components(d.func), D = d.D;
    const bool comp = func_composition(d.func);
    for (int c = 0; c < nc; ++c) {
        const int h = multi_hybrid(d.func, c);
        const T *o = static_cast<const T *>(d.shift) + c * d.shift_cs;
        const T *rot = static_cast<const T *>(d.rot) + c * d.rot_cs;
        __syncthreads();  // previous component (or tile) done with Ys / Ss / Ms
        for (int i = threadIdx.x; i < 8 * RPW * W; i += blockDim.x) {
            const int r = i / W, k = i - r * W;
            Ys[i] = (r < d.count && k < D) ? X[(size_t)r * d.ldx + k] - o[k] : T(0);
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
            for (int kc = 0; kc < D; kc += kChunk) {
                const int ke = min(kc + kChunk, D);
                __syncthreads();
                load_rot_rows<T, Q>(Ms, rot, d.ld_rot, D, kc, ke);
                __syncthreads();
                eval_accumulate<T, Q>(acc, Ys, W, row0, Ms, W, kc, ke, lane);
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
    if (lane == 0) {
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

// Tiles of 8 * RPW rows (one warp per RPW rows, 256 threads).
template <typename T, int Q, int RPW = kRowsPerWarp>
constexpr size_t multi_smem_bytes()
{
    return sizeof(T) * ((size_t)(8 * RPW + kChunk) * 32 * Q + 2 * 8 * RPW * kMaxComp) + sizeof(int) * 32 * Q;
}

template <typename T, int Q, int RPW = kRowsPerWarp>
__device__ __forceinline__ void multi_smem(unsigned char *raw, T *&Ys, T *&Ms, T *&fbuf, T *&sbuf, int *&Ss)
{
    Ys = reinterpret_cast<T *>(raw);
    Ms = Ys + 8 * RPW * 32 * Q;
    fbuf = Ms + kChunk * 32 * Q;
    sbuf = fbuf + 8 * RPW * kMaxComp;
    Ss = reinterpret_cast<int *>(sbuf + 8 * RPW * kMaxComp);
}

}  // namespace speo
