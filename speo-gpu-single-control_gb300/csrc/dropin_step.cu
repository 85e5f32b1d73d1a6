// dropin_step.cu -- whole generations of the reference-shaped drop-in path in one launch.
//
// DE_CUDA::Run (CUDA_EA_library/DE_CUDA.cc:200-216) issues API_DE_GenerateNewPopulation (best
// search + generate), API_evaluateFitness and API_DE_SelectSurvival per generation. With the loop
// in the library (speo_de_run_f32 / _f64), one block per sub-island (k_de_step), or a two-block
// cluster per sub-island (k_de_step2), runs K generations from shared
// memory: it reads the sub-island's rows (through the permutation) once, and per generation finds
// its best position (where a best-row strategy reads it, and after the last generation, whose best
// ids the three calls leave behind), draws donors and crossover masks from the same Philox counters as k_generate
// (for several generations at once: they depend only on seed, position and generation), builds
// the trials, evaluates them with the same FMA order as k_eval_ref and applies the strict-`<`
// selection. Each generation's fitness vector goes to a history buffer; after the last one the
// block writes what the three calls leave behind -- the last trials and their fitness (candidate
// buffers), the selected rows and fitness, the best ids -- and the generation counter advances by
// K, so the results are bit-identical to K rounds of the three calls.
#include "cluster.cuh"
#include "dropin.cuh"
#include "eval_simt.cuh"

SPEO_DEFINE_DEVERR(speo_deverr_dropin_step)

namespace speo {
namespace {

constexpr int kThreadsS = 512;
constexpr int kWarpsS = kThreadsS / 32;
constexpr int kPassRows = kWarpsS * kRowsPerWarp;  // 128 rows per evaluation pass

// Generations whose donor draws are made at once: enough to give every thread a position.
__host__ __device__ inline int step_draw_gens(int S)
{
    const int g = kThreadsS / S;
    return g < 1 ? 1 : g > 8 ? 8 : g;
}

template <typename T> struct StepArgs {
    T *pop, *pfit, *cand, *cfit;
    int D, S;
    const int *perm;
    const typename DeInfoT<T>::type *info;
    int *best_id;
    T lb, ub;
    RngState *rng;
    const T *shift, *rot;
    int func;
    int gens;     // generations in this launch
    int P;        // island size (row stride of the history)
    T *hist;      // gens x P fitness after each generation (may be null)
};

__host__ __device__ inline int round_up_i(int x, int m) { return (x + m - 1) / m * m; }

// Shared memory, W = 32Q = np2:  Xp[S][W] fp[round_up(S,4)] | Xt[S][W] | Yt[Sp][W] | Ms[D][W] |
// sF[Sp] | o[W] | sR[GB][S][8]   (Sp = S rounded up to the evaluation pass, GB generations of
// draws). Every region starts on a 16-byte boundary: rows are moved as 16-byte vectors.
template <typename T>
__host__ __device__ inline size_t step_smem_bytes(int Q, int S, int D)
{
    const size_t W = 32 * (size_t)Q, Sp = round_up_i(S, kPassRows);
    return sizeof(T) * (2 * (size_t)S * W + round_up_i(S, 4) + Sp * W + (size_t)D * W + Sp + W) +
           sizeof(int) * (size_t)step_draw_gens(S) * S * 8;
}

// G: the generic objective variant (ids other than 8, 9, 31).
template <typename T, int Q, bool G>
__global__ void __launch_bounds__(kThreadsS) k_de_step(StepArgs<T> a)
{
    using V = typename Vec<T>::type;
    constexpr int VN = Vec<T>::n, W = 32 * Q;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int S = a.S, D = a.D, Sp = round_up_i(S, kPassRows);
    T *Xp = reinterpret_cast<T *>(smem_raw);
    T *fp = Xp + (size_t)S * W;
    T *Xt = fp + round_up_i(S, 4);
    T *Yt = Xt + (size_t)S * W;
    T *Ms = Yt + (size_t)Sp * W;
    T *sF = Ms + (size_t)D * W;
    T *so = sF + Sp;
    int *sR = reinterpret_cast<int *>(so + W);
    __shared__ T s_bf[kWarpsS];
    __shared__ int s_bp[kWarpsS];

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int isl = blockIdx.x;
    const int base = isl * S;  // first position of this sub-island
    const uint32_t gen0 = *(volatile uint32_t *)&a.rng->gen;
    const uint2 key = make_uint2(a.rng->key0, a.rng->key1);
    const int nch = (D + VN - 1) / VN;
    const int GB = step_draw_gens(S);
    const T F = a.info[isl].F;
    const uint32_t thr = cr_threshold<T>(a.info[isl].CR);
    const int st = a.info[isl].strategy_ID;
    const int nd = ndonors(st);
    const T scale = sizeof(T) == 4 ? (T)func_scale(a.func) : (T)func_scale_f64(a.func);

    // ---- the sub-island's rows, M^T (reference layout rot[k * D + j]) and o -------------------
    for (int i = tid; i < S * (W / VN); i += kThreadsS) {
        const int p = i / (W / VN), c = i - p * (W / VN);
        reinterpret_cast<V *>(Xp + (size_t)p * W)[c] =
            reinterpret_cast<const V *>(a.pop + (size_t)a.perm[base + p] * W)[c];
    }
    for (int p = tid; p < S; p += kThreadsS) fp[p] = a.pfit[a.perm[base + p]];
    load_rot_rows<T, Q>(Ms, a.rot, D, D, 0, D);
    for (int k = tid; k < W; k += kThreadsS) so[k] = k < D ? a.shift[k] : T(0);
    for (int i = tid; i < (Sp - S) * W; i += kThreadsS) Yt[(size_t)S * W + i] = T(0);
    if (nch * VN < W) {  // columns past the last chunk stay zero in Xt and Yt
        const int tail = W - nch * VN;
        for (int i = tid; i < S * tail; i += kThreadsS) {
            const int p = i / tail, k = nch * VN + (i - p * tail);
            Xt[(size_t)p * W + k] = T(0);
            Yt[(size_t)p * W + k] = T(0);
        }
    }

    bool ok_draw = true, ok_bound = true;
    for (int g = 0; g < a.gens; ++g) {
        const uint32_t gen = gen0 + (uint32_t)g;
        const bool last = g == a.gens - 1;
        __syncthreads();
        // ---- best position (k_best): argmin of fitness, NaN as +inf, ties lowest position -----
        // read by the best-row strategies, and its id is left behind after the last generation
        const bool need_best = strategy_uses_best(st) || last;
        if (need_best) {
            T bf = T(INFINITY);
            int bp = 0x7fffffff;
            for (int p = tid; p < S; p += kThreadsS) {
                const T f = rank_t(fp[p]);
                if (f < bf || (f == bf && p < bp)) { bf = f; bp = p; }
            }
            for (int o = 16; o > 0; o >>= 1) {
                const T of = __shfl_xor_sync(0xffffffffu, bf, o);
                const int op = __shfl_xor_sync(0xffffffffu, bp, o);
                if (of < bf || (of == bf && op < bp)) { bf = of; bp = op; }
            }
            if (lane == 0) { s_bf[warp] = bf; s_bp[warp] = bp; }
        }
        // ---- donors and jrand of generations g .. g + GB - 1 (k_generate's draws) -------------
        if (g % GB == 0) {
            const int nb = a.gens - g < GB ? a.gens - g : GB;
            for (int t = tid; t < nb * S; t += kThreadsS) {
                const int gi = t / S, p = t - gi * S;
                IdxStream s(key, (uint32_t)(base + p), gen + (uint32_t)gi, kTagIdx);
                int r[5];
                ok_draw &= draw_donors(s, S, r);
                int *o = sR + (gi * S + p) * 8;
#pragma unroll
                for (int k = 0; k < 5; ++k) o[k] = r[k];
                o[5] = s.index(D);
            }
        }
        if (need_best || g % GB == 0) __syncthreads();  // block-uniform condition
        int bp = 0;
        if (need_best) {
            bp = s_bp[0];
            T bf = s_bf[0];
            for (int w = 1; w < kWarpsS; ++w)
                if (s_bf[w] < bf || (s_bf[w] == bf && s_bp[w] < bp)) { bf = s_bf[w]; bp = s_bp[w]; }
        }
        if (last && tid == 0) a.best_id[isl] = a.perm[base + bp];
        const int *sRg = sR + (g % GB) * S * 8;

        // ---- trials (k_generate): one 16-byte chunk per task ----------------------------------
        for (int t = tid; t < S * nch; t += kThreadsS) {
            const int p = t / nch, c = t - p * nch;
            const int pos = base + p;
            const int e0 = VN * c;
            const T *xi = Xp + (size_t)p * W;
            const T *xb = Xp + (size_t)(strategy_uses_best(st) ? bp : p) * W;
            const V ti = *reinterpret_cast<const V *>(xi + e0);
            const V tb = strategy_uses_best(st) ? *reinterpret_cast<const V *>(xb + e0) : ti;
            V tr[5];
#pragma unroll
            for (int k = 0; k < 5; ++k)
                tr[k] = k < nd ? *reinterpret_cast<const V *>(Xp + (size_t)sRg[p * 8 + k] * W + e0) : ti;
            const int jr = sRg[p * 8 + 5];
            const uint4 w = philox(make_uint4((uint32_t)(e0 >> 2), (uint32_t)pos, gen, kTagCr), key);
            V x = ti;
#pragma unroll
            for (int q = 0; q < VN; ++q) {
                const int e = e0 + q;
                T v;
                if (e == jr || cr_take(pick(w, (uint32_t)(e & 3)), thr)) {
                    T xr[5];
#pragma unroll
                    for (int k = 0; k < 5; ++k) xr[k] = vget<T>(tr[k], q);
                    v = mutant<T>(st, F, vget<T>(ti, q), vget<T>(tb, q), xr);
                } else {
                    v = vget<T>(ti, q);
                }
                vset<T>(x, q, check_bound<T>(v, a.lb, a.ub, ok_bound));
            }
            *reinterpret_cast<V *>(Xt + (size_t)p * W + e0) = x;
            V y;
#pragma unroll
            for (int q = 0; q < VN; ++q) {
                const int e = e0 + q;
                vset<T>(y, q, e < D ? sub_rn(vget<T>(x, q), so[e]) : T(0));
            }
            *reinterpret_cast<V *>(Yt + (size_t)p * W + e0) = y;
            if (last) {
                T *out = a.cand + (size_t)a.perm[pos] * W;
                if (e0 + VN <= D) {
                    *reinterpret_cast<V *>(out + e0) = x;
                } else {  // ragged last chunk: elements past D are never written (as in the reference)
#pragma unroll
                    for (int q = 0; q < VN; ++q)
                        if (e0 + q < D) out[e0 + q] = vget<T>(x, q);
                }
            }
        }
        __syncthreads();

        // ---- evaluation (k_eval_ref): 8 rows per warp, 128 per pass --------------------------
        for (int pb = 0; pb < S; pb += kPassRows) {
            T acc[kRowsPerWarp][Q];
#pragma unroll
            for (int rr = 0; rr < kRowsPerWarp; ++rr)
#pragma unroll
                for (int q = 0; q < Q; ++q) acc[rr][q] = T(0);
            if (func_rotated(a.func))
                eval_accumulate<T, Q>(acc, Yt, W, pb + warp * kRowsPerWarp, Ms, W, 0, D, lane);
            else
                eval_identity<T, Q>(acc, Yt, W, pb + warp * kRowsPerWarp, D, lane);
            T f[kRowsPerWarp];
            eval_reduce<T, Q, kRowsPerWarp, G>(acc, D, a.func, scale, lane, f);
            if (lane == 0)
#pragma unroll
                for (int rr = 0; rr < kRowsPerWarp; ++rr) sF[pb + warp * kRowsPerWarp + rr] = f[rr];
        }
        __syncthreads();

        // ---- selection (k_select): strict `<`, in shared memory -------------------------------
        for (int t = tid; t < S * nch; t += kThreadsS) {
            const int p = t / nch, c = t - p * nch;
            const T tf = sF[p];
            const bool win = tf < fp[p];
            if (win) *reinterpret_cast<V *>(Xp + (size_t)p * W + VN * c) = *reinterpret_cast<const V *>(Xt + (size_t)p * W + VN * c);
        }
        __syncthreads();
        for (int p = tid; p < S; p += kThreadsS) {
            const T tf = sF[p];
            const int row = a.perm[base + p];
            if (tf < fp[p]) fp[p] = tf;
            if (last) a.cfit[row] = tf;
            if (a.hist) a.hist[(size_t)g * a.P + row] = fp[p];
        }
    }
    __syncthreads();
    // ---- the sub-island's rows and fitness back (elements past D are never written) ------------
    for (int t = tid; t < S * nch; t += kThreadsS) {
        const int p = t / nch, c = t - p * nch, e0 = VN * c;
        T *dst = a.pop + (size_t)a.perm[base + p] * W;
        const V v = *reinterpret_cast<const V *>(Xp + (size_t)p * W + e0);
        if (e0 + VN <= D) {
            *reinterpret_cast<V *>(dst + e0) = v;
        } else {
#pragma unroll
            for (int q = 0; q < VN; ++q)
                if (e0 + q < D) dst[e0 + q] = vget<T>(v, q);
        }
    }
    for (int p = tid; p < S; p += kThreadsS) a.pfit[a.perm[base + p]] = fp[p];
    if (!ok_draw) atomicOr(&s_deverr, SPEO_DEVERR_REDRAW_LIMIT);
    if (!ok_bound) atomicOr(&s_deverr, SPEO_DEVERR_BOUND_LIMIT);
    // ---- advance the generation counter by K once every block has read it --------------------
    __syncthreads();
    if (tid == 0) {
        __threadfence();
        const unsigned done = atomicAdd(&a.rng->done, 1u);
        if (done == gridDim.x - 1) {
            a.rng->done = 0;
            a.rng->gen = gen0 + (uint32_t)a.gens;
            __threadfence();
        }
    }
}

template <typename T, int Q, bool G>
int launch_step_v(const StepArgs<T> &a, int nsub, cudaStream_t st)
{
    const size_t smem = step_smem_bytes<T>(Q, a.S, a.D);
    cudaError_t e = cudaFuncSetAttribute(k_de_step<T, Q, G>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return check_cuda(e, "cudaFuncSetAttribute(k_de_step)");
    k_de_step<T, Q, G><<<nsub, kThreadsS, smem, st>>>(a);
    return check_launch("k_de_step");
}

template <typename T, int Q>
int launch_step(const StepArgs<T> &a, int nsub, cudaStream_t st)
{
    return func_sum_form(a.func) ? launch_step_v<T, Q, false>(a, nsub, st) : launch_step_v<T, Q, true>(a, nsub, st);
}

// ---- two-block clusters: one sub-island per cluster of 2 -----------------------------------------
// Each block of the pair keeps a replica of the sub-island, double-buffered (generation g reads
// buffer g % 2), and runs the draws, trials, evaluation and selection of half of the positions. Its
// new rows (winner or parent) go to the next buffer of both replicas, the peer's through
// distributed shared memory; one cluster barrier per generation makes both replicas whole. The
// per-row arithmetic is k_de_step's, so the results are bit-identical. FP32 and FP64.
constexpr int kRowsPerWarp2 = 4;
constexpr int kPassRows2 = kWarpsS * kRowsPerWarp2;  // 64 rows per evaluation pass

__host__ __device__ inline int half_pos(int S) { return (S + 1) / 2; }

//   Xp[2][S][W] fp[2][round_up(S,4)] | Xt[h][W] | Yt[hp][W] | Ms[D][W] | sF[hp] | o[W] | sR[GB][h][8]
template <typename T>
__host__ __device__ inline size_t step2_smem_bytes(int Q, int S, int D)
{
    const size_t W = 32 * (size_t)Q, h = half_pos(S), hp = round_up_i((int)h, kPassRows2);
    return sizeof(T) * (2 * ((size_t)S * W + round_up_i(S, 4)) + h * W + hp * W + (size_t)D * W + hp + W) +
           sizeof(int) * (size_t)step_draw_gens((int)h) * h * 8;
}

// A row chunk (one vector) or a fitness value into the peer block's shared memory.
__device__ __forceinline__ void st_peer_v(uint32_t addr, float4 v) { st_peer4(addr, v); }
__device__ __forceinline__ void st_peer_v(uint32_t addr, double2 v)
{
    asm volatile("st.shared::cluster.v2.f64 [%0], {%1, %2};" ::"r"(addr), "d"(v.x), "d"(v.y) : "memory");
}
__device__ __forceinline__ void st_peer_s(uint32_t addr, float v) { st_peer1(addr, v); }
__device__ __forceinline__ void st_peer_s(uint32_t addr, double v)
{
    asm volatile("st.shared::cluster.f64 [%0], %1;" ::"r"(addr), "d"(v) : "memory");
}

template <typename T, int Q, bool G>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(kThreadsS, 1) k_de_step2(StepArgs<T> a)
{
    using V = typename Vec<T>::type;
    constexpr int VN = Vec<T>::n, W = 32 * Q;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int S = a.S, D = a.D, h = half_pos(S), hp = round_up_i(h, kPassRows2), Sf = round_up_i(S, 4);
    T *const Xp0 = reinterpret_cast<T *>(smem_raw);  // buffer b at Xp0 + b * S * W
    T *const fp0 = Xp0 + 2 * (size_t)S * W;              // buffer b at fp0 + b * Sf
    T *Xt = fp0 + 2 * Sf;
    T *Yt = Xt + (size_t)h * W;
    T *Ms = Yt + (size_t)hp * W;
    T *sF = Ms + (size_t)D * W;
    T *so = sF + hp;
    int *sR = reinterpret_cast<int *>(so + W);
    __shared__ T s_bf[kWarpsS];
    __shared__ int s_bp[kWarpsS];

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t me = cluster_rank(), peer = me ^ 1u;
    const int isl = blockIdx.x >> 1;
    const int base = isl * S;
    const int pb0 = (int)me * h, np = (S - pb0 < h ? S - pb0 : h);  // this block's positions [pb0, pb0 + np)
    const uint32_t gen0 = *(volatile uint32_t *)&a.rng->gen;
    const uint2 key = make_uint2(a.rng->key0, a.rng->key1);
    const int nch = (D + VN - 1) / VN;
    const int GB = step_draw_gens(h);
    const T F = a.info[isl].F;
    const uint32_t thr = cr_threshold<T>(a.info[isl].CR);
    const int st = a.info[isl].strategy_ID;
    const int nd = ndonors(st);
    const T scale = sizeof(T) == 4 ? (T)func_scale(a.func) : (T)func_scale_f64(a.func);

    for (int i = tid; i < S * (W / VN); i += kThreadsS) {
        const int p = i / (W / VN), c = i - p * (W / VN);
        reinterpret_cast<V *>(Xp0 + (size_t)p * W)[c] =
            reinterpret_cast<const V *>(a.pop + (size_t)a.perm[base + p] * W)[c];
    }
    for (int p = tid; p < S; p += kThreadsS) fp0[p] = a.pfit[a.perm[base + p]];
    load_rot_rows<T, Q>(Ms, a.rot, D, D, 0, D);
    for (int k = tid; k < W; k += kThreadsS) so[k] = k < D ? a.shift[k] : T(0);
    for (int i = tid; i < (hp - np) * W; i += kThreadsS) Yt[(size_t)np * W + i] = T(0);
    if (nch * VN < W) {
        const int tail = W - nch * VN;
        for (int i = tid; i < np * tail; i += kThreadsS) {
            const int p = i / tail, k = nch * VN + (i - p * tail);
            Xt[(size_t)p * W + k] = T(0);
            Yt[(size_t)p * W + k] = T(0);
        }
        for (int i = tid; i < S * tail; i += kThreadsS) {  // and in the second population buffer
            const int p = i / tail, k = nch * VN + (i - p * tail);
            Xp0[(size_t)S * W + (size_t)p * W + k] = T(0);
        }
    }
    const uint32_t peer_xp = map_peer(Xp0, peer), peer_fp = map_peer(fp0, peer);
    cluster_sync();

    bool ok_draw = true, ok_bound = true;
    for (int g = 0; g < a.gens; ++g) {
        const uint32_t gen = gen0 + (uint32_t)g;
        const bool last = g == a.gens - 1;
        const int cur = g & 1, nxt = cur ^ 1;
        const T *Xp = Xp0 + (size_t)cur * S * W;
        const T *fp = fp0 + cur * Sf;
        // The best position is read by the best-row strategies, and its id is left behind after
        // the last generation; other generations of other strategies skip the search.
        const bool need_best = strategy_uses_best(st) || last;
        if (need_best) {  // (the previous generation's cluster barrier ordered every access before this point)
            T bf = T(INFINITY);
            int bp = 0x7fffffff;
            for (int p = tid; p < S; p += kThreadsS) {
                const T f = rank_t(fp[p]);
                if (f < bf || (f == bf && p < bp)) { bf = f; bp = p; }
            }
            for (int o = 16; o > 0; o >>= 1) {
                const T of = __shfl_xor_sync(0xffffffffu, bf, o);
                const int op = __shfl_xor_sync(0xffffffffu, bp, o);
                if (of < bf || (of == bf && op < bp)) { bf = of; bp = op; }
            }
            if (lane == 0) { s_bf[warp] = bf; s_bp[warp] = bp; }
        }
        if (g % GB == 0) {
            const int nb = a.gens - g < GB ? a.gens - g : GB;
            for (int t = tid; t < nb * np; t += kThreadsS) {
                const int gi = t / np, lp = t - gi * np;
                IdxStream s(key, (uint32_t)(base + pb0 + lp), gen + (uint32_t)gi, kTagIdx);
                int r[5];
                ok_draw &= draw_donors(s, S, r);
                int *o = sR + (gi * h + lp) * 8;
#pragma unroll
                for (int k = 0; k < 5; ++k) o[k] = r[k];
                o[5] = s.index(D);
            }
        }
        if (need_best || g % GB == 0) __syncthreads();  // block-uniform condition
        int bp = 0;
        if (need_best) {
            bp = s_bp[0];
            T bf = s_bf[0];
            for (int w = 1; w < kWarpsS; ++w)
                if (s_bf[w] < bf || (s_bf[w] == bf && s_bp[w] < bp)) { bf = s_bf[w]; bp = s_bp[w]; }
        }
        if (last && me == 0 && tid == 0) a.best_id[isl] = a.perm[base + bp];
        const int *sRg = sR + (g % GB) * h * 8;
        T *nXp = Xp0 + (size_t)nxt * S * W;
        T *nfp = fp0 + nxt * Sf;
        const uint32_t pxp = peer_xp + (uint32_t)((size_t)nxt * S * W * sizeof(T));
        const uint32_t pfp = peer_fp + (uint32_t)(nxt * Sf * sizeof(T));
        // trials, evaluation and selection per warp, for its kRowsPerWarp2 positions of each
        // 64-position pass: a position's trial, fitness and selection stay in its warp
        for (int pb = 0; pb < np; pb += kPassRows2) {
            const int lr0 = pb + warp * kRowsPerWarp2;
            if (lr0 >= np) break;  // warp-uniform
            const int nrw = np - lr0 < kRowsPerWarp2 ? np - lr0 : kRowsPerWarp2;
            for (int t = lane; t < nrw * nch; t += 32) {
                const int lp = lr0 + t / nch, c = t % nch;
                const int p = pb0 + lp, pos = base + p;
                const int e0 = VN * c;
                const T *xi = Xp + (size_t)p * W;
                const T *xb = Xp + (size_t)(strategy_uses_best(st) ? bp : p) * W;
                const V ti = *reinterpret_cast<const V *>(xi + e0);
                const V tb = strategy_uses_best(st) ? *reinterpret_cast<const V *>(xb + e0) : ti;
                V tr[5];
#pragma unroll
                for (int k = 0; k < 5; ++k)
                    tr[k] = k < nd ? *reinterpret_cast<const V *>(Xp + (size_t)sRg[lp * 8 + k] * W + e0) : ti;
                const int jr = sRg[lp * 8 + 5];
                const uint4 w = philox(make_uint4((uint32_t)(e0 >> 2), (uint32_t)pos, gen, kTagCr), key);
                V x = ti;
#pragma unroll
                for (int q = 0; q < VN; ++q) {
                    const int e = e0 + q;
                    T v;
                    if (e == jr || cr_take(pick(w, (uint32_t)(e & 3)), thr)) {
                        T xr[5];
#pragma unroll
                        for (int k = 0; k < 5; ++k) xr[k] = vget<T>(tr[k], q);
                        v = mutant<T>(st, F, vget<T>(ti, q), vget<T>(tb, q), xr);
                    } else {
                        v = vget<T>(ti, q);
                    }
                    vset<T>(x, q, check_bound<T>(v, a.lb, a.ub, ok_bound));
                }
                *reinterpret_cast<V *>(Xt + (size_t)lp * W + e0) = x;
                V y;
#pragma unroll
                for (int q = 0; q < VN; ++q) {
                    const int e = e0 + q;
                    vset<T>(y, q, e < D ? sub_rn(vget<T>(x, q), so[e]) : T(0));
                }
                *reinterpret_cast<V *>(Yt + (size_t)lp * W + e0) = y;
                if (last) {
                    T *out = a.cand + (size_t)a.perm[pos] * W;
                    if (e0 + VN <= D) {
                        *reinterpret_cast<V *>(out + e0) = x;
                    } else {
#pragma unroll
                        for (int q = 0; q < VN; ++q)
                            if (e0 + q < D) out[e0 + q] = vget<T>(x, q);
                    }
                }
            }
            __syncwarp();
            T acc[kRowsPerWarp2][Q];
#pragma unroll
            for (int rr = 0; rr < kRowsPerWarp2; ++rr)
#pragma unroll
                for (int q = 0; q < Q; ++q) acc[rr][q] = T(0);
            if (func_rotated(a.func))
                eval_accumulate<T, Q>(acc, Yt, W, lr0, Ms, W, 0, D, lane);
            else
                eval_identity<T, Q>(acc, Yt, W, lr0, D, lane);
            T f[kRowsPerWarp2];
            eval_reduce<T, Q, kRowsPerWarp2, G>(acc, D, a.func, scale, lane, f);
            if (lane == 0)
#pragma unroll
                for (int rr = 0; rr < kRowsPerWarp2; ++rr) sF[lr0 + rr] = f[rr];
            __syncwarp();
            // selection into the next buffer of both replicas
            for (int t = lane; t < nrw * nch; t += 32) {
                const int lp = lr0 + t / nch, c = t % nch, p = pb0 + lp;
                const T tf = sF[lp];
                const bool win = tf < fp[p];
                const V v = *reinterpret_cast<const V *>((win ? Xt + (size_t)lp * W : Xp + (size_t)p * W) + VN * c);
                *reinterpret_cast<V *>(nXp + (size_t)p * W + VN * c) = v;
                st_peer_v(pxp + (uint32_t)(((size_t)p * W + VN * c) * sizeof(T)), v);
                if (c == 0) {
                    const int row = a.perm[base + p];
                    const T nf = win ? tf : fp[p];
                    nfp[p] = nf;
                    st_peer_s(pfp + (uint32_t)(p * sizeof(T)), nf);
                    if (last) a.cfit[row] = tf;
                    if (a.hist) a.hist[(size_t)g * a.P + row] = nf;
                }
            }
        }
        cluster_sync();
    }
    // this block's rows and fitness back (elements past D are never written)
    const T *Xp = Xp0 + (size_t)(a.gens & 1) * S * W;
    const T *fp = fp0 + (a.gens & 1) * Sf;
    for (int t = tid; t < np * nch; t += kThreadsS) {
        const int lp = t / nch, c = t - lp * nch, e0 = VN * c, p = pb0 + lp;
        T *dst = a.pop + (size_t)a.perm[base + p] * W;
        const V v = *reinterpret_cast<const V *>(Xp + (size_t)p * W + e0);
        if (e0 + VN <= D) {
            *reinterpret_cast<V *>(dst + e0) = v;
        } else {
#pragma unroll
            for (int q = 0; q < VN; ++q)
                if (e0 + q < D) dst[e0 + q] = vget<T>(v, q);
        }
    }
    for (int lp = tid; lp < np; lp += kThreadsS) a.pfit[a.perm[base + pb0 + lp]] = fp[pb0 + lp];
    if (!ok_draw) atomicOr(&s_deverr, SPEO_DEVERR_REDRAW_LIMIT);
    if (!ok_bound) atomicOr(&s_deverr, SPEO_DEVERR_BOUND_LIMIT);
    __syncthreads();
    if (tid == 0) {
        __threadfence();
        const unsigned done = atomicAdd(&a.rng->done, 1u);
        if (done == gridDim.x - 1) {
            a.rng->done = 0;
            a.rng->gen = gen0 + (uint32_t)a.gens;
            __threadfence();
        }
    }
}

template <typename T, int Q, bool G>
int launch_step2_v(const StepArgs<T> &a, int nsub, cudaStream_t st)
{
    const size_t smem = step2_smem_bytes<T>(Q, a.S, a.D);
    cudaError_t e = cudaFuncSetAttribute(k_de_step2<T, Q, G>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return check_cuda(e, "cudaFuncSetAttribute(k_de_step2)");
    k_de_step2<T, Q, G><<<2 * nsub, kThreadsS, smem, st>>>(a);
    return check_launch("k_de_step2");
}

template <typename T, int Q>
int launch_step2(const StepArgs<T> &a, int nsub, cudaStream_t st)
{
    return func_sum_form(a.func) ? launch_step2_v<T, Q, false>(a, nsub, st) : launch_step2_v<T, Q, true>(a, nsub, st);
}

int q_of(int D) { return D <= 32 ? 1 : D <= 64 ? 2 : D <= 128 ? 4 : 8; }

}  // namespace

bool dropin_step_fits_f32(int island_size, int subisland_num, int dim, int func)
{
    if (subisland_num < 1 || island_size % subisland_num || dim < 1 || dim > SPEO_MAX_DIM || !func_supported(func))
        return false;
    const int S = island_size / subisland_num;
    if (S < 2) return false;
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    return step_smem_bytes<float>(q_of(dim), S, dim) <= (size_t)optin;
}

bool dropin_step_fits_f64(int island_size, int subisland_num, int dim, int func)
{
    if (subisland_num < 1 || island_size % subisland_num || dim < 1 || dim > SPEO_MAX_DIM || !func_supported(func))
        return false;
    const int S = island_size / subisland_num;
    if (S < 2) return false;
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    return step_smem_bytes<double>(q_of(dim), S, dim) <= (size_t)optin;
}

namespace {

// Two-block clusters when there are SMs for two blocks per sub-island and the replicas fit, else
// one block per sub-island.
template <typename T>
int run_step(const StepArgs<T> &a, int nsub, int pair_mode, cudaStream_t st)
{
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    const int Q = q_of(a.D);
    const bool pair = pair_mode != 1 && a.S >= 4 && (pair_mode == 2 || 2LL * nsub <= sm_count()) &&
                      step2_smem_bytes<T>(Q, a.S, a.D) <= (size_t)optin;
    if (pair) {
        switch (Q) {
        case 1: return launch_step2<T, 1>(a, nsub, st);
        case 2: return launch_step2<T, 2>(a, nsub, st);
        case 4: return launch_step2<T, 4>(a, nsub, st);
        default: return launch_step2<T, 8>(a, nsub, st);
        }
    }
    switch (Q) {
    case 1: return launch_step<T, 1>(a, nsub, st);
    case 2: return launch_step<T, 2>(a, nsub, st);
    case 4: return launch_step<T, 4>(a, nsub, st);
    default: return launch_step<T, 8>(a, nsub, st);
    }
}

}  // namespace

int dropin_step_f64(speo_population_f64 pop, speo_population_f64 cand, int *d_best, speo_island_info ii,
                    speo_de_info_f64 *d_info, speo_rng_state *rng, speo_problem_info_f64 pi, const double *shift,
                    const double *rot, int generations, double *d_hist, int pair_mode, cudaStream_t st)
{
    if (generations < 1) return SPEO_OK;
    StepArgs<double> a{pop.elements, pop.fitness_value, cand.elements, cand.fitness_value, pi.dim,
                       ii.island_size / ii.subisland_num, ii.permutated_index, d_info, d_best,
                       pi.min_bound, pi.max_bound, reinterpret_cast<RngState *>(rng), shift, rot,
                       pi.function_ID, generations, ii.island_size, d_hist};
    return run_step(a, ii.subisland_num, pair_mode, st);
}

int dropin_step_f32(speo_population_f32 pop, speo_population_f32 cand, int *d_best, speo_island_info ii,
                    speo_de_info_f32 *d_info, speo_rng_state *rng, speo_problem_info_f32 pi, const float *shift,
                    const float *rot, int generations, float *d_hist, int pair_mode, cudaStream_t st)
{
    if (generations < 1) return SPEO_OK;
    StepArgs<float> a{pop.elements, pop.fitness_value, cand.elements, cand.fitness_value, pi.dim,
                      ii.island_size / ii.subisland_num, ii.permutated_index, d_info, d_best,
                      (float)pi.min_bound, (float)pi.max_bound, reinterpret_cast<RngState *>(rng), shift, rot,
                      pi.function_ID, generations, ii.island_size, d_hist};
    return run_step(a, ii.subisland_num, pair_mode, st);
}

}  // namespace speo
