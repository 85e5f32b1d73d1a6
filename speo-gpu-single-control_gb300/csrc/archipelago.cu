// archipelago.cu -- the reference's migration policy family (src/migrate.cc:34-186,
// src/buffer_manage.cc:36-313) as device operations over many islands on one GPU.
//
// The reference keeps one island per MPI rank: destination lists, an immigrant buffer and a
// sub-island permutation per rank, messages of migration_size rows over MPI, and the buffer and
// population updates on the host after full-population device-to-host copies. Here every
// island's lists and buffer live in one device state block and the three steps are kernels:
//   k_mig_out      one block per island: refill a used-up destination list (dynamicConnect), take
//                  the buffer's selection into distinct random rows, regroup;
//   k_mig_deliver  one block per receiving island: the messages sent to it this generation, in
//                  source-island order, through its buffer policy (OnlineCluster's nearest-centre
//                  search runs one thread per centre);
//   k_mig_advance  one thread per island: drop the head of every list that sent.
// State per island (ints): [0] list length, [1] list head, [2] buffer size, [3] 0, list[N],
// member[C], flag[C], order[C]; (floats): entry[C][D+1] (row + fitness), centre[C][D].
#include "common.cuh"
#include "host.h"

namespace speo {
namespace {

constexpr uint32_t kTagDest = 7u, kTagEmig = 8u, kTagImport = 9u, kTagRegroup = 10u, kTagRandSel = 11u;
constexpr int kMinSubisland = 4;  // MIN_SUBISLAND_SIZE (include/config.h:25)
constexpr int kMaxCap = SPEO_ARCHIPELAGO_MAX_CAPACITY;
constexpr int kThreads = 256;

struct Arch {
    int N, P, D, ld, C, k, policy, regroup;
    float rate;
    uint2 key;
    int istride, fstride;
    int *ints;
    float *flts;
    __device__ int *hdr(int i) const { return ints + (size_t)i * istride; }
    __device__ int *list(int i) const { return hdr(i) + 4; }
    __device__ int *member(int i) const { return hdr(i) + 4 + N; }
    __device__ int *flag(int i) const { return member(i) + C; }
    __device__ int *order(int i) const { return flag(i) + C; }
    __device__ float *entry(int i, int c) const { return flts + (size_t)i * fstride + (size_t)c * (D + 1); }
    __device__ float *centre(int i, int c) const
    {
        return flts + (size_t)i * fstride + (size_t)C * (D + 1) + (size_t)c * D;
    }
};

int istride_of(const speo_archipelago &a)
{
    return (4 + a.n_islands + 3 * a.buffer_capacity + 3) / 4 * 4;
}
int fstride_of(const speo_archipelago &a)
{
    return (a.buffer_capacity * (2 * a.dim + 1) + 3) / 4 * 4;
}

// ---- keyed Feistel permutation of [0, n) with cycle walking --------------------------------
struct FPerm {
    uint32_t n, h, mask;
    uint4 k;
};
__device__ __forceinline__ uint32_t fmix32(uint32_t v)
{
    v ^= v >> 16;
    v *= 0x85EBCA6Bu;
    v ^= v >> 13;
    v *= 0xC2B2AE35u;
    v ^= v >> 16;
    return v;
}
__device__ __forceinline__ FPerm fperm(uint32_t n, uint4 k)
{
    uint32_t bits = 0;
    while (bits < 30 && (1u << bits) < n) ++bits;
    uint32_t h = (bits + 1) / 2;
    if (h == 0) h = 1;
    return {n, h, (1u << h) - 1u, k};
}
__device__ __forceinline__ uint32_t fperm_at(const FPerm &p, uint32_t x)
{
    const uint32_t kr[4] = {p.k.x, p.k.y, p.k.z, p.k.w};
    const uint32_t lim = 1u << (2 * p.h);
    for (uint32_t it = 0; it < lim; ++it) {  // returns within one cycle of the permutation
        uint32_t L = x >> p.h, R = x & p.mask;
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const uint32_t t = L ^ (fmix32(R * 0x9E3779B1u ^ kr[r]) & p.mask);
            L = R;
            R = t;
        }
        x = (L << p.h) | R;
        if (x < p.n) return x;
    }
    return 0u;
}

__device__ __forceinline__ uint32_t draw_below(uint32_t w, uint32_t n)
{
    return (uint32_t)(((uint64_t)w * n) >> 32);
}

// Erase buffer position pos: its slot moves behind the live entries.
__device__ __forceinline__ void erase_pos(int *order, int size, int pos)
{
    const int slot = order[pos];
    for (int i = pos; i < size - 1; ++i) order[i] = order[i + 1];
    order[size - 1] = slot;
}

// ---- MigrateOut: UpdateDestination + UpdatePopulation + RegroupIslands ------------------------
__global__ void __launch_bounds__(kThreads) k_mig_out(Arch a, float *pop, float *fit, int *perm, int *subisland_num,
                                                      uint32_t g)
{
    __shared__ int sel[kMaxCap];
    __shared__ int nsel;
    const int s = blockIdx.x, tid = threadIdx.x;
    int *h = a.hdr(s);
    if (tid == 0) {
        // UpdateDestination (migrate.cc:34-44): refill a used-up list
        if (h[1] >= h[0]) {
            int cnt = 0;
            int *list = a.list(s);
            for (int t = 0; t < a.N; ++t) {
                if (t == s) continue;
                const uint4 w = philox(make_uint4((uint32_t)t, (uint32_t)s, g, kTagDest), a.key);
                if (u01(w.x) < a.rate) list[cnt++] = t;
            }
            h[0] = cnt;
            h[1] = 0;
        }
        // SelectFromBuffer (buffer_manage.cc:105-117, 193-212, 231-245, 264-278, 299-313)
        int size = h[2], n = 0;
        int *order = a.order(s), *flag = a.flag(s);
        if (a.policy == SPEO_BUFFER_ONLINE_CLUSTER) {
            for (int c = 0; c < size; ++c)
                if (flag[c]) {
                    sel[n++] = c;
                    flag[c] = 0;
                }
        } else {
            for (int q = 0; q < a.k && size > 0; ++q) {
                int pos = 0;
                if (a.policy == SPEO_BUFFER_BEST) {  // FindBestBufferMember: the largest fitness, first one
                    float bf = a.entry(s, order[0])[a.D];
                    for (int i = 1; i < size; ++i) {
                        const float f = a.entry(s, order[i])[a.D];
                        if (bf < f) { bf = f; pos = i; }
                    }
                } else if (a.policy == SPEO_BUFFER_RANDOM) {
                    const uint4 w = philox(make_uint4((uint32_t)q, (uint32_t)s, g, kTagRandSel), a.key);
                    pos = (int)draw_below(w.x, (uint32_t)size);
                } else if (a.policy == SPEO_BUFFER_LIFO) {
                    pos = size - 1;
                }
                sel[n++] = order[pos];
                erase_pos(order, size, pos);
                --size;
            }
        }
        h[2] = size;
        nsel = n;
    }
    __syncthreads();
    // UpdatePopulation (migrate.cc:46-62): the selection into distinct random rows
    const int n = nsel;
    if (n > 0) {
        const FPerm pr = fperm((uint32_t)a.P, philox(make_uint4((uint32_t)s, g, 0u, kTagImport), a.key));
        const int W = a.D + 1;
        for (int i = tid; i < n * W; i += kThreads) {
            const int q = i / W, j = i - q * W;
            const long long row = (long long)s * a.P + fperm_at(pr, (uint32_t)q);
            const float v = a.entry(s, sel[q])[j];
            if (j < a.D) pop[row * a.ld + j] = v;
            else fit[row] = v;
        }
    }
    // RegroupIslands (migrate.cc:147-186)
    const bool dynamic = a.regroup == SPEO_REGROUP_DYNAMIC_RANDOM || a.regroup == SPEO_REGROUP_DYNAMIC_ORDERED;
    const bool shuffled = a.regroup == SPEO_REGROUP_DYNAMIC_RANDOM || a.regroup == SPEO_REGROUP_STATIC_RANDOM;
    if (dynamic && tid == 0) {
        int max_index = 0, q = a.P / kMinSubisland;
        while (q > 1) {
            q /= 2;
            ++max_index;
        }
        const uint4 w = philox(make_uint4((uint32_t)s, g, 0u, kTagRegroup), a.key);
        const int size = kMinSubisland << draw_below(w.x, (uint32_t)(max_index + 1));
        subisland_num[s] = a.P / size;
    }
    if (shuffled) {
        const FPerm pr = fperm((uint32_t)a.P, philox(make_uint4((uint32_t)s, g, 1u, kTagRegroup), a.key));
        for (int r = tid; r < a.P; r += kThreads) perm[(size_t)s * a.P + r] = (int)fperm_at(pr, (uint32_t)r);
    }
}

// ---- MigrateIn: the messages of this generation into each receiving island's buffer ----------
__global__ void __launch_bounds__(kThreads) k_mig_deliver(Arch a, const float *pop, const float *fit, uint32_t g)
{
    __shared__ float dist[kMaxCap];
    __shared__ int slot_s;
    const int d = blockIdx.x, tid = threadIdx.x;
    int *h = a.hdr(d);
    for (int src = 0; src < a.N; ++src) {
        const int *hs = a.hdr(src);
        if (hs[1] >= hs[0] || a.list(src)[hs[1]] != d) continue;  // block-uniform
        // SendEmigrations (migrate.cc:105-136): migration_size distinct random rows of src
        const FPerm pr = fperm((uint32_t)a.P, philox(make_uint4((uint32_t)src, g, 0u, kTagEmig), a.key));
        for (int q = 0; q < a.k; ++q) {
            const long long row = (long long)src * a.P + fperm_at(pr, (uint32_t)q);
            const float *x = pop + row * a.ld;
            const float fx = fit[row];
            __syncthreads();  // previous insert done
            if (a.policy == SPEO_BUFFER_ONLINE_CLUSTER) {
                // OnlineCluster::UpdateBuffer (buffer_manage.cc:119-131)
                const int size = h[2];
                if (size < a.C) {  // CreatCluster (:51-58)
                    for (int j = tid; j <= a.D; j += kThreads) {
                        const float v = j < a.D ? x[j] : fx;
                        a.entry(d, size)[j] = v;
                        if (j < a.D) a.centre(d, size)[j] = v;
                    }
                    __syncthreads();
                    if (tid == 0) {
                        a.member(d)[size] = 1;
                        a.flag(d)[size] = 1;
                        h[2] = size + 1;
                    }
                    continue;
                }
                // FindNearestIndividual (:134-150) on CalDistance (:38-49), binary32 in order
                if (tid < a.C) {
                    const float *c = a.centre(d, tid);
                    float acc = 0.f;
                    for (int j = 0; j < a.D; ++j) {
                        const float df = __fsub_rn(x[j], c[j]);
                        acc = __fadd_rn(acc, __fmul_rn(df, df));
                    }
                    dist[tid] = __fsqrt_rn(acc);
                }
                __syncthreads();
                if (tid == 0) {
                    int best = 0;
                    float bv = dist[0];
                    for (int i = 1; i < a.C; ++i)
                        if (bv > dist[i]) { bv = dist[i]; best = i; }
                    slot_s = best;
                }
                __syncthreads();
                // ReplaceMemberToCluster (:60-76): running mean of the centre, the entry replaced
                const int c = slot_s, m = a.member(d)[c];
                for (int j = tid; j <= a.D; j += kThreads) {
                    if (j < a.D) {
                        float *cc = a.centre(d, c);
                        const float t = __fadd_rn(__fmul_rn((float)m, cc[j]), x[j]);
                        cc[j] = __double2float_rn(__ddiv_rn((double)t, (double)m + 1.0));
                        a.entry(d, c)[j] = x[j];
                    } else {
                        a.entry(d, c)[j] = fx;
                    }
                }
                __syncthreads();
                if (tid == 0) {
                    a.member(d)[c] = m + 1;
                    a.flag(d)[c] = 1;
                }
            } else {
                // BestSelect / RandomSelect / FIFO / LIFO ::UpdateBuffer: push_back, then drop the
                // oldest past capacity
                if (tid == 0) {
                    int *order = a.order(d);
                    const int size = h[2];
                    if (size < a.C) {
                        slot_s = order[size];
                        h[2] = size + 1;
                    } else {
                        const int slot = order[0];
                        erase_pos(order, size, 0);
                        slot_s = slot;
                    }
                }
                __syncthreads();
                float *e = a.entry(d, slot_s);
                for (int j = tid; j <= a.D; j += kThreads) e[j] = j < a.D ? x[j] : fx;
            }
        }
    }
}

__global__ void k_mig_advance(Arch a)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < a.N) {
        int *h = a.hdr(s);
        if (h[1] < h[0]) h[1] += 1;
    }
}

__global__ void k_mig_init(Arch a, int *perm, int *subisland_num, int nsub)
{
    const size_t n_int = (size_t)a.N * a.istride, n_flt = (size_t)a.N * a.fstride;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n_int + n_flt + (size_t)a.N * a.P;
         i += (size_t)gridDim.x * blockDim.x) {
        if (i < n_int) {
            const int s = (int)(i / a.istride), o = (int)(i - (size_t)s * a.istride);
            const int obase = 4 + a.N + 2 * a.C;
            a.ints[i] = (o >= obase && o < obase + a.C) ? o - obase : 0;
        } else if (i < n_int + n_flt) {
            a.flts[i - n_int] = 0.f;
        } else {
            const size_t r = i - n_int - n_flt;
            perm[r] = (int)(r % a.P);
            if (r % a.P == 0) subisland_num[r / a.P] = nsub;
        }
    }
}

int check_arch(const speo_archipelago *a, const void *state, const char *who)
{
    if (!a || !state || (reinterpret_cast<uintptr_t>(state) & 15)) return fail(SPEO_ERR_INVALID_ARG, "%s: state", who);
    if (a->n_islands < 1 || a->island_size < kMinSubisland || a->island_size >= (1 << 30) || a->dim < 1 ||
        a->dim > SPEO_MAX_DIM || a->ld < a->dim || a->migration_size < 1 || a->migration_size > a->island_size ||
        a->buffer_capacity < 1 || a->buffer_capacity > kMaxCap || a->buffer_capacity > a->island_size ||
        a->buffer_policy < SPEO_BUFFER_ONLINE_CLUSTER || a->buffer_policy > SPEO_BUFFER_LIFO ||
        a->regroup_option < SPEO_REGROUP_STATIC_ORDERED || a->regroup_option > SPEO_REGROUP_DYNAMIC_RANDOM ||
        !(a->migration_rate >= 0.f && a->migration_rate <= 1.f))
        return fail(SPEO_ERR_INVALID_ARG, "%s: bad archipelago description", who);
    return SPEO_OK;
}

Arch make_arch(const speo_archipelago *a, void *state)
{
    Arch r;
    r.N = a->n_islands;
    r.P = a->island_size;
    r.D = a->dim;
    r.ld = a->ld;
    r.C = a->buffer_capacity;
    r.k = a->migration_size;
    r.policy = a->buffer_policy;
    r.regroup = a->regroup_option;
    r.rate = a->migration_rate;
    r.key = make_uint2((uint32_t)a->seed, (uint32_t)(a->seed >> 32));
    r.istride = istride_of(*a);
    r.fstride = fstride_of(*a);
    r.ints = static_cast<int *>(state);
    r.flts = reinterpret_cast<float *>(r.ints + (size_t)r.N * r.istride);
    return r;
}

}  // namespace
}  // namespace speo

using namespace speo;

extern "C" size_t speo_archipelago_state_bytes(const speo_archipelago *a)
{
    if (!a || a->n_islands < 1 || a->buffer_capacity < 1 || a->dim < 1) return 0;
    return 4 * (size_t)a->n_islands * (size_t)(istride_of(*a) + fstride_of(*a));
}

extern "C" int speo_archipelago_init(const speo_archipelago *a, void *d_state, int32_t *d_perm,
                                     int32_t *d_subisland_num, int subisland_num, void *stream)
{
    if (int e = check_arch(a, d_state, "speo_archipelago_init")) return e;
    if (!d_perm || !d_subisland_num || subisland_num < 1 || subisland_num > a->island_size)
        return fail(SPEO_ERR_INVALID_ARG, "speo_archipelago_init: bad arguments");
    const Arch r = make_arch(a, d_state);
    k_mig_init<<<2 * sm_count(), kThreads, 0, static_cast<cudaStream_t>(stream)>>>(r, d_perm, d_subisland_num,
                                                                                    subisland_num);
    return check_launch("k_mig_init");
}

extern "C" int speo_migrate_out(const speo_archipelago *a, void *d_state, float *pop, float *fit, int32_t *d_perm,
                                int32_t *d_subisland_num, uint32_t generation, void *stream)
{
    if (int e = check_arch(a, d_state, "speo_migrate_out")) return e;
    if (!pop || !fit || !d_perm || !d_subisland_num) return fail(SPEO_ERR_INVALID_ARG, "speo_migrate_out: null pointer");
    k_mig_out<<<a->n_islands, kThreads, 0, static_cast<cudaStream_t>(stream)>>>(make_arch(a, d_state), pop, fit, d_perm,
                                                                                d_subisland_num, generation);
    return check_launch("k_mig_out");
}

extern "C" int speo_migrate_in(const speo_archipelago *a, void *d_state, const float *pop, const float *fit,
                               uint32_t generation, void *stream)
{
    if (int e = check_arch(a, d_state, "speo_migrate_in")) return e;
    if (!pop || !fit) return fail(SPEO_ERR_INVALID_ARG, "speo_migrate_in: null pointer");
    const Arch r = make_arch(a, d_state);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    k_mig_deliver<<<a->n_islands, kThreads, 0, st>>>(r, pop, fit, generation);
    if (int e = check_launch("k_mig_deliver")) return e;
    k_mig_advance<<<(a->n_islands + 255) / 256, 256, 0, st>>>(r);
    return check_launch("k_mig_advance");
}
