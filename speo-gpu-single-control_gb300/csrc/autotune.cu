// autotune.cu -- the library's own tile-shape tuner for the fused generation kernels.
//
// The reference fixes its launch shapes (CUDA_EA_library/kernel_CEC2014_CUDA.cu:56-73: blocks of
// 32 x 16 threads over P / 16 rows; kernel_DE_CUDA.cu:48-62). Here the number of rows one block of
// the fused generation (k_generation, k_generation_mixed) takes at once is chosen by measurement:
// each candidate tile height is timed on the caller's own segment table (scratch buffers of the
// same shape, the candidate's own work plan, a few generations after two warm-up ones), the
// fastest is kept, and the choice is cached per shape bucket so that later tables of a similar
// shape take it without timing. Every candidate computes the same rows bit for bit (the draws are
// functions of seed, row and generation only), so the choice changes the speed alone.
//
// Bucket of a table: (device, column classes of the smallest and largest D, log2 of the rows,
// log2 of the largest island, log2 of the number of segments, the candidate list).
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "host.h"

namespace speo {
namespace {

constexpr int kMaxCand = 16;

int qclass(int D) { return D <= 32 ? 1 : D <= 64 ? 2 : D <= 128 ? 4 : 8; }
int ilog2(long long v)
{
    int r = 0;
    while (v > 1) { v >>= 1; ++r; }
    return r;
}

struct TuneKey {
    int dev, qlo, qhi, lg_rows, lg_pmax, lg_segs;
    std::vector<int> cand;
    bool operator<(const TuneKey &o) const
    {
        return std::tie(dev, qlo, qhi, lg_rows, lg_pmax, lg_segs, cand) <
               std::tie(o.dev, o.qlo, o.qhi, o.lg_rows, o.lg_pmax, o.lg_segs, o.cand);
    }
};
struct TuneEntry {
    int tile;
    std::vector<float> ms;  // per candidate (empty when the choice was set by the caller)
};
std::mutex g_tune_mu;
std::map<TuneKey, TuneEntry> g_tune;

struct Shape {
    long long rows;
    int ld, dim_lo, dim_hi, pmax;
};

int shape_of(const speo_segment *h, int n, Shape *out)
{
    Shape s{0, 0, 1 << 30, 0, 0};
    for (int i = 0; i < n; ++i) {
        if (h[i].pop_size < 1 || h[i].dim < 1 || h[i].dim > SPEO_MAX_DIM || h[i].ld < h[i].dim || h[i].row0 < 0)
            return fail(SPEO_ERR_INVALID_ARG, "speo_autotune_tile_rows: segment %d is malformed", i);
        const long long end = h[i].row0 + h[i].pop_size;
        if (end > s.rows) s.rows = end;
        if (h[i].ld > s.ld) s.ld = h[i].ld;
        if (h[i].dim < s.dim_lo) s.dim_lo = h[i].dim;
        if (h[i].dim > s.dim_hi) s.dim_hi = h[i].dim;
        if (h[i].pop_size > s.pmax) s.pmax = h[i].pop_size;
    }
    *out = s;
    return SPEO_OK;
}

int key_of(const speo_segment *h, int n, const int *cand, int n_cand, TuneKey *k, Shape *sh)
{
    if (!h || n < 1 || !cand || n_cand < 1 || n_cand > kMaxCand)
        return fail(SPEO_ERR_INVALID_ARG, "speo_autotune: bad arguments (1 to %d candidates)", kMaxCand);
    for (int c = 0; c < n_cand; ++c)
        if (cand[c] < 1 || cand[c] > 1024)
            return fail(SPEO_ERR_INVALID_ARG, "speo_autotune: candidate tile %d outside [1, 1024]", cand[c]);
    if (int e = shape_of(h, n, sh)) return e;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        dev = -1;  // no device: only cached or set choices can be answered
    }
    k->dev = dev;
    k->qlo = qclass(sh->dim_lo);
    k->qhi = qclass(sh->dim_hi);
    k->lg_rows = ilog2(sh->rows);
    k->lg_pmax = ilog2(sh->pmax);
    k->lg_segs = ilog2(n);
    k->cand.assign(cand, cand + n_cand);
    return SPEO_OK;
}

// Times `reps` generations of one candidate's plan (after two warm-up generations) on scratch
// buffers; *ms = milliseconds per generation.
int time_candidate(const speo_segment *d_segs, const speo_segment *h_segs, int n_segs, const Shape &sh, int tile,
                   float *pop_a, float *pop_b, float *fit_a, float *fit_b, uint32_t *gen, speo_work_item *d_items,
                   int reps, cudaStream_t st, cudaEvent_t e0, cudaEvent_t e1, float *ms)
{
    int n = 0;
    if (int e = speo_plan_work(h_segs, n_segs, tile, nullptr, 0, &n)) return e;
    std::vector<speo_work_item> items((size_t)n);
    if (int e = speo_plan_work(h_segs, n_segs, tile, items.data(), n, &n)) return e;
    if (int e = check_cuda(cudaMemcpyAsync(d_items, items.data(), sizeof(speo_work_item) * (size_t)n,
                                           cudaMemcpyHostToDevice, st),
                           "autotune: items"))
        return e;
    if (int e = check_cuda(cudaMemsetAsync(gen, 0, 2 * sizeof(uint32_t), st), "autotune: counter")) return e;
    if (int e = speo_init_population(d_segs, n_segs, d_items, n, pop_a, st)) return e;
    if (int e = speo_evaluate(d_segs, d_items, n, sh.dim_lo, sh.dim_hi, pop_a, fit_a, st)) return e;
    float *pa = pop_a, *pb = pop_b, *fa = fit_a, *fb = fit_b;
    for (int r = -2; r < reps; ++r) {
        if (r == 0 && check_cuda(cudaEventRecord(e0, st), "autotune: event")) return SPEO_ERR_CUDA;
        if (int e = speo_generation(d_segs, d_items, n, sh.dim_lo, sh.dim_hi, pa, fa, pb, fb, gen, 0, nullptr, nullptr,
                                    st))
            return e;
        std::swap(pa, pb);
        std::swap(fa, fb);
    }
    if (int e = check_cuda(cudaEventRecord(e1, st), "autotune: event")) return e;
    if (int e = check_cuda(cudaEventSynchronize(e1), "autotune: sync")) return e;
    float t = 0.f;
    if (int e = check_cuda(cudaEventElapsedTime(&t, e0, e1), "autotune: elapsed")) return e;
    *ms = t / (float)reps;
    return SPEO_OK;
}

}  // namespace
}  // namespace speo

using namespace speo;

extern "C" int speo_autotune_set_tile_rows(const speo_segment *h_segs, int n_segs, const int *candidates, int n_cand,
                                           int tile)
{
    TuneKey k;
    Shape sh;
    if (int e = key_of(h_segs, n_segs, candidates, n_cand, &k, &sh)) return e;
    if (tile < 1 || tile > 1024) return fail(SPEO_ERR_INVALID_ARG, "speo_autotune_set_tile_rows: tile %d", tile);
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_tune[k] = TuneEntry{tile, {}};
    return SPEO_OK;
}

extern "C" int speo_autotune_tile_rows(const speo_segment *h_segs, int n_segs, const int *candidates, int n_cand,
                                       int reps, int *tile_out, float *ms_out, int *cached, void *stream)
{
    if (!tile_out) return fail(SPEO_ERR_INVALID_ARG, "speo_autotune_tile_rows: tile_out is null");
    TuneKey k;
    Shape sh;
    if (int e = key_of(h_segs, n_segs, candidates, n_cand, &k, &sh)) return e;
    {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        auto it = g_tune.find(k);
        if (it != g_tune.end()) {
            *tile_out = it->second.tile;
            if (ms_out)
                for (int c = 0; c < n_cand; ++c) ms_out[c] = it->second.ms.empty() ? -1.f : it->second.ms[(size_t)c];
            if (cached) *cached = 1;
            return SPEO_OK;
        }
    }
    if (cached) *cached = 0;
    if (k.dev < 0) return fail(SPEO_ERR_CUDA, "speo_autotune_tile_rows: no device to time the candidates on");
    if (reps < 1 || reps > 1000) return fail(SPEO_ERR_INVALID_ARG, "speo_autotune_tile_rows: reps %d", reps);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // scratch: the segment table, two population and fitness buffers, the counter, the work items
    int max_items = 0;
    for (int c = 0; c < n_cand; ++c) {
        int n = 0;
        if (int e = speo_plan_work(h_segs, n_segs, candidates[c], nullptr, 0, &n)) return e;
        if (n > max_items) max_items = n;
    }
    const size_t pop_bytes = sizeof(float) * (size_t)sh.rows * (size_t)sh.ld;
    const size_t fit_bytes = sizeof(float) * (size_t)sh.rows;
    const size_t seg_bytes = sizeof(speo_segment) * (size_t)n_segs;
    const size_t item_bytes = sizeof(speo_work_item) * (size_t)max_items;
    auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const size_t total = up(seg_bytes) + 2 * up(pop_bytes) + 2 * up(fit_bytes) + up(8) + up(item_bytes);
    uint8_t *scratch = nullptr;
    if (int e = check_cuda(cudaMalloc(&scratch, total), "autotune: scratch")) return e;
    uint8_t *p = scratch;
    auto take = [&](size_t b) { uint8_t *q = p; p += up(b); return q; };
    speo_segment *d_segs = reinterpret_cast<speo_segment *>(take(seg_bytes));
    float *pop_a = reinterpret_cast<float *>(take(pop_bytes)), *pop_b = reinterpret_cast<float *>(take(pop_bytes));
    float *fit_a = reinterpret_cast<float *>(take(fit_bytes)), *fit_b = reinterpret_cast<float *>(take(fit_bytes));
    uint32_t *gen = reinterpret_cast<uint32_t *>(take(8));
    speo_work_item *d_items = reinterpret_cast<speo_work_item *>(take(item_bytes));
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int e = check_cuda(cudaEventCreate(&e0), "autotune: event");
    if (!e) e = check_cuda(cudaEventCreate(&e1), "autotune: event");
    if (!e) e = check_cuda(cudaMemsetAsync(scratch, 0, total, st), "autotune: clear");
    if (!e) e = check_cuda(cudaMemcpyAsync(d_segs, h_segs, seg_bytes, cudaMemcpyHostToDevice, st), "autotune: segments");
    std::vector<float> ms((size_t)n_cand, 0.f);
    int best = 0;
    for (int c = 0; !e && c < n_cand; ++c) {
        e = time_candidate(d_segs, h_segs, n_segs, sh, candidates[c], pop_a, pop_b, fit_a, fit_b, gen, d_items, reps,
                           st, e0, e1, &ms[(size_t)c]);
        if (!e && ms[(size_t)c] < ms[(size_t)best]) best = c;
    }
    const int es = check_cuda(cudaStreamSynchronize(st), "autotune: sync");
    if (!e) e = es;
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(scratch);
    if (e) return e;
    *tile_out = candidates[best];
    if (ms_out)
        for (int c = 0; c < n_cand; ++c) ms_out[c] = ms[(size_t)c];
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_tune[k] = TuneEntry{candidates[best], ms};
    return SPEO_OK;
}
