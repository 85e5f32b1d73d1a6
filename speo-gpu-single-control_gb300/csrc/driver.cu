// driver.cu -- the reference's host generation loop, natively.
//
// DE_CUDA::Run (CUDA_EA_library/DE_CUDA.cc:200-216) calls, per generation,
// API_DE_GenerateNewPopulation, CEC2014_CUDA::EvaluateFitness (-> API_evaluateFitness) and
// API_DE_SelectSurvival, with a device synchronisation after each launch; the island driver then
// reads results back to the host (src/island_EA.cc:78-113). speo_de_run_f32 runs that loop on a
// private stream, ordered after the caller's stream (speo_de_run_f64: the same in FP64):
//   * when a sub-island fits a block, kStepGens generations per launch of the fused kernel
//     (dropin_step.cu, bit-identical to the three calls), each generation's fitness vector
//     collected in one of two device history buffers and copied to the host on a second stream
//     while the next launch runs;
//   * otherwise over this library's drop-in entry points, where blocks of kBlock generations
//     (each with its read-back of the fitness vector into pinned host memory) are captured once as
//     a CUDA graph and replayed, so the per-generation host cost is one graph launch per block
//     instead of a synchronisation per kernel. There the best-in-sub-island search is left out
//     of generations whose strategies do not read it, except the last one.
#include <vector>

#include "common.cuh"
#include "host.h"

namespace speo {
namespace {

constexpr int kBlock = 10;     // generations per captured graph (three-call path)
constexpr int kStepGens = 100;             // generations per fused launch (at most)
constexpr size_t kHistElems = 1u << 22;    // bound of one history buffer (16 MiB FP32, 32 MiB FP64)

struct DriverHistory {
    void *p = nullptr;
    size_t cap = 0;  // bytes
};
thread_local DriverHistory t_hist;

// The device history buffer of this host thread, grown on demand (the previous call has
// synchronised its stream, so nothing is using the old one).
template <typename T>
int history_buffer(size_t count, T **out)
{
    DriverHistory &h = t_hist;
    const size_t bytes = sizeof(T) * count;
    if (h.cap < bytes) {
        if (h.p) cudaFree(h.p);
        h.p = nullptr;
        h.cap = 0;
        if (int e = check_cuda(cudaMalloc(&h.p, bytes), "driver: history")) return e;
        h.cap = bytes;
    }
    *out = static_cast<T *>(h.p);
    return SPEO_OK;
}

struct DriverStream {
    cudaStream_t s = nullptr, copy = nullptr;   // generations; fitness read-backs
    cudaEvent_t in = nullptr, out = nullptr;
    cudaEvent_t made[2] = {nullptr, nullptr};    // history buffer b written
    cudaEvent_t read[2] = {nullptr, nullptr};    // history buffer b copied to the host
};
thread_local DriverStream t_drv;

int driver_stream(DriverStream **out)
{
    DriverStream &d = t_drv;
    if (!d.s) {
        if (int e = check_cuda(cudaStreamCreateWithFlags(&d.s, cudaStreamNonBlocking), "driver stream")) return e;
        if (int e = check_cuda(cudaEventCreateWithFlags(&d.in, cudaEventDisableTiming), "driver event")) return e;
        if (int e = check_cuda(cudaEventCreateWithFlags(&d.out, cudaEventDisableTiming), "driver event")) return e;
        if (int e = check_cuda(cudaStreamCreateWithFlags(&d.copy, cudaStreamNonBlocking), "driver stream")) return e;
        for (int b = 0; b < 2; ++b) {
            if (int e = check_cuda(cudaEventCreateWithFlags(&d.made[b], cudaEventDisableTiming), "driver event"))
                return e;
            if (int e = check_cuda(cudaEventCreateWithFlags(&d.read[b], cudaEventDisableTiming), "driver event"))
                return e;
        }
    }
    *out = &d;
    return SPEO_OK;
}

bool is_pinned(const void *p)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

// The drop-in entry points and the fused step of one precision.
inline int gen_call(speo_population_f32 c, speo_population_f32 p, int *b, speo_island_info ii, speo_de_info_f32 *info,
                    speo_rng_state *r, speo_problem_info_f32 pi, bool with_best)
{
    return dropin_generate_f32(c, p, b, ii, info, r, pi, with_best);
}
inline int gen_call(speo_population_f64 c, speo_population_f64 p, int *b, speo_island_info ii, speo_de_info_f64 *info,
                    speo_rng_state *r, speo_problem_info_f64 pi, bool with_best)
{
    return dropin_generate_f64(c, p, b, ii, info, r, pi, with_best);
}
inline void eval_call(float *f, float *x, const float *o, const float *m, const int *sh, int n, int d, int fid)
{
    API_evaluateFitness_f32(f, nullptr, nullptr, x, const_cast<float *>(o), const_cast<float *>(m),
                            const_cast<int *>(sh), nullptr, nullptr, nullptr, n, d, 0.f, fid);
}
inline void eval_call(double *f, double *x, const double *o, const double *m, const int *sh, int n, int d, int fid)
{
    API_evaluateFitness(f, nullptr, nullptr, x, const_cast<double *>(o), const_cast<double *>(m),
                        const_cast<int *>(sh), nullptr, nullptr, nullptr, n, d, 0.0, fid);
}
inline int sel_call(speo_population_f32 p, speo_population_f32 c, speo_island_info ii, speo_problem_info_f32 pi)
{
    return API_DE_SelectSurvival_f32(p, c, ii, pi);
}
inline int sel_call(speo_population_f64 p, speo_population_f64 c, speo_island_info ii, speo_problem_info_f64 pi)
{
    return API_DE_SelectSurvival(p, c, ii, pi);
}
inline bool step_fits(float *, const speo_island_info &ii, int dim, int fid)
{
    return dropin_step_fits_f32(ii.island_size, ii.subisland_num, dim, fid);
}
inline bool step_fits(double *, const speo_island_info &ii, int dim, int fid)
{
    return dropin_step_fits_f64(ii.island_size, ii.subisland_num, dim, fid);
}
inline int step_call(speo_population_f32 p, speo_population_f32 c, int *b, speo_island_info ii, speo_de_info_f32 *info,
                     speo_rng_state *r, speo_problem_info_f32 pi, const float *o, const float *m, int k, float *hist,
                     cudaStream_t st)
{
    return dropin_step_f32(p, c, b, ii, info, r, pi, o, m, k, hist, 0, st);
}
inline int step_call(speo_population_f64 p, speo_population_f64 c, int *b, speo_island_info ii, speo_de_info_f64 *info,
                     speo_rng_state *r, speo_problem_info_f64 pi, const double *o, const double *m, int k,
                     double *hist, cudaStream_t st)
{
    return dropin_step_f64(p, c, b, ii, info, r, pi, o, m, k, hist, 0, st);
}

template <typename T, typename Pop, typename Info, typename Prob>
int de_run(Pop pop, Pop cand, speo_rng_state *rng, speo_island_info ii, Info *d_info, int *d_best, Prob pi,
           const T *d_shift, const T *d_rot, const int *d_shuffle, int generations, T *h_fitness, int history,
           void *stream, const char *who)
{
    if (!pop.elements || !pop.fitness_value || !cand.elements || !cand.fitness_value || !rng || !d_info || !d_best ||
        !d_shift || !d_rot || !ii.permutated_index || generations < 0 || ii.island_size <= 0)
        return fail(SPEO_ERR_INVALID_ARG, "%s: bad arguments", who);
    if (generations == 0) return SPEO_OK;
    DriverStream *d = nullptr;
    if (int e = driver_stream(&d)) return e;
    const int n = ii.island_size;
    cudaStream_t caller = static_cast<cudaStream_t>(stream);
    if (int e = check_cuda(cudaEventRecord(d->in, caller), "driver: record")) return e;
    if (int e = check_cuda(cudaStreamWaitEvent(d->s, d->in, 0), "driver: wait")) return e;
    const cudaStream_t prev = api_stream();
    speo_set_stream(d->s);

    const bool fused = step_fits(static_cast<T *>(nullptr), ii, pi.dim, pi.function_ID);
    const bool hist = h_fitness && history;
    int e = SPEO_OK, done = 0;
    if (fused) {
        // two history buffers: launch i writes buffer i % 2 while the copy stream reads the other
        // one back, so the read-back of a block of generations overlaps the next block
        T *d_hist = nullptr;
        int per = kStepGens;  // generations per launch: the history of one launch within kHistElems
        if (hist) {
            const size_t cap = kHistElems / (size_t)n;
            per = cap < 1 ? 1 : cap < (size_t)kStepGens ? (int)cap : kStepGens;
            e = history_buffer(2 * (size_t)per * n, &d_hist);
        }
        for (int i = 0; !e && done < generations; done += per, ++i) {
            const int k = generations - done < per ? generations - done : per, b = i & 1;
            T *hb = hist ? d_hist + (size_t)b * per * n : nullptr;
            if (hist && i >= 2) e = check_cuda(cudaStreamWaitEvent(d->s, d->read[b], 0), "driver: wait");
            if (!e) e = step_call(pop, cand, d_best, ii, d_info, rng, pi, d_shift, d_rot, k, hb, d->s);
            if (!e && hist) {
                e = check_cuda(cudaEventRecord(d->made[b], d->s), "driver: record");
                if (!e) e = check_cuda(cudaStreamWaitEvent(d->copy, d->made[b], 0), "driver: wait");
                if (!e)
                    e = check_cuda(cudaMemcpyAsync(h_fitness + (size_t)done * n, hb, sizeof(T) * (size_t)k * n,
                                                   cudaMemcpyDeviceToHost, d->copy),
                                   "driver: fitness read-back");
                if (!e) e = check_cuda(cudaEventRecord(d->read[b], d->copy), "driver: record");
            }
        }
        if (hist) {  // the generation stream (synchronised below) also covers the last read-backs
            for (int b = 0; b < 2; ++b)
                if (int e2 = check_cuda(cudaStreamWaitEvent(d->s, d->read[b], 0), "driver: wait"); e2 && !e) e = e2;
        }
        if (!e && h_fitness && !hist)
            e = check_cuda(cudaMemcpyAsync(h_fitness, pop.fitness_value, sizeof(T) * (size_t)n,
                                           cudaMemcpyDeviceToHost, d->s),
                           "driver: fitness read-back");
    }

    // the three entry points in turn; generation g's fitness goes to h_fitness (+ g n with history).
    // The best-in-sub-island search runs where a sub-island's strategy reads it and in the last
    // generation, whose ids the calls leave behind (the search reads the population before that
    // generation's selection, so the last generation never runs inside a captured block).
    bool any_best = true;
    if (!e && !fused && generations >= 2 && ii.subisland_num > 0) {
        std::vector<Info> h_info((size_t)ii.subisland_num);
        e = check_cuda(cudaMemcpyAsync(h_info.data(), d_info, sizeof(Info) * h_info.size(), cudaMemcpyDeviceToHost,
                                       d->s),
                       "driver: DE info");
        if (!e) e = check_cuda(cudaStreamSynchronize(d->s), "driver: sync");
        if (!e) {
            any_best = false;
            for (const Info &x : h_info) any_best = any_best || strategy_uses_best(x.strategy_ID);
        }
    }
    int g_next = 0;
    auto one_generation = [&](bool in_graph) -> int {
        const bool with_best = any_best || (!in_graph && g_next == generations - 1);
        if (int e2 = gen_call(cand, pop, d_best, ii, d_info, rng, pi, with_best)) return e2;
        const int before = sticky_status();
        eval_call(cand.fitness_value, cand.elements, d_shift, d_rot, d_shuffle, n, pi.dim, pi.function_ID);
        if (sticky_status() != before) return sticky_status();
        if (int e2 = sel_call(pop, cand, ii, pi)) return e2;
        T *dst = h_fitness + (hist && !in_graph ? (size_t)g_next * n : 0);
        ++g_next;
        if (h_fitness)
            return check_cuda(cudaMemcpyAsync(dst, pop.fitness_value, sizeof(T) * (size_t)n,
                                              cudaMemcpyDeviceToHost, d->s),
                              "driver: fitness read-back");
        return SPEO_OK;
    };
    if (!fused && !hist && generations >= 2 * kBlock && (!h_fitness || is_pinned(h_fitness))) {
        cudaGraph_t g = nullptr;
        cudaGraphExec_t x = nullptr;
        e = check_cuda(cudaStreamBeginCapture(d->s, cudaStreamCaptureModeThreadLocal), "driver: begin capture");
        if (!e) {
            for (int i = 0; !e && i < kBlock; ++i) e = one_generation(true);
            const cudaError_t ce = cudaStreamEndCapture(d->s, &g);  // always ends the capture
            if (!e) e = check_cuda(ce, "driver: end capture");
        }
        if (!e) e = check_cuda(cudaGraphInstantiate(&x, g, 0), "driver: instantiate");
        for (; !e && done + kBlock < generations; done += kBlock)  // the last generation runs below
            e = check_cuda(cudaGraphLaunch(x, d->s), "driver: graph launch");
        const int es = check_cuda(cudaStreamSynchronize(d->s), "driver: sync");
        if (!e) e = es;
        if (x) cudaGraphExecDestroy(x);
        if (g) cudaGraphDestroy(g);
    }
    g_next = done;
    for (; !e && done < generations; ++done) e = one_generation(false);
    speo_set_stream(prev);
    const int es = check_cuda(cudaStreamSynchronize(d->s), "driver: sync");
    if (!e) e = es;
    if (!e) e = check_cuda(cudaEventRecord(d->out, d->s), "driver: record");
    if (!e) e = check_cuda(cudaStreamWaitEvent(caller, d->out, 0), "driver: wait");
    return e;
}

}  // namespace
}  // namespace speo

using namespace speo;

extern "C" int speo_de_run_f32(speo_population_f32 pop, speo_population_f32 cand, speo_rng_state *rng,
                               speo_island_info ii, speo_de_info_f32 *d_info, int *d_best, speo_problem_info_f32 pi,
                               const float *d_shift, const float *d_rot, const int *d_shuffle, int generations,
                               float *h_fitness, int history, void *stream)
{
    return de_run<float>(pop, cand, rng, ii, d_info, d_best, pi, d_shift, d_rot, d_shuffle, generations, h_fitness,
                         history, stream, "speo_de_run_f32");
}

extern "C" int speo_de_run_f64(speo_population_f64 pop, speo_population_f64 cand, speo_rng_state *rng,
                               speo_island_info ii, speo_de_info_f64 *d_info, int *d_best, speo_problem_info_f64 pi,
                               const double *d_shift, const double *d_rot, const int *d_shuffle, int generations,
                               double *h_fitness, int history, void *stream)
{
    return de_run<double>(pop, cand, rng, ii, d_info, d_best, pi, d_shift, d_rot, d_shuffle, generations,
                          h_fitness, history, stream, "speo_de_run_f64");
}

