// capi.cu -- library control entry points and the host helpers shared by the other
// translation units: per-thread error text and stream, API_CheckCUDAError, work planning.
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "host.h"

namespace speo {
namespace {
thread_local char t_msg[512] = "";
thread_local int t_sticky = SPEO_OK;  // first failure since the last API_CheckCUDAError
thread_local cudaStream_t t_stream = nullptr;
int g_sm_count[64] = {0};

// The device error words of every translation unit, gathered (read and cleared) by one kernel
// into a mapped host word: one launch and one synchronisation per read instead of a copy per unit.
constexpr int kErrUnits = 10;
struct DevErr {
    bool ready = false;
    unsigned int **d_addrs = nullptr;
    unsigned int *h_out = nullptr, *d_out = nullptr;
};
DevErr g_deverr[64];
std::mutex g_deverr_mu;

__global__ void k_gather_errors(unsigned int *const *addrs, int n, unsigned int *out)
{
    unsigned int v = 0;
    for (int i = 0; i < n; ++i) v |= atomicExch(addrs[i], 0u);
    *out = v;
}

int deverr_state(DevErr **out)
{
    int dev = 0;
    if (int e = check_cuda(cudaGetDevice(&dev), "speo_device_error_bits: device")) return e;
    if (dev < 0 || dev >= 64) return fail(SPEO_ERR_CUDA, "speo_device_error_bits: device %d", dev);
    std::lock_guard<std::mutex> lock(g_deverr_mu);
    DevErr &s = g_deverr[dev];
    if (!s.ready) {
        void *addrs[kErrUnits] = {speo_deverr_de_ops(),  speo_deverr_objective(),  speo_deverr_generation(),
                                  speo_deverr_tc(),      speo_deverr_resident(),   speo_deverr_surrogate(),
                                  speo_deverr_mlp(),     speo_deverr_dropin_step(), speo_deverr_objective_multi(),
                                  speo_deverr_resident_tc()};
        for (void *a : addrs)
            if (!a) return fail(SPEO_ERR_CUDA, "speo_device_error_bits: cannot locate the device flags");
        if (int e = check_cuda(cudaMalloc(reinterpret_cast<void **>(&s.d_addrs), sizeof addrs), "deverr: alloc"))
            return e;
        if (int e = check_cuda(cudaMemcpy(s.d_addrs, addrs, sizeof addrs, cudaMemcpyHostToDevice), "deverr: copy"))
            return e;
        if (int e = check_cuda(cudaHostAlloc(reinterpret_cast<void **>(&s.h_out), sizeof(unsigned int),
                                             cudaHostAllocMapped),
                               "deverr: host word"))
            return e;
        if (int e = check_cuda(cudaHostGetDevicePointer(reinterpret_cast<void **>(&s.d_out), s.h_out, 0),
                               "deverr: mapped word"))
            return e;
        s.ready = true;
    }
    *out = &s;
    return SPEO_OK;
}
}  // namespace

int fail(int status, const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(t_msg, sizeof t_msg, fmt, ap);
    va_end(ap);
    if (t_sticky == SPEO_OK) t_sticky = status;
    return status;
}

int check_cuda(cudaError_t e, const char *what)
{
    if (e == cudaSuccess) return SPEO_OK;
    return fail(SPEO_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

int check_launch(const char *what) { return check_cuda(cudaGetLastError(), what); }

cudaStream_t api_stream() { return t_stream; }

int sticky_status() { return t_sticky; }

int sm_count()
{
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) dev = 0;
    if (!g_sm_count[dev]) {
        int n = 0;
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        g_sm_count[dev] = n > 0 ? n : 1;
    }
    return g_sm_count[dev];
}

}  // namespace speo

using namespace speo;

extern "C" int speo_set_stream(void *stream)
{
    t_stream = static_cast<cudaStream_t>(stream);
    return SPEO_OK;
}

extern "C" const char *speo_last_error(void) { return t_msg; }

extern "C" const char *speo_version(void) { return "speo_gb300 0.1 (sm_103a)"; }

extern "C" int speo_device_error_bits(uint32_t *bits_out)
{
    if (int e = check_cuda(cudaDeviceSynchronize(), "speo_device_error_bits: sync")) return e;
    DevErr *s = nullptr;
    if (int e = deverr_state(&s)) return e;
    *const_cast<volatile unsigned int *>(s->h_out) = 0u;
    k_gather_errors<<<1, 1>>>(s->d_addrs, kErrUnits, s->d_out);
    if (int e = check_launch("k_gather_errors")) return e;
    if (int e = check_cuda(cudaDeviceSynchronize(), "speo_device_error_bits: sync")) return e;
    const unsigned bits = *const_cast<volatile unsigned int *>(s->h_out);
    if (bits_out) *bits_out = bits;
    return SPEO_OK;
}

// CUDA_EA_library/kernel_EA_CUDA.cu:64-69 (+ __cudaCheckError :39-62): last launch error, then a
// device-wide sync; here the result is returned instead of exit(-1), and the device error
// flags and the first host-side failure since the previous call are reported too.
extern "C" int API_CheckCUDAError(void)
{
    const int sticky = t_sticky;
    t_sticky = SPEO_OK;
    if (int e = check_cuda(cudaGetLastError(), "API_CheckCUDAError")) { t_sticky = SPEO_OK; return e; }
    if (int e = check_cuda(cudaDeviceSynchronize(), "API_CheckCUDAError: sync")) { t_sticky = SPEO_OK; return e; }
    uint32_t bits = 0;
    if (int e = speo_device_error_bits(&bits)) { t_sticky = SPEO_OK; return e; }
    if (bits) {
        fail(SPEO_ERR_DEVICE_FLAG, "API_CheckCUDAError: device error flags 0x%x", bits);
        t_sticky = SPEO_OK;
        return SPEO_ERR_DEVICE_FLAG;
    }
    return sticky;
}

extern "C" int speo_plan_work(const speo_segment *segs, int n_segs, int tile_rows, speo_work_item *items, int cap,
                              int *n_out)
{
    if (!segs || n_segs < 0 || tile_rows < 1 || !n_out || cap < 0)
        return fail(SPEO_ERR_INVALID_ARG, "speo_plan_work: bad arguments");
    int n = 0;
    for (int s = 0; s < n_segs; ++s) {
        const int P = segs[s].pop_size;
        if (P < 1) return fail(SPEO_ERR_INVALID_ARG, "speo_plan_work: segment %d has pop_size %d", s, P);
        // balanced tiles: ceil(P / tile_rows) tiles of nearly equal size
        const int nt = (P + tile_rows - 1) / tile_rows;
        for (int t = 0; t < nt; ++t) {
            const int a = (int)((long long)P * t / nt), b = (int)((long long)P * (t + 1) / nt);
            if (items && n < cap) {
                items[n].segment = s;
                items[n].first = a;
                items[n].count = b - a;
                items[n].pad = 0;
            }
            ++n;
        }
    }
    *n_out = n;
    if (items && n > cap) return fail(SPEO_ERR_INVALID_ARG, "speo_plan_work: %d items exceed capacity %d", n, cap);
    return SPEO_OK;
}

// ---- DE_CUDA::ConfigureEA (CUDA_EA_library/DE_CUDA.cc:89-118) ------------------------------------
namespace {

// Philox-4x32-10 on the host (Salmon et al., SC'11; the same rounds as the device copy).
void philox_host(const uint32_t ctr[4], uint32_t k0, uint32_t k1, uint32_t out[4])
{
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    for (int r = 0; r < 10; ++r) {
        if (r) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
        const uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
        const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0, n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        c0 = n0; c1 = (uint32_t)p1; c2 = n2; c3 = (uint32_t)p0;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

template <typename T, typename Info>
int configure_de(Info *h, int nsub, int island_size, T F, T CR, int strategy, int dynamic, uint64_t seed,
                 const char *who)
{
    if (!h || nsub < 1 || island_size < 1 || island_size % nsub || (dynamic != 0 && dynamic != 1) ||
        (!dynamic && (strategy < 0 || strategy > 8)))
        return speo::fail(SPEO_ERR_INVALID_ARG, "%s: bad arguments", who);
    for (int i = 0; i < nsub; ++i) {
        h[i].F = F;
        h[i].pop_size = island_size / nsub;
        if (dynamic) {
            const uint32_t ctr[4] = {(uint32_t)i, 0u, 0u, 6u};
            uint32_t w[4];
            philox_host(ctr, (uint32_t)seed, (uint32_t)(seed >> 32), w);
            h[i].CR = (w[0] & 1u) ? (T)0.9 : (T)0.1;
            h[i].strategy_ID = (w[1] & 1u) ? 6 : 4;
        } else {
            h[i].CR = CR;
            h[i].strategy_ID = strategy;
        }
    }
    return SPEO_OK;
}

}  // namespace

extern "C" int speo_configure_de_f32(speo_de_info_f32 *h, int nsub, int island_size, float F, float CR, int strategy,
                                     int dynamic, uint64_t seed)
{
    return configure_de<float>(h, nsub, island_size, F, CR, strategy, dynamic, seed, "speo_configure_de_f32");
}

extern "C" int speo_configure_de_f64(speo_de_info_f64 *h, int nsub, int island_size, double F, double CR,
                                     int strategy, int dynamic, uint64_t seed)
{
    return configure_de<double>(h, nsub, island_size, F, CR, strategy, dynamic, seed, "speo_configure_de_f64");
}
