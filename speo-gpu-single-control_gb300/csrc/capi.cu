// capi.cu -- library control entry points and the host helpers shared by the other
// translation units: per-thread error text and stream, API_CheckCUDAError, work planning.
#include <cstdarg>
#include <cstdio>
#include <cstring>

#include "host.h"

namespace speo {
namespace {
thread_local char t_msg[512] = "";
thread_local int t_sticky = SPEO_OK;  // first failure since the last API_CheckCUDAError
thread_local cudaStream_t t_stream = nullptr;
int g_sm_count[64] = {0};
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
    const unsigned bits = speo_deverr_de_ops() | speo_deverr_objective() | speo_deverr_generation() | speo_deverr_tc() |
                          speo_deverr_resident() | speo_deverr_surrogate() | speo_deverr_mlp() |
                          speo_deverr_dropin_step();
    if (bits & 0x80000000u) return fail(SPEO_ERR_CUDA, "speo_device_error_bits: cannot read the device flags");
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
