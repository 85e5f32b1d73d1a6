// xorwow_capture.cu -- records cuRAND XORWOW streams in the reference's state layout.
// TEST INFRASTRUCTURE ONLY (built into oracle/lib/xorwow_capture.fatbin).
//
// The reference seeds one XORWOW state per (individual, lane) with
// curand_init(seed, individual*32 + lane, 0) (CUDA_EA_library/kernel_EA_CUDA.cu:85-89) and draws
// curand_uniform / curand_uniform_double from it (kernel_EA_CUDA.cu:104-117,
// kernel_DE_CUDA.cu:184-237). These kernels replay the first `len` uniforms of each state through
// the same device API, so the oracle can consume them in the reference's order.
#include <curand_kernel.h>

extern "C" __global__ void capture_uniform_f32(unsigned long long seed, int n_states, int len, float *out)
{
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= n_states) return;
    curandState s;
    curand_init(seed, id, 0, &s);
    for (int i = 0; i < len; ++i) out[(size_t)id * len + i] = curand_uniform(&s);
}

extern "C" __global__ void capture_uniform_f64(unsigned long long seed, int n_states, int len, double *out)
{
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= n_states) return;
    curandState s;
    curand_init(seed, id, 0, &s);
    for (int i = 0; i < len; ++i) out[(size_t)id * len + i] = curand_uniform_double(&s);
}
