// host.h -- host-side helpers shared by the translation units of libspeo_gb300.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/speo_gb300.h"

namespace speo {

// Records `msg` as this host thread's last error and returns `status`.
int fail(int status, const char *fmt, ...);
// Checks a CUDA runtime result; on failure records it and returns SPEO_ERR_CUDA.
int check_cuda(cudaError_t e, const char *what);
// Checks the last launch error (no synchronisation).
int check_launch(const char *what);
// Stream of the group-1 (reference-shaped) entry points on this host thread.
cudaStream_t api_stream();
// First failure status recorded on this host thread since the last API_CheckCUDAError.
int sticky_status();
// Number of SMs of the current device (cached per device).
int sm_count();

// Opaque Philox state behind speo_rng_state* (SPEO_RNG_STATE_BYTES bytes).
struct RngState {
    uint32_t key0, key1;  // Philox key = seed
    uint32_t gen;         // generation counter, advanced by each generate launch
    uint32_t done;        // blocks finished in the current launch
    uint32_t pad[12];
};
static_assert(sizeof(RngState) == SPEO_RNG_STATE_BYTES, "rng state size");

// Mutable surrogate state kept on the device, so that captured generations replay correctly.
struct SurrDev {
    long long head, count;  // archive ring head and fill
    uint32_t step;          // Adam steps taken
    uint32_t done;          // blocks of the running Adam launch that have finished
    float c1, c2;           // bias corrections 1 - beta^t of the next step, t = step + 1
};
// Training batch drawn from the archive inside the gradient kernel: row i of the batch is archive
// slot philox({i/4, step, 0, 4}, key)[i%4] mod count (rows AX[slot][0..din), target AT[slot]).
struct MlpArchive {
    const float *AX, *AT;
    int lda;
    const SurrDev *st;
    uint32_t key0, key1;
};

// Surrogate MLP forward on the tensor cores (BF16 operands, FP32 accumulation), mlp_tc.cu.
// theta: W1 (h x din) | b1 | W2 (h x h) | b2 | w3 | b3; img: mlp_bf16_image_bytes(h) bytes of
// device scratch for the packed weights.
bool mlp_bf16_supported(int din, int h);
size_t mlp_bf16_image_bytes(int h);
int mlp_forward_bf16(const float *theta, int din, int h, const float *mu, const float *isig, const float *X,
                     long long n, int ldx, float *y, uint8_t *img, cudaStream_t st);
// Gradient of the mean squared error of one batch (n rows of X, targets T) on the tensor cores:
// chunk z of 128 rows writes its partial gradient vector to gpart + z * round_up(n_params, 4) (summed over
// chunks by the caller); the squared-error sum is added to *loss. Scratch: BF16 [features][rp]
// transposes of the layer inputs and deltas, dy [rp]; rp = batch rounded up to 128.
struct MlpTrainBufs {
    uint16_t *xnT, *h1T, *h2T, *dz2T, *dz1T;
    float *dy;
    long long rp;
};
// X/T: the batch rows, or null with `arch` set to draw them from the archive. pack_weights: refresh
// the BF16 weight images from theta first (the Adam kernel keeps them current between steps).
int mlp_grad_bf16(const float *theta, int din, int h, const float *mu, const float *isig, const float *X, int n,
                  int ldx, const float *T, const MlpArchive *arch, uint8_t *img, bool pack_weights,
                  const MlpTrainBufs &b, float *gpart, float *loss, cudaStream_t st);
// `generations` generations of the reference-shaped path in one launch (dropin_step.cu): best
// search, generate, evaluate and select, bit-identical to as many rounds of
// API_DE_GenerateNewPopulation_f32 + API_evaluateFitness_f32 + API_DE_SelectSurvival_f32.
// d_hist (generations x island_size, may be null) receives the fitness after each generation.
// pair_mode: 0 = two-block clusters per sub-island when 2 x sub-islands <= SMs, 1 = one block,
// 2 = two-block clusters (bit-identical to one block). Fits when a sub-island's rows, trials and
// M^T fit one block's shared memory.
bool dropin_step_fits_f32(int island_size, int subisland_num, int dim, int func);
// API_evaluateFitness(_f32) for ids 17-30 (objective_multi.cu); arguments already checked.
template <typename T>
int eval_ref_multi(T *fit, const T *X, const T *shift, const T *rot, const int *shuf, int P, int D, int func,
                   cudaStream_t st);

int dropin_step_f32(speo_population_f32 pop, speo_population_f32 cand, int *d_best, speo_island_info ii,
                    speo_de_info_f32 *d_info, speo_rng_state *rng, speo_problem_info_f32 pi, const float *shift,
                    const float *rot, int generations, float *d_hist, int pair_mode, cudaStream_t st);
// The same in FP64 (the reference's shipped precision).
bool dropin_step_fits_f64(int island_size, int subisland_num, int dim, int func);
int dropin_step_f64(speo_population_f64 pop, speo_population_f64 cand, int *d_best, speo_island_info ii,
                    speo_de_info_f64 *d_info, speo_rng_state *rng, speo_problem_info_f64 pi, const double *shift,
                    const double *rot, int generations, double *d_hist, int pair_mode, cudaStream_t st);

// API_DE_GenerateNewPopulation(_f32) with the best-in-sub-island search optional (de_ops.cu):
// with_best = false leaves d_best untouched.
int dropin_generate_f32(speo_population_f32 c, speo_population_f32 p, int *b, speo_island_info ii,
                        speo_de_info_f32 *info, speo_rng_state *r, speo_problem_info_f32 pi, bool with_best);
int dropin_generate_f64(speo_population_f64 c, speo_population_f64 p, int *b, speo_island_info ii,
                        speo_de_info_f64 *info, speo_rng_state *r, speo_problem_info_f64 pi, bool with_best);

// Byte offsets of the BF16 weight images inside `img`: W1 (h x 64), W2 (h x h), W2^T (h x h).
size_t mlp_img_w2_offset(int h);
size_t mlp_img_w2t_offset(int h);

}  // namespace speo

// Bit readers of the per-translation-unit device error words.
extern "C" void *speo_deverr_de_ops(void);
extern "C" void *speo_deverr_objective(void);
extern "C" void *speo_deverr_generation(void);
extern "C" void *speo_deverr_tc(void);
extern "C" void *speo_deverr_resident(void);
extern "C" void *speo_deverr_surrogate(void);
extern "C" void *speo_deverr_mlp(void);
extern "C" void *speo_deverr_dropin_step(void);
extern "C" void *speo_deverr_objective_multi(void);
extern "C" void *speo_deverr_resident_tc(void);
