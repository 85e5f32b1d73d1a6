/*
 * speo_gb300.h -- C ABI of the GB300 (sm_103a) island-model differential-evolution library.
 *
 * Two groups of entry points:
 *
 *  1. Drop-in replacements for the reference's CUDA_EA_library C entry points. Same names,
 *     same argument meaning, same by-value struct layouts, so a caller compiled against the
 *     reference headers links against libspeo_gb300.so unchanged:
 *        API_Initilize                 <- CUDA_EA_library/EA_CUDA.h:41-42   (kernel_EA_CUDA.cu:121-134)
 *        API_CheckCUDAError            <- CUDA_EA_library/EA_CUDA.h:43-44   (kernel_EA_CUDA.cu:64-69)
 *        API_DE_GenerateNewPopulation  <- CUDA_EA_library/DE_CUDA.cc:2-3    (kernel_DE_CUDA.cu:291-302)
 *        API_DE_SelectSurvival         <- CUDA_EA_library/DE_CUDA.cc:4-5    (kernel_DE_CUDA.cu:329-338)
 *        API_evaluateFitness           <- CUDA_EA_library/CEC2014_CUDA.h:35-37 (kernel_CEC2014_CUDA.cu:1672-1797)
 *     The unsuffixed names use `real = double`, the layout the reference ships with
 *     (CUDA_EA_library/config.h:31-34). The `_f32` names are the `real = float` layout
 *     (the reference's GPU_SINGLE_PRECISION build) and are the fast path.
 *     Differences from the reference, all deliberate:
 *       - the `curandState*` slot is an opaque Philox key/counter block (speo_rng_state);
 *         a caller's existing curandState allocation is large enough to hold it;
 *       - every individual gets a trial and a selection step, also when the population
 *         size is not a multiple of 16 (the reference leaves the last P mod 16 untouched);
 *       - the best-in-sub-island search honours the sub-island offset;
 *       - errors are returned as status codes, never exit(); no implicit device sync
 *         except in API_CheckCUDAError, which synchronises like the reference's.
 *
 *  2. GB300-native extensions (speo_*): a fused generate+evaluate+select generation kernel
 *     over a table of segments (islands / independent runs of uneven size), island-resident
 *     epochs, the on-device ring migration that replaces the reference's MPI exchange
 *     (src/migrate.cc:46-136), the reference's migration policy family over an archipelago of
 *     islands on one device (src/migrate.cc:34-186, src/buffer_manage.cc:36-313), the
 *     reference's DE_CUDA::Run loop as one call, its DE configuration modes, the tcgen05
 *     rotation GEMM in two-way split FP16 precision (power-of-two row scaling), FP64
 *     re-evaluation of each segment's best,
 *     and the online MLP surrogate.
 *
 * All pointers to population data are device pointers owned by the caller; no entry point
 * in group 1 allocates or frees device memory.
 */
#ifndef SPEO_GB300_H
#define SPEO_GB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define SPEO_API __attribute__((visibility("default")))
#else
#define SPEO_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------------------------ */
/* Status codes                                                                          */
/* ------------------------------------------------------------------------------------ */
#define SPEO_OK                 0
#define SPEO_ERR_INVALID_ARG    1  /* bad size, null pointer, misaligned stride ...      */
#define SPEO_ERR_CUDA           2  /* a CUDA runtime call failed (see speo_last_error)   */
#define SPEO_ERR_UNSUPPORTED    3  /* function id / strategy / shape not implemented     */
#define SPEO_ERR_DEVICE_FLAG    4  /* a kernel raised its device-side error flag         */

/* Device error flag bits (speo_device_error_bits) */
#define SPEO_DEVERR_REDRAW_LIMIT  0x1u  /* distinct-index rejection loop hit its bound      */
#define SPEO_DEVERR_BOUND_LIMIT   0x2u  /* reflection loop hit its bound (non-finite value) */
#define SPEO_DEVERR_WAIT_TIMEOUT  0x4u  /* a bounded device wait gave up                    */
#define SPEO_DEVERR_BAD_SEGMENT   0x8u  /* a segment descriptor failed the device check     */

/* Objective ids: 1..30 are the CEC2014 functions of the reference's dispatch
 * (kernel_CEC2014_CUDA.cu:1672-1797; CPU definitions CUDA_EA_library/CEC2014.cc), 9 being F9
 * (rotated Rastrigin, scale 0.0512). The reference has no GPU rotated sphere; it gets an id
 * outside the reference's 1..30 range. All return f(x) - f*. */
#define SPEO_FUNC_ROTATED_RASTRIGIN  9
#define SPEO_FUNC_ROTATED_SPHERE     31

/* DE strategy ids, as in DE_CUDA::GetParameters (CUDA_EA_library/DE_CUDA.cc:36-53). */
#define SPEO_DE_CURRENT_1        0
#define SPEO_DE_CURRENT_2        1
#define SPEO_DE_CURRENT_TO_BEST_1 2
#define SPEO_DE_CURRENT_TO_BEST_2 3
#define SPEO_DE_RAND_1           4
#define SPEO_DE_RAND_2           5
#define SPEO_DE_BEST_1           6
#define SPEO_DE_BEST_2           7
#define SPEO_DE_CURRENT_TO_RAND_1 8

#define SPEO_MAX_DIM          256  /* largest D any kernel accepts                          */
#define SPEO_RNG_STATE_BYTES   64  /* bytes the caller must provide behind speo_rng_state*  */

/* ------------------------------------------------------------------------------------ */
/* Reference-shaped by-value structs                                                     */
/* ------------------------------------------------------------------------------------ */
/* GPU_Population (CUDA_EA_library/EA_CUDA.h:21-25): rows of `np2` elements,
 * np2 = max(32, next_pow2(dim)) (EA_CUDA.cc:197-206), one fitness per row. */
typedef struct { double *elements; double *fitness_value; } speo_population_f64;
typedef struct { float  *elements; float  *fitness_value; } speo_population_f32;

/* GPU_IslandInfo (EA_CUDA.h:26-31). island_size = total rows on the device,
 * subisland_num partitions, permutated_index maps positions to rows. */
typedef struct { int island_size; int subisland_num; int *permutated_index; } speo_island_info;

/* DEInfo (EA_CUDA.h:33-38), one per sub-island, in device memory. */
typedef struct { double CR; double F; int strategy_ID; int pop_size; } speo_de_info_f64;
typedef struct { float  CR; float  F; int strategy_ID; int pop_size; } speo_de_info_f32;

/* ProblemInfo (config.h:48-59). */
typedef struct {
    int dim, function_ID, run_ID, max_base_FEs, seed, running_time, computing_time;
    double max_bound, min_bound;
} speo_problem_info_f64;
typedef struct {
    int dim, function_ID, run_ID, max_base_FEs, seed, running_time, computing_time;
    float max_bound, min_bound;
} speo_problem_info_f32;

/* Opaque Philox-4x32-10 key + generation counter, in device memory, at least
 * SPEO_RNG_STATE_BYTES bytes, 16-byte aligned. Replaces the reference's curandState array. */
typedef struct speo_rng_state speo_rng_state;

/* ------------------------------------------------------------------------------------ */
/* Group 1: drop-in entry points (real = double)                                         */
/* ------------------------------------------------------------------------------------ */
/* Replaces API_Initilize (EA_CUDA.h:41-42): seeds the Philox key from problem_info.seed,
 * resets the generation counter, and fills every row with x = lb + u*(ub-lb), u in (0,1]. */
SPEO_API int API_Initilize(speo_population_f64 d_population, speo_rng_state *d_rng,
                  speo_island_info island_info, speo_problem_info_f64 problem_info);

/* Replaces API_CheckCUDAError (EA_CUDA.h:43-44): cudaGetLastError + device sync + device
 * error flag; returns a status instead of calling exit(-1). */
SPEO_API int API_CheckCUDAError(void);

/* Replaces API_DE_GenerateNewPopulation (DE_CUDA.cc:2-3): per-sub-island best search
 * into d_best_individual_ID, then mutation + binomial crossover + reflection into d_candidate. */
SPEO_API int API_DE_GenerateNewPopulation(speo_population_f64 d_candidate, speo_population_f64 d_population,
                                 int *d_best_individual_ID, speo_island_info island_info,
                                 speo_de_info_f64 *d_DE_info, speo_rng_state *d_rng,
                                 speo_problem_info_f64 problem_info);

/* Replaces API_DE_SelectSurvival (DE_CUDA.cc:4-5): strict `<` greedy replacement per row. */
SPEO_API int API_DE_SelectSurvival(speo_population_f64 d_population, speo_population_f64 d_candidate,
                          speo_island_info island_info, speo_problem_info_f64 problem_info);

/* Replaces API_evaluateFitness (CEC2014_CUDA.h:35-37). d_rotated_data is the reference's
 * padded transposed matrix: d_rotated_data[k*problem_dim + j] = M[j][k] for k < np2
 * (rows k >= problem_dim zero), d_shift_data holds o in its first problem_dim entries,
 * rows of d_original_elements have np2 elements. Implemented ids: 1-30 (CEC2014) and 31
 * (rotated sphere). Ids 23-30 read one block per component: shift c at d_shift_data + c*np2,
 * matrix c at d_rotated_data + c*np2*problem_dim (CEC2014_CUDA.cc:160-281); ids 17-22, 29, 30
 * read d_shuffle_data (1-based, component c at + c*np2). The composition deltas are the
 * reference's fixed tables (the values CEC2014_CUDA.cc:336-390 puts in d_sigma). Scratch
 * arguments (shuffled, rotated, tmp_fitness, wi, sigma) are accepted and unused: each
 * component's rotation is fused with its reduction and the mixing, so no intermediate is
 * written. */
SPEO_API void API_evaluateFitness(double *d_fitness_value, double *d_shuffled_elements,
                         double *d_rotated_elements, double *d_original_elements,
                         double *d_shift_data, double *d_rotated_data, int *d_shuffle_data,
                         double *d_tmp_fitness, double *d_wi, double *d_sigma,
                         int pop_size, int problem_dim, double bias, int function_ID);

/* Group 1, real = float. */
SPEO_API int API_Initilize_f32(speo_population_f32 d_population, speo_rng_state *d_rng,
                      speo_island_info island_info, speo_problem_info_f32 problem_info);
SPEO_API int API_DE_GenerateNewPopulation_f32(speo_population_f32 d_candidate, speo_population_f32 d_population,
                                     int *d_best_individual_ID, speo_island_info island_info,
                                     speo_de_info_f32 *d_DE_info, speo_rng_state *d_rng,
                                     speo_problem_info_f32 problem_info);
SPEO_API int API_DE_SelectSurvival_f32(speo_population_f32 d_population, speo_population_f32 d_candidate,
                              speo_island_info island_info, speo_problem_info_f32 problem_info);
SPEO_API void API_evaluateFitness_f32(float *d_fitness_value, float *d_shuffled_elements,
                             float *d_rotated_elements, float *d_original_elements,
                             float *d_shift_data, float *d_rotated_data, int *d_shuffle_data,
                             float *d_tmp_fitness, float *d_wi, float *d_sigma,
                             int pop_size, int problem_dim, float bias, int function_ID);

/* The reference's host generation loop (DE_CUDA::Run, CUDA_EA_library/DE_CUDA.cc:200-216),
 * natively: `generations` x (API_DE_GenerateNewPopulation_f32, API_evaluateFitness_f32 on
 * (d_shift, d_rot, d_shuffle, problem_info.function_ID), API_DE_SelectSurvival_f32), with the same results
 * as those calls issued one by one. When a sub-island fits one block's shared memory, blocks of
 * generations run in one launch with the sub-island resident on chip; otherwise the three entry
 * points run in turn (replayed as a CUDA graph when h_fitness is pinned or null). h_fitness (may
 * be null): with history = 0, island_size floats that receive the last generation's fitness;
 * with history != 0, generations x island_size floats that receive every generation's fitness
 * (generation g at h_fitness + g * island_size). Runs on a private stream ordered after
 * `stream`. Synchronous: returns when the generations are done. d_DE_info is read at the start
 * of the call (on the three-call path its strategy set decides where the best-row search runs)
 * and must not change while the call runs. No counterpart function in the reference (it is the
 * reference's caller loop, as a library call). */
SPEO_API int speo_de_run_f32(speo_population_f32 d_population, speo_population_f32 d_candidate,
                             speo_rng_state *d_rng, speo_island_info island_info, speo_de_info_f32 *d_DE_info,
                             int *d_best_individual_ID, speo_problem_info_f32 problem_info, const float *d_shift,
                             const float *d_rotated, const int *d_shuffle, int generations, float *h_fitness,
                             int history, void *stream);
/* The same loop in FP64 (API_DE_GenerateNewPopulation, API_evaluateFitness, API_DE_SelectSurvival),
 * the precision the reference ships; h_fitness holds doubles. The fused launches keep one
 * sub-island per block. */
SPEO_API int speo_de_run_f64(speo_population_f64 d_population, speo_population_f64 d_candidate,
                             speo_rng_state *d_rng, speo_island_info island_info, speo_de_info_f64 *d_DE_info,
                             int *d_best_individual_ID, speo_problem_info_f64 problem_info, const double *d_shift,
                             const double *d_rotated, const int *d_shuffle, int generations, double *h_fitness,
                             int history, void *stream);

/* Per-sub-island DE parameters, as DE_CUDA::ConfigureEA (CUDA_EA_library/DE_CUDA.cc:89-118)
 * fills them before copying them to the device: `dynamic` = 0 ("constant") gives every
 * sub-island (CR, F, strategy); `dynamic` = 1 gives each sub-island CR in {0.1, 0.9} and strategy
 * in {4, 6}, chosen independently with probability 1/2 each, and F. pop_size = island_size /
 * subisland_num. The reference draws the choices from its host RNG (random.cc); here sub-island i
 * takes word 0 (CR) and word 1 (strategy) of Philox-4x32-10({i, 0, 0, 6}, seed), low bit. Host
 * arrays of subisland_num entries; nothing on the device. */
SPEO_API int speo_configure_de_f32(speo_de_info_f32 *h_info, int subisland_num, int island_size, float F, float CR,
                                   int strategy, int dynamic, uint64_t seed);
SPEO_API int speo_configure_de_f64(speo_de_info_f64 *h_info, int subisland_num, int island_size, double F, double CR,
                                   int strategy, int dynamic, uint64_t seed);

/* ------------------------------------------------------------------------------------ */
/* Library control                                                                       */
/* ------------------------------------------------------------------------------------ */
/* Stream used by the group-1 entry points of the calling host thread (default: legacy 0).
 * `stream` is a cudaStream_t. */
SPEO_API int speo_set_stream(void *stream);
/* Message of the last failing call on this host thread ("" if none). */
SPEO_API const char *speo_last_error(void);
/* Reads and clears the device error flag bits of the current device (synchronises). */
SPEO_API int speo_device_error_bits(uint32_t *bits_out);
/* Library version string. */
SPEO_API const char *speo_version(void);

/* ------------------------------------------------------------------------------------ */
/* Group 2: GB300-native extensions                                                      */
/* ------------------------------------------------------------------------------------ */
/* One segment = one island of a ring, or one independent run. Rows row0 .. row0+pop_size-1
 * of the population buffers, `ld` floats apart. The objective instance is (shift, rot):
 * rot is M^T, rot[k*ld_rot + j] = M[j][k]. Rows are addressed as global row indices, which
 * also key the Philox counters, so results do not depend on how segments are tiled. */
typedef struct {
    int64_t      row0;
    int32_t      pop_size;   /* P >= 4 */
    int32_t      dim;        /* 1 <= D <= SPEO_MAX_DIM */
    int32_t      ld;         /* row stride in floats, >= D, multiple of 4 */
    int32_t      func_id;    /* SPEO_FUNC_* */
    int32_t      strategy;   /* SPEO_DE_* */
    float        F, CR;
    float        lb, ub;     /* search bounds (reflection) */
    const float *shift;      /* device, round_up(D, 4) floats, 16-byte aligned, zero past D */
    const float *rot;        /* device, D rows of ld_rot floats, 16-byte aligned */
    int32_t      ld_rot;     /* >= D, multiple of 4 */
    int32_t      ring_next;  /* segment that receives this one's emigrants, -1 = none */
    uint64_t     seed;       /* Philox key */
    const int32_t *shuffle;  /* ids 17-22, 29, 30: device, 1-based shuffles; else unused (NULL) */
} speo_segment;
/* Ids 17-30 (CEC2014 hybrid and composition functions) carry one shift / matrix / shuffle per
 * component (5 for 23, 26-28; 3 for 24, 25, 29, 30; 1 for 17-22): component c's shift starts at
 * shift + c*ld_rot, its D rows of M^T at rot + c*dim*ld_rot, its shuffle at shuffle + c*ld_rot.
 * speo_evaluate evaluates them; the fused generation, epoch and tensor-core kernels flag them
 * (SPEO_DEVERR_BAD_SEGMENT / SPEO_ERR_UNSUPPORTED). */

#define SPEO_TILE_SIMT  64   /* largest work item of the CUDA-core kernels */
#define SPEO_TILE_TC   128   /* largest work item of the tcgen05 kernels   */

/* Work item: a tile of up to `tile_rows` consecutive rows of one segment. */
typedef struct { int32_t segment; int32_t first; int32_t count; int32_t pad; } speo_work_item;

/* Fills `items` (host array of capacity `cap`) with the tiles of `segs` (host copy) for
 * tiles of `tile_rows` rows; returns the number of items in *n_out. */
SPEO_API int speo_plan_work(const speo_segment *segs, int n_segs, int tile_rows,
                   speo_work_item *items, int cap, int *n_out);

/* Initial population of every segment: x = lb + u*(ub-lb), and gen counter untouched. */
SPEO_API int speo_init_population(const speo_segment *d_segs, int n_segs, const speo_work_item *d_items,
                         int n_items, float *pop, void *stream);

/* Fitness of every row of every segment (FP32 SIMT evaluation; work items of any size).
 * dim_lo/dim_hi bound the segments' D (they select which kernel variants are launched). */
SPEO_API int speo_evaluate(const speo_segment *d_segs, const speo_work_item *d_items, int n_items,
                  int dim_lo, int dim_hi, const float *pop, float *fit, void *stream);

/* Same, with the rotation on the tcgen05 tensor cores: each row y = x - o scaled by its own power
 * of two (largest |y_j| into [2^14, 2^15)) and M by one per instance, each split two ways into
 * FP16 (hi + lo, ~2^-22 relative residue), three products per K step (y_lo M_hi, y_hi M_lo,
 * y_hi M_hi), FP32 accumulation in tensor memory (as exact as an FP32 CUDA-core rotation: fitness
 * within 1e-5 relative of FP64 for the rotated Rastrigin and sphere), fused
 * unscale/shift/scale/objective/row-reduction epilogue (one
 * tile row per thread; the per-coordinate sums 9 and 31 packed two columns per operation, the
 * other rotated ids 1-7, 11-16 through the row accumulator). Ids 8, 10 (no rotation) and 17-30
 * (several matrices) are flagged (SPEO_DEVERR_BAD_SEGMENT) and skipped.
 * The population is one flat buffer of n_rows rows, `ld` floats apart, shared by all segments
 * (it is read with TMA tensor loads); tiles are up to SPEO_TILE_TC rows and D <= 128. One
 * persistent block per SM holds all 512 tensor-memory columns of its SM and more than half of
 * its shared memory while it runs. */
SPEO_API int speo_evaluate_tc(const speo_segment *d_segs, const speo_work_item *d_items, int n_items,
                     int dim_lo, int dim_hi, const float *pop, int64_t n_rows, int ld, float *fit,
                     void *stream);

/* One fused DE generation over all work items: for each target row, draw indices and
 * crossover mask from Philox(key=seed, ctr={block,row,gen,tag}), build the trial
 * (DE/<strategy>/bin + reflection), evaluate it, and write the winner of the strict-`<`
 * greedy selection into (pop_out, fit_out). Reads (pop_in, fit_in). *d_gen is read by every
 * block and advanced by one by the last block to finish (d_gen[1] is its scratch word; both
 * start at the caller's values, d_gen[1] = 0). Tiles have at most SPEO_TILE_SIMT rows.
 * `use_tc` must be 0 (the tensor-core generation is speo_generation_tc, which needs the flat
 * buffer's extent); 1 returns SPEO_ERR_UNSUPPORTED.
 * trial_out / trial_fit_out (may be NULL) receive every trial vector and its fitness. */
SPEO_API int speo_generation(const speo_segment *d_segs, const speo_work_item *d_items, int n_items,
                    int dim_lo, int dim_hi, const float *pop_in, const float *fit_in,
                    float *pop_out, float *fit_out, uint32_t *d_gen, int use_tc,
                    float *trial_out, float *trial_fit_out, void *stream);

/* `generations` fused DE generations of every segment in one launch, each island held in one
 * block's shared memory for the whole epoch (read from pop_in/fit_in once, written to
 * pop_out/fit_out once; in place is allowed). Bit-identical to `generations` calls of
 * speo_generation. Segments need P <= max_pop and D <= dim_hi with max_pop/dim_hi accepted by
 * speo_epoch_fits (P <= 512, D <= 64, and the island fits one block's shared memory); all
 * segments in one column class (D <= 32, or 32 < D <= 64). *d_gen advances by `generations`. */
SPEO_API int speo_epoch_fits(int max_pop, int dim_hi);
SPEO_API int speo_generation_epoch(const speo_segment *d_segs, int n_segs, int dim_lo, int dim_hi,
                                   int max_pop, const float *pop_in, const float *fit_in,
                                   float *pop_out, float *fit_out, uint32_t *d_gen, int generations,
                                   void *stream);
/* speo_generation_epoch with the block shape chosen explicitly: cluster = 1 runs one block per
 * island; cluster = 2 runs each island on a two-block cluster (each block holds a replica of the
 * island, computes half of the rows and writes them into both replicas through distributed
 * shared memory; one cluster barrier per generation), bit-identical to cluster = 1;
 * cluster = 0 picks 2 when there are SMs for two blocks per island and the replicas fit. */
SPEO_API int speo_generation_epoch_ex(const speo_segment *d_segs, int n_segs, int dim_lo, int dim_hi, int max_pop,
                                      const float *pop_in, const float *fit_in, float *pop_out, float *fit_out,
                                      uint32_t *d_gen, int generations, int cluster, void *stream);

/* The island-resident epoch with the rotation on the tcgen05 tensor cores (one block per island,
 * P <= 256, D <= 64, the rotated Rastrigin 9 and sphere 31; other segments are flagged with
 * SPEO_DEVERR_BAD_SEGMENT and left unchanged). Each generation builds the same trial rows as
 * speo_generation (same Philox counters, bit-identical), evaluates them with the split-FP16
 * product and epilogue of speo_evaluate_tc (bit-identical fitness per row) and selects with
 * strict `<`; `generations` such generations equal, row for row, speo_generation's trials +
 * speo_evaluate_tc + speo_select_rows repeated. Replaces DE_CUDA::Run's generation
 * (CUDA_EA_library/DE_CUDA.cc:200-216) with the rotation of kernel_CEC2014_CUDA.cu:147-181 on
 * the tensor cores. One block per SM holds all 512 tensor-memory columns of its SM while it
 * runs. speo_epoch_tc_fits: 1 when islands of max_pop rows and dimension dim_hi are supported. */
SPEO_API int speo_epoch_tc_fits(int max_pop, int dim_hi);
SPEO_API int speo_generation_epoch_tc(const speo_segment *d_segs, int n_segs, int dim_lo, int dim_hi, int max_pop,
                                      const float *pop_in, const float *fit_in, float *pop_out, float *fit_out,
                                      uint32_t *d_gen, int generations, void *stream);

/* The island loop of IslandEA::Execute (src/island_EA.cc:78-113) as one call: `generations`
 * generations of speo_generation_epoch_tc on the islands of d_segs (in place in pop / fit, rows
 * rows, P <= 256, D <= 64) and the ring migration of speo_ring_migrate (migrants rows, caller
 * staging of n_segs * migrants * (max_ld + 1) floats) after every generation count that is a
 * multiple of `interval`, counted from the start of the run: `first` is the number of generations
 * the run has already done. When every island's block can be resident at once (one block per SM:
 * n_segs <= the SM count) and migrants <= 32, the migrations run inside the launches (a cooperative
 * launch; each island sends its best rows through a staging area the library owns, the blocks meet
 * at a grid barrier with a bounded wait, and each island takes its predecessor's rows), one launch
 * for the whole call or, with h_fitness, four intervals per launch (the last launch at most 8
 * generations, so that little of the history copy is left after it); otherwise launches of up to
 * `interval` generations with speo_ring_migrate between them. h_fitness (may be null; pinned host
 * memory for the copies to overlap): generations x rows floats that receive every generation's
 * fitness (generation g of this call at h_fitness + g * rows), read back on a second stream while
 * the next launch runs. Runs on `stream`; synchronous (returns when the generations and copies are
 * done). The results equal speo_generation_epoch_tc + speo_ring_migrate called in the same order. */
SPEO_API int speo_island_run_tc(const speo_segment *d_segs, int n_segs, int dim_lo, int dim_hi, int max_pop,
                                float *pop, float *fit, long long rows, uint32_t *d_gen, int first, int generations,
                                int interval, int migrants, float *staging, int max_ld, float *h_fitness,
                                void *stream);
/* The same generations and migrations without read-back and without waiting: enqueued on `stream`
 * (asynchronous), for callers that keep the population on the device. */
SPEO_API int speo_island_epochs_tc(const speo_segment *d_segs, int n_segs, int dim_lo, int dim_hi, int max_pop,
                                   float *pop, float *fit, long long rows, uint32_t *d_gen, int first,
                                   int generations, int interval, int migrants, float *staging, int max_ld,
                                   void *stream);

/* The library's tile-shape tuner for speo_generation (k_generation / k_generation_mixed), in
 * place of the reference's fixed launch shapes (CUDA_EA_library/kernel_CEC2014_CUDA.cu:56-73,
 * kernel_DE_CUDA.cu:48-62). h_segs is a HOST copy of a segment table whose shift / rot pointers are
 * device pointers. Each of the n_cand candidate tile heights (rows per work item, 1 to 1024; at
 * most 16 candidates) is timed over `reps` generations (after two warm-up ones) on scratch
 * buffers of the table's shape (the call allocates and frees them; the caller's buffers are not
 * touched) with its own work plan; *tile_out receives the fastest, ms_out (may be null) the
 * milliseconds per generation of each candidate. The choice is cached per shape bucket (device,
 * column classes of the smallest and largest D, log2 of rows, of the largest island and of the
 * number of segments, candidate list): a later call with a table of the same bucket returns it
 * without timing (*cached = 1, ms_out as measured, or -1 for a choice that was set). Every
 * candidate gives the same rows bit for bit: the choice changes the speed alone. Synchronous.
 * No counterpart function in the reference. */
SPEO_API int speo_autotune_tile_rows(const speo_segment *h_segs, int n_segs, const int *candidates, int n_cand,
                                     int reps, int *tile_out, float *ms_out, int *cached, void *stream);
/* Sets the cached choice of the bucket of h_segs (and candidates) to `tile`, as if it had been
 * measured: later speo_autotune_tile_rows calls of that bucket return it without timing. Host
 * only (no device work). */
SPEO_API int speo_autotune_set_tile_rows(const speo_segment *h_segs, int n_segs, const int *candidates, int n_cand,
                                         int tile);

/* Ring migration: each segment's k best rows (by fitness, then row) replace the k worst
 * rows (by fitness, then row, from the worst) of segment ring_next. All emigrants are
 * chosen before any row is replaced. `staging` holds n_segs*k*(max ld + 1) floats. */
SPEO_API int speo_ring_migrate(const speo_segment *d_segs, int n_segs, int k, float *pop, float *fit,
                      float *staging, int max_ld, void *stream);

/* speo_ring_migrate without a caller staging buffer, for callers that cannot allocate device
 * memory themselves (for instance a plugin whose host process owns and pre-reserves all device
 * memory through its own allocator, or a loop that must not allocate once it has started).
 * No counterpart in the reference (its migration is host MPI, src/migrate.cc:46-136).
 * The staging lives in a fixed array of SPEO_NOALLOC_STAGING_FLOATS floats (4 MiB) inside the
 * library, held by every GPU that loads the library until the process exits;
 * n_segs * k * (max_ld + 1) beyond that is rejected with SPEO_ERR_INVALID_ARG. The function
 * allocates nothing. The array's device address belongs to the CUDA context that loaded the
 * library's module, so every call made outside stream capture looks it up (in the current
 * device's current context: after a device reset, or with a context the caller bound, the new
 * address is found), and a call during stream capture takes the address that the last call
 * outside capture found in the same context: make one call outside capture, on that device and
 * in that context, before capturing one (otherwise the captured call fails with
 * SPEO_ERR_INVALID_ARG). Every call shares the one array, each call writes every staging slot
 * it reads (nothing needs clearing), and calls that overlap on the GPU (other streams, other
 * threads) race on it. */
#define SPEO_NOALLOC_STAGING_FLOATS (1 << 20)
SPEO_API int speo_ring_migrate_noalloc(const speo_segment *d_segs, int n_segs, int k, float *pop,
                                       float *fit, int max_ld, void *stream);

/* ---- Archipelago migration policies (src/migrate.cc:34-186, src/buffer_manage.cc:36-313) ----
 * The reference runs one island per MPI rank and migrates through host buffers; here n_islands
 * islands share one device: island i is rows [i*island_size, (i+1)*island_size) of pop / fit
 * (ld floats apart), with its own sub-island permutation d_perm + i*island_size (island-local
 * rows, the drop-in permutated_index) and sub-island count d_subisland_num[i]. Per generation g
 * the caller runs its DE generation on every island, then speo_migrate_out when g % interval
 * == 0, then speo_migrate_in (the order of IslandEA::Execute, src/island_EA.cc:86-105).
 *  - destinations (dynamicConnect, migrate.cc:34-44): when an island's list is used up, every
 *    other island joins it with probability migration_rate, in island order;
 *  - migrate_in (SendEmigrations + CheckAndRecvEmigrations, migrate.cc:71-144): every island
 *    whose list is not used up sends migration_size distinct random rows (with fitness) to the
 *    head of its list and drops that head; each island takes the messages sent to it this
 *    generation in source-island order into its immigrant buffer (buffer_policy);
 *  - migrate_out (UpdateDestination + UpdatePopulation + RegroupIslands, migrate.cc:46-69,
 *    147-186): refill used-up lists, take the buffer's selection (OnlineCluster: every entry
 *    updated since the last selection; the others: up to migration_size) into distinct random
 *    rows, then regroup (regroup_option).
 * Draws (Philox-4x32-10 keyed by `seed`, in place of the reference's host rand() and partial
 * Fisher-Yates, random.cc:14-53), for island s at generation g:
 *   destination t joins:  u01(word 0 of philox({t, s, g, 7})) < migration_rate
 *   emigrant rows:        perm_{P}(philox({s, g, 0, 8}))[0 .. migration_size)
 *   import rows:          perm_{P}(philox({s, g, 0, 9}))[0 .. count)
 *   regroup size index:   (word 0 of philox({s, g, 0, 10}) * (max_index + 1)) >> 32
 *   regroup permutation:  perm_{P}(philox({s, g, 1, 10}))
 *   RandomSelect draw q:  (word 0 of philox({q, s, g, 11}) * buffer size) >> 32
 * perm_n(k)[x] is a 4-round Feistel network on 2h bits (h = max(1, ceil(ceil(log2 n) / 2))),
 * round r: (L, R) <- (R, L ^ (fmix32(R * 0x9E3779B1 ^ k_r) & (2^h - 1))), fmix32 the MurmurHash3
 * finaliser, walked until the value is below n. MPI's asynchronous delivery becomes delivery
 * in the generation the message is sent. */
#define SPEO_BUFFER_ONLINE_CLUSTER 0  /* OnlineCluster (buffer_manage.cc:36-131), the reference driver's buffer */
#define SPEO_BUFFER_BEST           1  /* BestSelect (:169-212): largest fitness first, as the reference's */
#define SPEO_BUFFER_RANDOM         2  /* RandomSelect (:214-245) */
#define SPEO_BUFFER_FIFO           3  /* FIFO (:247-278) */
#define SPEO_BUFFER_LIFO           4  /* LIFO (:280-313) */
#define SPEO_REGROUP_STATIC_ORDERED  0  /* static_and_ordered: no regroup */
#define SPEO_REGROUP_STATIC_RANDOM   1  /* new random permutation */
#define SPEO_REGROUP_DYNAMIC_ORDERED 2  /* new sub-island size 4 << U{0..log2(P/4)} */
#define SPEO_REGROUP_DYNAMIC_RANDOM  3  /* both (the reference's published runs) */
#define SPEO_ARCHIPELAGO_MAX_CAPACITY 64
typedef struct {
    int32_t  n_islands;        /* >= 1 */
    int32_t  island_size;      /* rows per island, >= 4, < 2^30 */
    int32_t  dim, ld;          /* 1 <= dim <= SPEO_MAX_DIM, ld >= dim */
    int32_t  migration_size;   /* rows per message, 1..island_size */
    int32_t  buffer_capacity;  /* 1..SPEO_ARCHIPELAGO_MAX_CAPACITY, <= island_size */
    int32_t  buffer_policy;    /* SPEO_BUFFER_* */
    int32_t  regroup_option;   /* SPEO_REGROUP_* */
    float    migration_rate;   /* [0, 1] */
    int32_t  reserved;         /* 0 */
    uint64_t seed;             /* Philox key of every draw */
} speo_archipelago;
/* Device bytes of the migration state (destination lists and immigrant buffers of every island). */
SPEO_API size_t speo_archipelago_state_bytes(const speo_archipelago *a);
/* Empty lists and buffers; d_perm = identity per island; d_subisland_num[i] = subisland_num. */
SPEO_API int speo_archipelago_init(const speo_archipelago *a, void *d_state, int32_t *d_perm,
                                   int32_t *d_subisland_num, int subisland_num, void *stream);
SPEO_API int speo_migrate_out(const speo_archipelago *a, void *d_state, float *pop, float *fit, int32_t *d_perm,
                              int32_t *d_subisland_num, uint32_t generation, void *stream);
SPEO_API int speo_migrate_in(const speo_archipelago *a, void *d_state, const float *pop, const float *fit,
                             uint32_t generation, void *stream);

/* ---- Online MLP surrogate (no counterpart in the reference) -------------------------------
 * din -> hidden -> hidden -> 1 with ReLU, FP32 parameters in one flat vector
 * (W1[h][din], b1[h], W2[h][h], b2[h], w3[h], b3), inputs scaled by in_scale, trained by Adam
 * (beta1 0.9, beta2 0.999, eps 1e-8) on the mean squared error of log(f + 1e-8) over batches
 * sampled from a ring-buffer archive of exact evaluations. The object owns its device memory. */
typedef struct speo_surrogate speo_surrogate;
SPEO_API int speo_surrogate_create(speo_surrogate **out, int din, int hidden, long long archive_cap, int batch,
                                   float lr, float in_scale, uint64_t seed);
SPEO_API int speo_surrogate_destroy(speo_surrogate *s);
SPEO_API int speo_surrogate_params(speo_surrogate *s, float **d_theta, float **d_grad, int *n_params);
SPEO_API int speo_surrogate_forward(speo_surrogate *s, const float *X, int n, int ldx, float *y, void *stream);
/* The same forward pass on the tcgen05 tensor cores: inputs standardised in FP32 and rounded to
 * BF16, weights and hidden activations in BF16, FP32 accumulation and head. Takes din <= 64 and
 * hidden 64, 128 or 256 (SPEO_ERR_UNSUPPORTED otherwise). speo_surrogate_generation screens with
 * this pass whenever the shape allows it. */
SPEO_API int speo_surrogate_forward_bf16(speo_surrogate *s, const float *X, long long n, int ldx, float *y,
                                         void *stream);
/* Gradient of the batch loss on the tcgen05 tensor cores into the gradient buffer: BF16 operands
 * (standardised inputs, weights, hidden activations and back-propagated deltas), FP32
 * accumulation. The weight gradients are sums over 128-row chunks added in a fixed order, so the
 * result is deterministic. Same shapes as speo_surrogate_forward_bf16. */
SPEO_API int speo_surrogate_grad_bf16(speo_surrogate *s, const float *X, int n, int ldx, const float *T,
                                      float *loss_out, void *stream);
/* Which passes run on the tensor cores in speo_surrogate_generation / speo_surrogate_train:
 * SPEO_SURROGATE_BF16_SCREEN (screening forward) and SPEO_SURROGATE_BF16_TRAIN (training
 * gradient); 0 = FP32 CUDA-core passes throughout. Default: both where the shape allows. */
#define SPEO_SURROGATE_BF16_SCREEN 1
#define SPEO_SURROGATE_BF16_TRAIN 2
SPEO_API int speo_surrogate_set_mode(speo_surrogate *s, int mode);
/* Gradient of the batch MSE w.r.t. theta into the object's gradient buffer; mean loss out. */
SPEO_API int speo_surrogate_grad(speo_surrogate *s, const float *X, int n, int ldx, const float *T,
                                 float *loss_out, void *stream);
SPEO_API int speo_surrogate_adam_step(speo_surrogate *s, void *stream);
/* Standardise the MLP's inputs by the per-dimension mean and standard deviation of `rows` rows of
 * pop (stride ld) from now on (until then x' = x * in_scale). speo_surrogate_generation calls it
 * with its parents every generation, so the network sees the population's region at unit scale. */
SPEO_API int speo_surrogate_standardize(speo_surrogate *s, const float *pop, long long rows, int ld,
                                        void *stream);
SPEO_API int speo_surrogate_archive_append(speo_surrogate *s, const float *X, int n, int ldx, const float *f,
                                           void *stream);
SPEO_API int speo_surrogate_train(speo_surrogate *s, int steps, float *loss_out, void *stream);
/* k trial vectors per target: trial t of row r is written to T[(r*k + t)*ld ...]; its donor and
 * crossover draws use Philox tags (1 | (t+1) << 8) and (2 | (t+1) << 8). */
SPEO_API int speo_make_trials(const speo_segment *d_segs, const speo_work_item *d_items, int n_items,
                              int dim_hi, int k, const float *pop, const float *fit, float *T,
                              const uint32_t *d_gen, void *stream);
/* One screened generation over a flat population (rows x ld): k trials per target, the MLP
 * picks one (an `explore` fraction of targets, chosen by Philox, takes a uniformly drawn trial
 * instead, so the archive also holds unbiased labels), exact evaluation, strict-`<` selection
 * into (pop_out, fit_out), archive append (the first call also archives the parents),
 * `train_steps` Adam steps; *d_gen advances by one. */
SPEO_API int speo_surrogate_generation(speo_surrogate *s, const speo_segment *d_segs,
                                       const speo_work_item *d_items, int n_items, int dim_lo, int dim_hi,
                                       long long rows, int ld, int k, const float *pop_in,
                                       const float *fit_in, float *pop_out, float *fit_out,
                                       uint32_t *d_gen, int train_steps, float explore, void *stream);

/* One DE generation with the rotation on the tensor cores, over a flat population of n_rows rows
 * (stride ld) planned with tiles of at most SPEO_TILE_TC rows: one trial per target
 * (speo_make_trials, k = 1: the trial draws use tags 1 | 1 << 8 and 2 | 1 << 8), tcgen05 split-FP16
 * evaluation (speo_evaluate_tc) into trial_fit, strict-`<` selection into (pop_out, fit_out)
 * (speo_select_rows); *d_gen advances by one. trial / trial_fit: caller scratch of n_rows rows. */
SPEO_API int speo_generation_tc(const speo_segment *d_segs, const speo_work_item *d_items, int n_items,
                                int dim_lo, int dim_hi, const float *pop_in, const float *fit_in, float *pop_out,
                                float *fit_out, int64_t n_rows, int ld, uint32_t *d_gen, float *trial,
                                float *trial_fit, void *stream);

/* Strict-`<` greedy selection over a flat buffer of `rows` rows (stride ld, a multiple of 4):
 * row r of (pop_out, fit_out) = trial r if trial_fit[r] < fit_in[r], else parent r
 * (kernel_DE_CUDA.cu:305-327 over double buffers). */
SPEO_API int speo_select_rows(const float *pop_in, const float *fit_in, const float *trial,
                              const float *trial_fit, float *pop_out, float *fit_out, long long rows, int ld,
                              void *stream);

/* Per segment: argmin of fit (ties: lowest row) -> best_row[s]; FP64 re-evaluation of that
 * row -> best_err[s] = f(x) - f* in double. */
SPEO_API int speo_best_reeval_f64(const speo_segment *d_segs, int n_segs, const float *pop,
                         const float *fit, int64_t *best_row, double *best_err, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* SPEO_GB300_H */
