/*
 * speo_oracle.h -- CPU oracle for the island-model DE hot path.
 *
 * TEST INFRASTRUCTURE ONLY. This is a plain-C restatement of the reference's algorithm,
 * used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the checker.
 * The product path (libspeo_gb300.so) never links, loads or calls it.
 *
 * Every function cites the reference file:line it restates (paths inside the reference
 * project SPEO-GPU-single-control/). Integer/index work and the FP32 mutant arithmetic are
 * bit-exact restatements; objectives are evaluated in FP64 (the reference's `real`).
 */
#ifndef SPEO_ORACLE_H
#define SPEO_ORACLE_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- Philox-4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11; Random123 v1.09 philox4x32_10) -- */
void speo_oracle_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
/* u32 -> float in (0,1]: ((w >> 8) + 1) * 2^-24, exact in binary32. */
float speo_oracle_u01(uint32_t w);

/* Draw tags (4th Philox counter word); surrogate trial t uses tag | (t << 8). */
#define SPEO_TAG_IDX  1u
#define SPEO_TAG_CR   2u
#define SPEO_TAG_INIT 3u

/* Draw source for the DE generate restatement.
 *  kind 0 (Philox, this library's layout): index draw k of position p at generation gen is
 *     u01(philox({k/4, p, gen, TAG_IDX | tag_hi}, key)[k%4]); the crossover uniform of
 *     element e is u01(philox({e/4, p, gen, TAG_CR | tag_hi}, key)[e%4]).
 *  kind 1 (captured stream, the reference's layout, kernel_DE_CUDA.cu:184-237): one
 *     stream per (position p, lane l) = state p*32+l; lane 0's stream serves the index
 *     draws and then its crossover draws; element e uses lane e%32's (e/32)-th crossover
 *     draw of this generation. cap[(p*32+l)*cap_len + i] is the i-th uniform of that
 *     stream; cap_pos[p*32+l] is advanced as draws are consumed. */
typedef struct {
    int kind;
    uint32_t key[2];
    uint32_t gen;
    uint32_t tag_hi;
    int64_t pos0;        /* Philox row counter = pos0 + position */
    const double *cap;   /* captured uniforms (kind 1), as double (exact for float draws) */
    int cap_len;
    int *cap_pos;
} speo_oracle_draws;

/* ---- Reference-semantics operators (FP32 `real`), identity of argument meaning with
 * the reference's kernels. Rows are `ld` floats apart. Return 0, or a SPEO_DEVERR_* bit
 * mask when a bounded loop hit its limit. ---------------------------------------- */

/* global_DE_FindBestIndividualInIsland (kernel_DE_CUDA.cu:120-158) with the sub-island
 * offset honoured: best_id[s] = row of min fitness among perm[s*S .. s*S+S-1]
 * (ties: first position). */
int speo_oracle_best_per_subisland_f32(const float *fit, int island_size, int subisland_num,
                                       const int *perm, int *best_id);

/* global_DE_GenerateNewPopulation (kernel_DE_CUDA.cu:172-289) + device_CheckBound
 * (:160-170). de_* arrays have one entry per sub-island. */
int speo_oracle_de_generate_f32(float *cand, const float *pop, int ld, int dim,
                                int island_size, int subisland_num, const int *perm,
                                const float *de_CR, const float *de_F, const int *de_strategy,
                                const int *best_id, float lb, float ub,
                                const speo_oracle_draws *draws);
/* FP64 twin (reference as shipped, real = double). Crossover uniforms compared as double;
 * index draws use the same float arithmetic as the FP32 path. */
int speo_oracle_de_generate_f64(double *cand, const double *pop, int ld, int dim,
                                int island_size, int subisland_num, const int *perm,
                                const double *de_CR, const double *de_F, const int *de_strategy,
                                const int *best_id, double lb, double ub,
                                const speo_oracle_draws *draws);

/* global_DE_SelectSurvival (kernel_DE_CUDA.cu:305-327): strict `<`, row copy of dim
 * elements and fitness. Writes sel[i] = 1 where the candidate won (may be NULL). */
void speo_oracle_select_f32(float *pop, float *pop_fit, const float *cand, const float *cand_fit,
                            int n, int ld, int dim, uint8_t *sel);
void speo_oracle_select_f64(double *pop, double *pop_fit, const double *cand, const double *cand_fit,
                            int n, int ld, int dim, uint8_t *sel);

/* global_InitiPopulation (kernel_EA_CUDA.cu:91-118) with Philox draws:
 * x[e] = fmaf(u01(philox({e/4, row, 0, TAG_INIT}, key)[e%4]), ub-lb, lb). */
void speo_oracle_init_population_f32(float *pop, int64_t row0, int n, int ld, int dim,
                                     float lb, float ub, const uint32_t key[2]);

/* ---- Objectives in FP64. o has D entries; M is row-major D x D (file layout,
 * CEC2014.cc:354-369), z = M * (rate * (x - o)) as in sr_func (CEC2014.cc:1395-1435), no
 * rotation for ids 8 and 10, plus the fixed shift 1 of ids 4 and 15. Ids 1-16 follow the
 * reference's EvaluateFitness dispatch (CEC2014.cc:14-144); 31 is sphere_func
 * (CEC2014.cc:462-478), which the reference never dispatches. All return f - f*. */
double speo_oracle_func_rate(int fid);
int speo_oracle_func_rotated(int fid);
/* f from the transformed vector z (rate, rotation and fixed shift already applied). */
double speo_oracle_cec_from_z(int fid, const double *z, int nx);
double speo_oracle_objective_f64(int func_id, const double *x, const double *o, const double *M, int dim);
/* Batch helper for float rows: x rows are `ld` floats apart, o/M given as float (exactly
 * upcast to double). */
void speo_oracle_evaluate_rows(int func_id, const float *x, int n, int ld, int dim,
                               const float *o, const float *M, double *f_out);

/* Hybrid (17-22) and composition (23-30) functions (CEC2014.cc:954-1369, cf_cal :1481-1520).
 * o: nc x D (component-major), M: nc row-major D x D blocks, S: nc x D 1-based shuffles (used by
 * 17-22, 29, 30; may be NULL otherwise); nc = speo_oracle_cec_components(fid). Other ids forward to
 * speo_oracle_objective_f64. */
int speo_oracle_cec_components(int fid);
/* Group starts / lengths of hybrid fid (17-22) at dimension nx; returns the group count. */
int speo_oracle_hybrid_groups(int fid, int nx, int *G, int *G_nx);
double speo_oracle_objective_multi_f64(int fid, const double *x, const double *o, const double *M, const int *S,
                                       int nx);
void speo_oracle_evaluate_rows_multi(int fid, const float *x, int n, int ld, int dim, const float *o,
                                     const float *M, const int *S, double *f_out);

/* Archipelago migration policies: the reference's migrate.cc / buffer_manage.cc for n islands
 * held together, with this library's draws (layout of speo_archipelago in speo_gb300.h). */
typedef struct {
    int n_islands, island_size, dim, ld, migration_size, buffer_capacity, buffer_policy, regroup_option;
    float migration_rate;
    int reserved;
    uint64_t seed;
} speo_oracle_arch;
size_t speo_oracle_arch_state_bytes(const speo_oracle_arch *a);
uint32_t speo_oracle_fperm(uint32_t n, const uint32_t key[4], uint32_t x);
void speo_oracle_arch_init(const speo_oracle_arch *a, uint8_t *state, int *perm, int *subisland_num, int nsub);
void speo_oracle_migrate_out(const speo_oracle_arch *a, uint8_t *state, float *pop, float *fit, int *perm,
                             int *subisland_num, uint32_t g);
void speo_oracle_migrate_in(const speo_oracle_arch *a, uint8_t *state, const float *pop, const float *fit,
                            uint32_t g);

/* ---- Extended (this library's) semantics ------------------------------------------- */
/* Fused generation over segments of identity-permuted rows: what speo_generation computes.
 * Segment arrays are parallel host arrays. pop_in/fit_in -> pop_out/fit_out. fit values of
 * trials are taken from `trial_fit` when non-NULL (so the selection decision can be checked
 * exactly against a device fitness), else evaluated in FP64 and rounded to float. Trials are
 * written to `trial_out` when non-NULL (rows as in pop). */
int speo_oracle_generation_f32(int n_segs, const int64_t *row0, const int *P, const int *D,
                               const int *ld, const int *func, const int *strategy,
                               const float *F, const float *CR, const float *lb, const float *ub,
                               const float *const *o, const float *const *M, const uint64_t *seed,
                               uint32_t gen, const float *pop_in, const float *fit_in,
                               float *pop_out, float *fit_out, float *trial_out,
                               const float *trial_fit, uint8_t *sel_out);

/* Ring migration (replaces src/migrate.cc:46-136): emigrants of s = its k best rows by
 * (fitness, row) ascending, NaN treated as +inf; they replace, in order, the k worst rows of
 * ring_next[s] by (fitness, row) descending. All emigrants are taken before any write. */
void speo_oracle_ring_migrate(int n_segs, const int64_t *row0, const int *P, const int *D,
                              const int *ld, const int *ring_next, int k, float *pop, float *fit);

/* CPU baseline: `gens` generations of the island loop (DE/rand/1/bin, FP64 `real`, objective
 * evaluated in FP64 as the reference does), islands of one ring with shared o/M, ring
 * migration every `interval` generations, spread over `threads` POSIX threads.
 * Population in/out is FP64 rows of `ld`. Returns total exact evaluations done. */
int64_t speo_oracle_run_islands_f64(int n_islands, int P, int D, int ld, int func_id,
                                    double F, double CR, double lb, double ub,
                                    const double *o, const double *M, uint64_t seed,
                                    uint32_t gen0, int gens, int interval, int k_migrate,
                                    double *pop, double *fit, int threads);

/* ---- Surrogate MLP (this library's learned pre-screen; no reference counterpart) -----------
 * din -> h (ReLU) -> h (ReLU) -> 1. Flat FP32 parameter vector, in order:
 *   W1[h][din], b1[h], W2[h][h], b2[h], w3[h], b3[1]   (din=50, h=256: 79105 values).
 * Inputs are scaled by `in_scale` before the first layer. Forward and backward in FP64. */
int speo_oracle_mlp_nparams(int din, int h);
void speo_oracle_mlp_forward(const float *theta, int din, int h, float in_scale, const float *X, int n, int ldx,
                             double *y);
/* Mean-squared-error loss sum_i (y_i - t_i)^2 / n and its gradient w.r.t. theta (FP64). */
double speo_oracle_mlp_loss_grad(const float *theta, int din, int h, float in_scale, const float *X, int n, int ldx,
                                 const float *t, double *grad);
/* One Adam step (Kingma & Ba, 2015) with bias correction; `step` counts from 1. */
void speo_oracle_adam(float *theta, float *m, float *v, const float *g, int n, float lr, float beta1, float beta2,
                      float eps, int step);

#ifdef __cplusplus
}
#endif
#endif
