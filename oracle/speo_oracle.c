/*
 * speo_oracle.c -- CPU oracle for the island-model DE hot path.
 *
 * TEST INFRASTRUCTURE ONLY: a plain-C restatement of the reference's algorithm that the
 * tests, smoke() and the CPU-baseline leg of bench.py use as the checker. It is never
 * linked into, loaded by or called from libspeo_gb300.so.
 *
 * Build: -O2 -ffp-contract=off (every fused multiply-add is an explicit fma/fmaf, so the
 * results are the same on x86-64 and aarch64).
 */
#include "speo_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define SPEO_DEVERR_REDRAW_LIMIT 0x1
#define SPEO_DEVERR_BOUND_LIMIT 0x2
#define SPEO_REDRAW_ITERS 4096
#define SPEO_BOUND_ITERS 64
#define SPEO_ORACLE_MAX_DIM 256

#define CAT_(a, b) a##b
#define CAT(a, b) CAT_(a, b)

/* ------------------------------------------------------------------------------------ */
/* Philox-4x32-10. Restated from the published algorithm (Salmon et al., "Parallel random  */
/* numbers: as easy as 1, 2, 3", SC'11), Random123 v1.09 constants.                       */
/* ------------------------------------------------------------------------------------ */
void speo_oracle_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int round = 0; round < 10; ++round) {
        if (round) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
        const uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        const uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        c0 = hi1 ^ c1 ^ k0;
        c1 = lo1;
        c2 = hi0 ^ c3 ^ k1;
        c3 = lo0;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

float speo_oracle_u01(uint32_t w)
{
    return (float)((w >> 8) + 1u) * 5.9604644775390625e-8f; /* 2^-24 */
}

/* NaN ranks as +inf in every best/worst search. */
static float nan_as_inf(float f) { return isnan(f) ? INFINITY : f; }

static int next_pow2_dim(int dim)
{
    /* EA_CUDA::CalNextPow2Dim, CUDA_EA_library/EA_CUDA.cc:197-206 */
    int y = 1;
    while (y < dim) y <<= 1;
    return y < 32 ? 32 : y;
}

/* ---- draw source --------------------------------------------------------------------- */
typedef struct {
    const speo_oracle_draws *d;
    int64_t row;          /* Philox row counter */
    int pos;
    uint32_t k;           /* next index-draw number (Philox) */
    uint32_t block[4];
    uint32_t block_id;
    int have_block;
} draw_cursor;

static void cursor_begin(draw_cursor *c, const speo_oracle_draws *d, int pos)
{
    c->d = d;
    c->pos = pos;
    c->row = d->pos0 + pos;
    c->k = 0;
    c->have_block = 0;
}

static void cursor_end(draw_cursor *c, const speo_oracle_draws *d, int pos)
{
    (void)c; (void)d; (void)pos;
}

static double captured_next(const speo_oracle_draws *d, int stream)
{
    const int i = d->cap_pos[stream]++;
    return d->cap[(size_t)stream * d->cap_len + (i < d->cap_len ? i : d->cap_len - 1)];
}

/* Uniform for the k-th index draw of this position. */
static double draw_uniform_idx(draw_cursor *c)
{
    const speo_oracle_draws *d = c->d;
    if (d->kind == 1) return captured_next(d, c->pos * 32);
    const uint32_t blk = c->k >> 2, w = c->k & 3u;
    if (!c->have_block || c->block_id != blk) {
        const uint32_t ctr[4] = {blk, (uint32_t)c->row, d->gen, SPEO_TAG_IDX | d->tag_hi};
        speo_oracle_philox(ctr, d->key, c->block);
        c->block_id = blk;
        c->have_block = 1;
    }
    c->k++;
    return (double)speo_oracle_u01(c->block[w]);
}

/* (int)(u * n): float arithmetic, except for a captured FP64 stream, which uses the double
 * arithmetic of the reference's GPU_DOUBLE_PRECISION build (kernel_DE_CUDA.cu:190). */
static int draw_index(draw_cursor *c, int n, int real_size)
{
    const double u = draw_uniform_idx(c);
    if (c->d->kind == 1 && real_size == 8) return (int)(u * (double)n);
    return (int)((float)u * (float)n);
}

static double draw_cr(draw_cursor *c, const speo_oracle_draws *d, int pos, int e, int lane)
{
    if (d->kind == 1) return captured_next(d, pos * 32 + lane);
    const uint32_t ctr[4] = {(uint32_t)(e >> 2), (uint32_t)c->row, d->gen, SPEO_TAG_CR | d->tag_hi};
    uint32_t out[4];
    speo_oracle_philox(ctr, d->key, out);
    (void)lane;
    return (double)speo_oracle_u01(out[e & 3]);
}

/* ---- precision-generic DE operators ---------------------------------------------------- */
#define REAL float
#define FMA fmaf
#define SFX _f32
#include "oracle_de_impl.h"
#undef REAL
#undef FMA
#undef SFX
#define REAL double
#define FMA fma
#define SFX _f64
#include "oracle_de_impl.h"
#undef REAL
#undef FMA
#undef SFX

int speo_oracle_best_per_subisland_f32(const float *fit, int island_size, int subisland_num,
                                       const int *perm, int *best_id)
{
    /* kernel_DE_CUDA.cu:120-158, reading perm[s*S + i] (the reference omits s*S). */
    const int S = island_size / subisland_num;
    for (int s = 0; s < subisland_num; ++s) {
        int best = perm[s * S];
        float bf = nan_as_inf(fit[best]);
        for (int i = 1; i < S; ++i) {
            const int row = perm[s * S + i];
            if (bf > nan_as_inf(fit[row])) { bf = nan_as_inf(fit[row]); best = row; }
        }
        best_id[s] = best;
    }
    return 0;
}

void speo_oracle_init_population_f32(float *pop, int64_t row0, int n, int ld, int dim,
                                     float lb, float ub, const uint32_t key[2])
{
    /* kernel_EA_CUDA.cu:91-118: x = min + u * (max - min), u from this library's stream */
    const float range = ub - lb;
    for (int i = 0; i < n; ++i) {
        const uint32_t row = (uint32_t)(row0 + i);
        for (int e = 0; e < dim; ++e) {
            const uint32_t ctr[4] = {(uint32_t)(e >> 2), row, 0u, SPEO_TAG_INIT};
            uint32_t out[4];
            speo_oracle_philox(ctr, key, out);
            pop[(size_t)i * ld + e] = fmaf(speo_oracle_u01(out[e & 3]), range, lb);
        }
    }
}

/* ---- objectives ---------------------------------------------------------------------- */
/* CEC2014 functions 1-16 and the rotated sphere (31), restated from the reference's CPU code
 * (CUDA_EA_library/CEC2014.cc): EvaluateFitness dispatch :14-144 (id, rate, rotation, fixed
 * shift), sr_func :1395-1435 (ye = (x - o) * rate, z = M ye), the function bodies :462-953.
 * Returns f(x) - f*, the reference's convention. */
#define ORACLE_PI 3.1415926535897932384626433832795029
#define ORACLE_E 2.7182818284590452353602874713526625

double speo_oracle_func_rate(int fid)
{
    switch (fid) {
    case 4: return 2.048 / (double)100;
    case 6: return 0.5 / (double)100;
    case 7: return 6.0;
    case 8: case 9: return 5.12 / (double)100;
    case 10: case 11: return 10.0;
    case 12: case 13: case 14: case 15: return 5 / (double)100;
    default: return 1.0;
    }
}
int speo_oracle_func_rotated(int fid) { return fid != 8 && fid != 10; }
static double fixed_shift(int fid) { return (fid == 4 || fid == 15) ? 1.0 : 0.0; }

/* f from z (after rate, rotation and the fixed shift), in the reference's order of operations. */
double speo_oracle_cec_from_z(int fid, const double *z, int nx)
{
    double f = 0.0;
    switch (fid) {
    case 1: /* ellips_func :481-497 */
        for (int i = 0; i < nx; i++) f += pow(10.0, 6.0 * i / (nx - 1)) * z[i] * z[i];
        return f;
    case 2: /* bent_cigar_func :499-516 */
        f = z[0] * z[0];
        for (int i = 1; i < nx; i++) f += pow(10.0, 6.0) * z[i] * z[i];
        return f;
    case 3: /* discus_func :518-531 */
        f = pow(10.0, 6.0) * z[0] * z[0];
        for (int i = 1; i < nx; i++) f += z[i] * z[i];
        return f;
    case 4: /* rosenbrock_func :552-567 */
        for (int i = 0; i < nx - 1; i++) {
            const double t1 = z[i] * z[i] - z[i + 1], t2 = z[i] - 1.0;
            f += 100.0 * t1 * t1 + t2 * t2;
        }
        return f;
    case 5: { /* ackley_func :590-613 */
        double s1 = 0.0, s2 = 0.0;
        for (int i = 0; i < nx; i++) { s1 += z[i] * z[i]; s2 += cos(2.0 * ORACLE_PI * z[i]); }
        s1 = -0.2 * sqrt(s1 / (double)nx);
        s2 /= (double)nx;
        return ORACLE_E - 20.0 * exp(s1) + 20.0 - exp(s2);
    }
    case 6: { /* weierstrass_func :615-644 */
        double sum2 = 0.0;
        for (int i = 0; i < nx; i++) {
            double sum = 0.0;
            sum2 = 0.0;
            for (int j = 0; j <= 20; j++) {
                sum += pow(0.5, j) * cos(2.0 * ORACLE_PI * pow(3.0, j) * (z[i] + 0.5));
                sum2 += pow(0.5, j) * cos(2.0 * ORACLE_PI * pow(3.0, j) * 0.5);
            }
            f += sum;
        }
        return f - nx * sum2;
    }
    case 7: { /* griewank_func :646-666 */
        double s = 0.0, p = 1.0;
        for (int i = 0; i < nx; i++) { s += z[i] * z[i]; p *= cos(z[i] / sqrt(1.0 + i)); }
        return 1.0 + s / 4000.0 - p;
    }
    case 8: case 9: /* rastrigin_func :668-683 */
        for (int i = 0; i < nx; i++) f += (z[i] * z[i] - 10.0 * cos(2.0 * ORACLE_PI * z[i]) + 10.0);
        return f;
    case 10: case 11: /* schwefel_func :705-737 */
        for (int i = 0; i < nx; i++) {
            const double zi = z[i] + 4.209687462275036e+002;
            if (zi > 500) {
                f -= (500.0 - fmod(zi, 500)) * sin(pow(500.0 - fmod(zi, 500), 0.5));
                const double t = (zi - 500.0) / 100;
                f += t * t / nx;
            } else if (zi < -500) {
                f -= (-500.0 + fmod(fabs(zi), 500)) * sin(pow(500.0 - fmod(fabs(zi), 500), 0.5));
                const double t = (zi + 500.0) / 100;
                f += t * t / nx;
            } else {
                f -= zi * sin(pow(fabs(zi), 0.5));
            }
        }
        return f + 4.189828872724338e+002 * nx;
    case 12: { /* katsuura_func :739-763 */
        double p = 1.0;
        const double e3 = pow(1.0 * nx, 1.2);
        for (int i = 0; i < nx; i++) {
            double t = 0.0;
            for (int j = 1; j <= 32; j++) {
                const double a = pow(2.0, j), b = a * z[i];
                t += fabs(b - floor(b + 0.5)) / a;
            }
            p *= pow(1.0 + (i + 1) * t, 10.0 / e3);
        }
        const double c = 10.0 / nx / nx;
        return p * c - c;
    }
    case 13: case 14: { /* happycat_func :907-929, hgbat_func :931-953 */
        double r2 = 0.0, sz = 0.0;
        for (int i = 0; i < nx; i++) { const double zi = z[i] - 1.0; r2 += zi * zi; sz += zi; }
        if (fid == 13) return pow(fabs(r2 - nx), 2 * (1.0 / 8.0)) + (0.5 * r2 + sz) / nx + 0.5;
        return pow(fabs(pow(r2, 2.0) - pow(sz, 2.0)), 2 * (1.0 / 4.0)) + (0.5 * r2 + sz) / nx + 0.5;
    }
    case 15: /* grie_rosen_func :842-868 */
        for (int i = 0; i < nx; i++) {
            const int k = i + 1 < nx ? i + 1 : 0;
            const double t1 = z[i] * z[i] - z[k], t2 = z[i] - 1.0;
            const double t = 100.0 * t1 * t1 + t2 * t2;
            f += (t * t) / 4000.0 - cos(t) + 1.0;
        }
        return f;
    case 16: /* escaffer6_func :870-905 */
        if (nx == 1) {
            const double t1 = sin(z[0]), t2 = 1.0 + 0.001 * (z[0] * z[0]);
            return 0.5 + (t1 * t1 - 0.5) / (t2 * t2);
        }
        for (int i = 0; i < nx; i++) {
            const int k = i + 1 < nx ? i + 1 : 0;
            const double s2 = z[i] * z[i] + z[k] * z[k];
            const double t1 = sin(sqrt(s2)), t2 = 1.0 + 0.001 * s2;
            f += 0.5 + (t1 * t1 - 0.5) / (t2 * t2);
        }
        return f;
    default: /* 31: sphere_func :462-478 */
        for (int i = 0; i < nx; i++) f += z[i] * z[i];
        return f;
    }
}

double speo_oracle_objective_f64(int func_id, const double *x, const double *o, const double *M, int dim)
{
    /* sr_func (CEC2014.cc:1395-1435): ye = (x - o) * rate; z = M * ye (rotatefunc :1382-1393) */
    double ye[SPEO_ORACLE_MAX_DIM], z[SPEO_ORACLE_MAX_DIM];
    const double rate = speo_oracle_func_rate(func_id), fs = fixed_shift(func_id);
    for (int i = 0; i < dim; ++i) ye[i] = (x[i] - o[i]) * rate;
    for (int i = 0; i < dim; ++i) {
        double zi = ye[i];
        if (speo_oracle_func_rotated(func_id)) {
            zi = 0;
            for (int j = 0; j < dim; ++j) zi = zi + ye[j] * M[i * dim + j];
        }
        z[i] = zi + fs;
    }
    return speo_oracle_cec_from_z(func_id, z, dim);
}

void speo_oracle_evaluate_rows(int func_id, const float *x, int n, int ld, int dim,
                               const float *o, const float *M, double *f_out)
{
    double od[SPEO_ORACLE_MAX_DIM], xd[SPEO_ORACLE_MAX_DIM];
    double *Md = (double *)malloc(sizeof(double) * (size_t)dim * dim);
    for (int i = 0; i < dim; ++i) od[i] = o[i];
    for (int i = 0; i < dim * dim; ++i) Md[i] = M[i];
    for (int r = 0; r < n; ++r) {
        for (int i = 0; i < dim; ++i) xd[i] = x[(size_t)r * ld + i];
        f_out[r] = speo_oracle_objective_f64(func_id, xd, od, Md, dim);
    }
    free(Md);
}

/* ---- CEC2014 hybrid (17-22) and composition (23-30) functions ---------------------------
 * Hybrid functions hf01..hf06 (CEC2014.cc:954-1206): z = M (x - o) (rate 1), y_i = z[S_i - 1]
 * (S 1-based), y cut into groups of ceil(gp_g * D) coordinates (the last takes the rest); group g
 * is body fid_g on y_g * rate(fid_g) + its fixed shift, with the group's own length; f = sum of
 * the groups in order.
 * Composition functions cf01..cf08 (CEC2014.cc:1209-1369): component c evaluates its body on
 * rate * M_c (x - o_c) (or without M_c) and is rescaled as num * f / den; cf07 / cf08 take the
 * hybrids hf01-03 / hf04-06 on (o_c, M_c, S_c). cf_cal (:1481-1520) adds bias_c = 100 c, weights
 * w_c = (1 / S_c)^0.5 exp(-S_c / (2 D delta_c^2)), S_c = sum (x - o_c)^2 (1e99 at S_c = 0; all 1
 * when every weight is 0) and returns sum w_c / w_sum * fit_c. Bodies are chosen by the ids 1-16
 * whose code they share (schwefel = 10, rastrigin = 8), with those ids' rates and fixed shifts. */
typedef struct { int n; double gp[5]; int fid[5]; } oracle_hybrid;
static const oracle_hybrid k_hybrid[6] = {
    {3, {0.3, 0.3, 0.4}, {10, 8, 1}},                        /* hf01 :954-991  */
    {3, {0.3, 0.3, 0.4}, {2, 14, 8}},                        /* hf02 :993-1032 */
    {4, {0.2, 0.2, 0.3, 0.3}, {7, 6, 4, 16}},                /* hf03 :1034-1075 */
    {4, {0.2, 0.2, 0.3, 0.3}, {14, 3, 15, 8}},               /* hf04 :1077-1117 */
    {5, {0.1, 0.2, 0.2, 0.2, 0.3}, {16, 14, 4, 10, 1}},      /* hf05 :1119-1162 */
    {5, {0.1, 0.2, 0.2, 0.2, 0.2}, {12, 13, 15, 10, 5}},     /* hf06 :1164-1207 */
};
typedef struct { int fid, rotated; double num, den; } oracle_piece; /* den 0: no rescale */
typedef struct { int n, hybrid0; double delta[5]; oracle_piece c[5]; } oracle_comp;
static const oracle_comp k_comp[8] = {
    {5, -1, {10, 20, 30, 40, 50},                           /* cf01 :1209-1233 */
     {{4, 1, 10000, 1e+4}, {1, 1, 10000, 1e+10}, {2, 1, 10000, 1e+30}, {3, 1, 10000, 1e+10}, {1, 0, 10000, 1e+10}}},
    {3, -1, {20, 20, 20}, {{10, 0, 0, 0}, {8, 1, 0, 0}, {14, 1, 0, 0}}},                    /* cf02 :1235-1249 */
    {3, -1, {10, 30, 50}, {{10, 1, 1000, 4e+3}, {8, 1, 1000, 1e+3}, {1, 1, 1000, 1e+10}}}, /* cf03 :1251-1267 */
    {5, -1, {10, 10, 10, 10, 10},                           /* cf04 :1269-1291 */
     {{10, 1, 1000, 4e+3}, {13, 1, 1000, 1e+3}, {1, 1, 1000, 1e+10}, {6, 1, 1000, 400}, {7, 1, 1000, 100}}},
    {5, -1, {10, 10, 10, 20, 20},                           /* cf05 :1293-1315 */
     {{14, 1, 10000, 1000}, {8, 1, 10000, 1e+3}, {10, 1, 10000, 4e+3}, {6, 1, 10000, 400}, {1, 1, 10000, 1e+10}}},
    {5, -1, {10, 20, 30, 40, 50},                           /* cf06 :1317-1339 */
     {{15, 1, 10000, 4e+3}, {13, 1, 10000, 1e+3}, {10, 1, 10000, 4e+3}, {16, 1, 10000, 2e+7}, {1, 1, 10000, 1e+10}}},
    {3, 0, {10, 30, 50}, {{0}}},                            /* cf07 :1341-1354: hf01, hf02, hf03 */
    {3, 3, {10, 30, 50}, {{0}}},                            /* cf08 :1356-1369: hf04, hf05, hf06 */
};

int speo_oracle_cec_components(int fid)
{
    return (fid >= 23 && fid <= 30) ? k_comp[fid - 23].n : 1;
}

int speo_oracle_hybrid_groups(int fid, int nx, int *G, int *G_nx)
{
    if (fid < 17 || fid > 22) return 0;
    const oracle_hybrid *h = &k_hybrid[fid - 17];
    int tmp = 0;
    for (int i = 0; i < h->n - 1; i++) {
        G_nx[i] = (int)ceil(h->gp[i] * nx);
        tmp += G_nx[i];
    }
    G_nx[h->n - 1] = nx - tmp;
    G[0] = 0;
    for (int i = 1; i < h->n; i++) G[i] = G[i - 1] + G_nx[i - 1];
    return h->n;
}

static double hybrid_f64(int hi, const double *x, const double *o, const double *M, const int *S, int nx)
{
    double ze[SPEO_ORACLE_MAX_DIM], ye[SPEO_ORACLE_MAX_DIM], zg[SPEO_ORACLE_MAX_DIM];
    int G[5], G_nx[5];
    const oracle_hybrid *h = &k_hybrid[hi];
    speo_oracle_hybrid_groups(17 + hi, nx, G, G_nx);
    for (int i = 0; i < nx; ++i) ye[i] = (x[i] - o[i]) * 1.0;
    for (int i = 0; i < nx; ++i) {
        double zi = 0;
        for (int j = 0; j < nx; ++j) zi = zi + ye[j] * M[i * nx + j];
        ze[i] = zi;
    }
    for (int i = 0; i < nx; ++i) ye[i] = ze[S[i] - 1];
    double f = 0.0;
    for (int g = 0; g < h->n; ++g) {
        const int fid = h->fid[g];
        const double rate = speo_oracle_func_rate(fid), fs = fixed_shift(fid);
        for (int i = 0; i < G_nx[g]; ++i) zg[i] = ye[G[g] + i] * rate + fs;
        f += speo_oracle_cec_from_z(fid, zg, G_nx[g]);
    }
    return f;
}

static double piece_f64(const oracle_piece *pc, const double *x, const double *o, const double *M, int nx)
{
    double ye[SPEO_ORACLE_MAX_DIM], z[SPEO_ORACLE_MAX_DIM];
    const double rate = speo_oracle_func_rate(pc->fid), fs = fixed_shift(pc->fid);
    for (int i = 0; i < nx; ++i) ye[i] = (x[i] - o[i]) * rate;
    for (int i = 0; i < nx; ++i) {
        double zi = ye[i];
        if (pc->rotated) {
            zi = 0;
            for (int j = 0; j < nx; ++j) zi = zi + ye[j] * M[i * nx + j];
        }
        z[i] = zi + fs;
    }
    double f = speo_oracle_cec_from_z(pc->fid, z, nx);
    if (pc->den != 0) f = pc->num * f / pc->den;
    return f;
}

double speo_oracle_objective_multi_f64(int fid, const double *x, const double *o, const double *M, const int *S,
                                       int nx)
{
    if (fid >= 17 && fid <= 22) return hybrid_f64(fid - 17, x, o, M, S, nx);
    if (fid < 23 || fid > 30) return speo_oracle_objective_f64(fid, x, o, M, nx);
    const oracle_comp *cp = &k_comp[fid - 23];
    double fit[5], w[5], w_max = 0, w_sum = 0;
    for (int c = 0; c < cp->n; ++c) {
        const double *oc = o + (size_t)c * nx, *Mc = M + (size_t)c * nx * nx;
        fit[c] = cp->hybrid0 >= 0 ? hybrid_f64(cp->hybrid0 + c, x, oc, Mc, S + (size_t)c * nx, nx)
                                  : piece_f64(&cp->c[c], x, oc, Mc, nx);
    }
    for (int c = 0; c < cp->n; ++c) {   /* cf_cal :1481-1520 */
        fit[c] += 100.0 * c;
        w[c] = 0;
        for (int j = 0; j < nx; ++j) w[c] += pow(x[j] - o[(size_t)c * nx + j], 2.0);
        if (w[c] != 0)
            w[c] = pow(1.0 / w[c], 0.5) * exp(-w[c] / 2.0 / nx / pow(cp->delta[c], 2.0));
        else
            w[c] = 1.0e99;
        if (w[c] > w_max) w_max = w[c];
    }
    for (int c = 0; c < cp->n; ++c) w_sum = w_sum + w[c];
    if (w_max == 0) {
        for (int c = 0; c < cp->n; ++c) w[c] = 1;
        w_sum = cp->n;
    }
    double f = 0.0;
    for (int c = 0; c < cp->n; ++c) f = f + w[c] / w_sum * fit[c];
    return f;
}

void speo_oracle_evaluate_rows_multi(int fid, const float *x, int n, int ld, int dim, const float *o,
                                     const float *M, const int *S, double *f_out)
{
    const int nc = speo_oracle_cec_components(fid);
    double xd[SPEO_ORACLE_MAX_DIM];
    double *od = (double *)malloc(sizeof(double) * (size_t)nc * dim);
    double *Md = (double *)malloc(sizeof(double) * (size_t)nc * dim * dim);
    for (int i = 0; i < nc * dim; ++i) od[i] = o[i];
    for (int i = 0; i < nc * dim * dim; ++i) Md[i] = M[i];
    for (int r = 0; r < n; ++r) {
        for (int i = 0; i < dim; ++i) xd[i] = x[(size_t)r * ld + i];
        f_out[r] = speo_oracle_objective_multi_f64(fid, xd, od, Md, S, dim);
    }
    free(od);
    free(Md);
}

/* ---- archipelago migration policies ------------------------------------------------------
 * The reference's migration (src/migrate.cc:34-186) and immigrant buffers
 * (src/buffer_manage.cc:36-313) for n islands held together, with this library's draws: Philox
 * tags 7-11 and keyed Feistel permutations in place of rand() and the partial Fisher-Yates of
 * random.cc:29-53. Same state layout as the library, so states compare byte for byte:
 * ints per island [0] list length, [1] head, [2] buffer size, [3] 0, list[N], member[C], flag[C],
 * order[C] (padded to 4); floats per island entry[C][D+1], centre[C][D] (padded to 4). */
static int arch_istride(const speo_oracle_arch *a) { return (4 + a->n_islands + 3 * a->buffer_capacity + 3) / 4 * 4; }
static int arch_fstride(const speo_oracle_arch *a) { return (a->buffer_capacity * (2 * a->dim + 1) + 3) / 4 * 4; }

size_t speo_oracle_arch_state_bytes(const speo_oracle_arch *a)
{
    return 4 * (size_t)a->n_islands * (size_t)(arch_istride(a) + arch_fstride(a));
}

typedef struct { int *ints; float *flts; int N, C, D, is, fs; } arch_view;
static arch_view arch_of(const speo_oracle_arch *a, uint8_t *state)
{
    arch_view v;
    v.N = a->n_islands; v.C = a->buffer_capacity; v.D = a->dim;
    v.is = arch_istride(a); v.fs = arch_fstride(a);
    v.ints = (int *)state;
    v.flts = (float *)(v.ints + (size_t)v.N * v.is);
    return v;
}
static int *a_hdr(const arch_view *v, int i) { return v->ints + (size_t)i * v->is; }
static int *a_list(const arch_view *v, int i) { return a_hdr(v, i) + 4; }
static int *a_member(const arch_view *v, int i) { return a_hdr(v, i) + 4 + v->N; }
static int *a_flag(const arch_view *v, int i) { return a_member(v, i) + v->C; }
static int *a_order(const arch_view *v, int i) { return a_flag(v, i) + v->C; }
static float *a_entry(const arch_view *v, int i, int c) { return v->flts + (size_t)i * v->fs + (size_t)c * (v->D + 1); }
static float *a_centre(const arch_view *v, int i, int c)
{
    return v->flts + (size_t)i * v->fs + (size_t)v->C * (v->D + 1) + (size_t)c * v->D;
}

static uint32_t fmix32(uint32_t v)
{
    v ^= v >> 16; v *= 0x85EBCA6Bu; v ^= v >> 13; v *= 0xC2B2AE35u; v ^= v >> 16;
    return v;
}

uint32_t speo_oracle_fperm(uint32_t n, const uint32_t key[4], uint32_t x)
{
    uint32_t bits = 0;
    while (bits < 30 && (1u << bits) < n) ++bits;
    uint32_t h = (bits + 1) / 2;
    if (h == 0) h = 1;
    const uint32_t mask = (1u << h) - 1u;
    for (uint64_t it = 0; it < (1ull << (2 * h)); ++it) {
        uint32_t L = x >> h, R = x & mask;
        for (int r = 0; r < 4; ++r) {
            const uint32_t t = L ^ (fmix32(R * 0x9E3779B1u ^ key[r]) & mask);
            L = R;
            R = t;
        }
        x = (L << h) | R;
        if (x < n) return x;
    }
    return 0u;
}

static void arch_draw(const speo_oracle_arch *a, uint32_t c0, uint32_t c1, uint32_t c2, uint32_t tag, uint32_t out[4])
{
    const uint32_t ctr[4] = {c0, c1, c2, tag};
    const uint32_t key[2] = {(uint32_t)a->seed, (uint32_t)(a->seed >> 32)};
    speo_oracle_philox(ctr, key, out);
}
static uint32_t below(uint32_t w, uint32_t n) { return (uint32_t)(((uint64_t)w * n) >> 32); }

/* vector::erase(begin + pos) on the live order, the freed slot kept behind it */
static void order_erase(int *order, int size, int pos)
{
    const int slot = order[pos];
    for (int i = pos; i < size - 1; ++i) order[i] = order[i + 1];
    order[size - 1] = slot;
}

void speo_oracle_arch_init(const speo_oracle_arch *a, uint8_t *state, int *perm, int *subisland_num, int nsub)
{
    arch_view v = arch_of(a, state);
    memset(state, 0, speo_oracle_arch_state_bytes(a));
    for (int i = 0; i < v.N; ++i) {
        for (int c = 0; c < v.C; ++c) a_order(&v, i)[c] = c;
        for (int r = 0; r < a->island_size; ++r) perm[(size_t)i * a->island_size + r] = r;
        subisland_num[i] = nsub;
    }
}

void speo_oracle_migrate_out(const speo_oracle_arch *a, uint8_t *state, float *pop, float *fit, int *perm,
                             int *subisland_num, uint32_t g)
{
    arch_view v = arch_of(a, state);
    const int P = a->island_size, D = a->dim;
    for (int s = 0; s < v.N; ++s) {
        int *h = a_hdr(&v, s);
        /* UpdateDestination (migrate.cc:34-44): each other island with probability migration_rate */
        if (h[1] >= h[0]) {
            int cnt = 0;
            for (int t = 0; t < v.N; ++t) {
                uint32_t w[4];
                if (t == s) continue;
                arch_draw(a, (uint32_t)t, (uint32_t)s, g, 7u, w);
                if (speo_oracle_u01(w[0]) < a->migration_rate) a_list(&v, s)[cnt++] = t;
            }
            h[0] = cnt;
            h[1] = 0;
        }
        /* UpdatePopulation (migrate.cc:46-62): SelectFromBuffer, then distinct random rows */
        int sel[64], n = 0, size = h[2];
        int *order = a_order(&v, s), *flag = a_flag(&v, s);
        if (a->buffer_policy == 0) {            /* OnlineCluster::SelectFromBuffer :105-117 */
            for (int c = 0; c < size; ++c)
                if (flag[c]) { sel[n++] = c; flag[c] = 0; }
        } else {
            for (int q = 0; q < a->migration_size && size > 0; ++q) {
                int pos = 0;
                if (a->buffer_policy == 1) {    /* BestSelect::FindBestBufferMember :178-191 */
                    float bf = a_entry(&v, s, order[0])[D];
                    for (int i = 1; i < size; ++i)
                        if (bf < a_entry(&v, s, order[i])[D]) { bf = a_entry(&v, s, order[i])[D]; pos = i; }
                } else if (a->buffer_policy == 2) { /* RandomSelect :235-245 */
                    uint32_t w[4];
                    arch_draw(a, (uint32_t)q, (uint32_t)s, g, 11u, w);
                    pos = (int)below(w[0], (uint32_t)size);
                } else if (a->buffer_policy == 4) { /* LIFO :303-313: the newest */
                    pos = size - 1;
                }                                   /* FIFO :268-278: the oldest */
                sel[n++] = order[pos];
                order_erase(order, size, pos);
                --size;
            }
        }
        h[2] = size;
        if (n > 0) {
            uint32_t key[4];
            arch_draw(a, (uint32_t)s, g, 0u, 9u, key);
            for (int q = 0; q < n; ++q) {
                const size_t row = (size_t)s * P + speo_oracle_fperm((uint32_t)P, key, (uint32_t)q);
                const float *e = a_entry(&v, s, sel[q]);
                for (int j = 0; j < D; ++j) pop[row * a->ld + j] = e[j];
                fit[row] = e[D];
            }
        }
        /* RegroupIslands (migrate.cc:147-186) */
        const int opt = a->regroup_option;
        if (opt == 2 || opt == 3) {
            int max_index = 0, q = P / 4;
            uint32_t w[4];
            while (q > 1) { q /= 2; max_index++; }
            arch_draw(a, (uint32_t)s, g, 0u, 10u, w);
            subisland_num[s] = P / (4 << below(w[0], (uint32_t)(max_index + 1)));
        }
        if (opt == 1 || opt == 3) {
            uint32_t key[4];
            arch_draw(a, (uint32_t)s, g, 1u, 10u, key);
            for (int r = 0; r < P; ++r) perm[(size_t)s * P + r] = (int)speo_oracle_fperm((uint32_t)P, key, (uint32_t)r);
        }
    }
}

void speo_oracle_migrate_in(const speo_oracle_arch *a, uint8_t *state, const float *pop, const float *fit, uint32_t g)
{
    arch_view v = arch_of(a, state);
    const int P = a->island_size, D = a->dim, C = v.C;
    for (int d = 0; d < v.N; ++d) {
        int *h = a_hdr(&v, d);
        for (int src = 0; src < v.N; ++src) {
            const int *hs = a_hdr(&v, src);
            if (hs[1] >= hs[0] || a_list(&v, src)[hs[1]] != d) continue;
            /* SendEmigrations (migrate.cc:105-136): migration_size distinct random rows */
            uint32_t key[4];
            arch_draw(a, (uint32_t)src, g, 0u, 8u, key);
            for (int q = 0; q < a->migration_size; ++q) {
                const size_t row = (size_t)src * P + speo_oracle_fperm((uint32_t)P, key, (uint32_t)q);
                const float *x = pop + row * a->ld;
                const float fx = fit[row];
                if (a->buffer_policy == 0) {    /* OnlineCluster::UpdateBuffer :119-131 */
                    const int size = h[2];
                    if (size < C) {             /* CreatCluster :51-58 */
                        memcpy(a_entry(&v, d, size), x, sizeof(float) * D);
                        a_entry(&v, d, size)[D] = fx;
                        memcpy(a_centre(&v, d, size), x, sizeof(float) * D);
                        a_member(&v, d)[size] = 1;
                        a_flag(&v, d)[size] = 1;
                        h[2] = size + 1;
                        continue;
                    }
                    int best = 0;               /* FindNearestIndividual :134-150, CalDistance :38-49 */
                    float bv = 0.f;
                    for (int c = 0; c < C; ++c) {
                        const float *cc = a_centre(&v, d, c);
                        float acc = 0.f;
                        for (int j = 0; j < D; ++j) {
                            const float df = x[j] - cc[j];
                            acc = acc + df * df;
                        }
                        const float dist = sqrtf(acc);
                        if (c == 0 || bv > dist) { bv = dist; best = c; }
                    }
                    /* ReplaceMemberToCluster :60-76 */
                    const int m = a_member(&v, d)[best];
                    float *cc = a_centre(&v, d, best);
                    for (int j = 0; j < D; ++j) {
                        const float t = (float)m * cc[j] + x[j];
                        cc[j] = (float)((double)t / ((double)m + 1.0));
                    }
                    memcpy(a_entry(&v, d, best), x, sizeof(float) * D);
                    a_entry(&v, d, best)[D] = fx;
                    a_member(&v, d)[best] = m + 1;
                    a_flag(&v, d)[best] = 1;
                } else {                        /* push_back, then erase(begin) past capacity */
                    int *order = a_order(&v, d);
                    const int size = h[2];
                    int slot;
                    if (size < C) {
                        slot = order[size];
                        h[2] = size + 1;
                    } else {
                        slot = order[0];
                        order_erase(order, size, 0);
                    }
                    memcpy(a_entry(&v, d, slot), x, sizeof(float) * D);
                    a_entry(&v, d, slot)[D] = fx;
                }
            }
        }
    }
    for (int s = 0; s < v.N; ++s) {
        int *h = a_hdr(&v, s);
        if (h[1] < h[0]) h[1] += 1;
    }
}

/* ---- fused generation (this library's extended semantics) ------------------------------ */
static int seg_best_row(const float *fit, int64_t row0, int P)
{
    int best = 0;
    float bf = nan_as_inf(fit[row0]);
    for (int i = 1; i < P; ++i)
        if (nan_as_inf(fit[row0 + i]) < bf) { bf = nan_as_inf(fit[row0 + i]); best = i; }
    return best;
}

int speo_oracle_generation_f32(int n_segs, const int64_t *row0, const int *P, const int *D,
                               const int *ld, const int *func, const int *strategy,
                               const float *F, const float *CR, const float *lb, const float *ub,
                               const float *const *o, const float *const *M, const uint64_t *seed,
                               uint32_t gen, const float *pop_in, const float *fit_in,
                               float *pop_out, float *fit_out, float *trial_out,
                               const float *trial_fit, uint8_t *sel_out)
{
    int err = 0;
    for (int s = 0; s < n_segs; ++s) {
        const int n = P[s], dim = D[s], l = ld[s];
        const int64_t base = row0[s];
        int *perm = (int *)malloc(sizeof(int) * (size_t)n);
        for (int i = 0; i < n; ++i) perm[i] = i;
        float *cand = (float *)calloc((size_t)n * l, sizeof(float));
        const float *pin = pop_in + (size_t)base * l;
        int best = seg_best_row(fit_in, base, n);
        speo_oracle_draws dr;
        memset(&dr, 0, sizeof dr);
        dr.kind = 0;
        dr.key[0] = (uint32_t)seed[s];
        dr.key[1] = (uint32_t)(seed[s] >> 32);
        dr.gen = gen;
        dr.pos0 = base;
        err |= speo_oracle_de_generate_f32(cand, pin, l, dim, n, 1, perm, &CR[s], &F[s],
                                           &strategy[s], &best, lb[s], ub[s], &dr);
        double *fd = (double *)malloc(sizeof(double) * (size_t)n);
        if (!trial_fit) speo_oracle_evaluate_rows(func[s], cand, n, l, dim, o[s], M[s], fd);
        for (int i = 0; i < n; ++i) {
            const int64_t row = base + i;
            const float tf = trial_fit ? trial_fit[row] : (float)fd[i];
            const int win = tf < fit_in[row];
            if (sel_out) sel_out[row] = (uint8_t)win;
            if (trial_out) memcpy(trial_out + (size_t)row * l, cand + (size_t)i * l, sizeof(float) * (size_t)dim);
            memcpy(pop_out + (size_t)row * l, win ? cand + (size_t)i * l : pin + (size_t)i * l,
                   sizeof(float) * (size_t)dim);
            fit_out[row] = win ? tf : fit_in[row];
        }
        free(fd);
        free(cand);
        free(perm);
    }
    return err;
}

/* ---- ring migration ------------------------------------------------------------------ */

/* k best (ascending (f,row)) and k worst (descending (f,row)) local indices of a segment. */
static void seg_extremes(const float *fit, int64_t base, int n, int k, int *best, int *worst)
{
    unsigned char *taken = (unsigned char *)calloc((size_t)n, 1);
    for (int t = 0; t < k; ++t) {
        int b = -1;
        for (int i = 0; i < n; ++i) {
            if (taken[i]) continue;
            if (b < 0) { b = i; continue; }
            const float fi = nan_as_inf(fit[base + i]), fb = nan_as_inf(fit[base + b]);
            if (fi < fb) b = i; /* ties keep the lower row */
        }
        taken[b] = 1;
        best[t] = b;
    }
    memset(taken, 0, (size_t)n);
    for (int t = 0; t < k; ++t) {
        int w = -1;
        for (int i = n - 1; i >= 0; --i) {
            if (taken[i]) continue;
            if (w < 0) { w = i; continue; }
            const float fi = nan_as_inf(fit[base + i]), fw = nan_as_inf(fit[base + w]);
            if (fi > fw) w = i; /* ties keep the higher row */
        }
        taken[w] = 1;
        worst[t] = w;
    }
    free(taken);
}

void speo_oracle_ring_migrate(int n_segs, const int64_t *row0, const int *P, const int *D,
                              const int *ld, const int *ring_next, int k, float *pop, float *fit)
{
    int *best = (int *)malloc(sizeof(int) * (size_t)n_segs * k);
    int *worst = (int *)malloc(sizeof(int) * (size_t)n_segs * k);
    float *stage = NULL;
    int maxld = 0;
    for (int s = 0; s < n_segs; ++s) if (ld[s] > maxld) maxld = ld[s];
    stage = (float *)malloc(sizeof(float) * (size_t)n_segs * k * (maxld + 1));
    for (int s = 0; s < n_segs; ++s) {
        seg_extremes(fit, row0[s], P[s], k, best + s * k, worst + s * k);
        for (int t = 0; t < k; ++t) {
            const int64_t row = row0[s] + best[s * k + t];
            float *dst = stage + ((size_t)s * k + t) * (maxld + 1);
            memcpy(dst, pop + (size_t)row * ld[s], sizeof(float) * (size_t)D[s]);
            dst[maxld] = fit[row];
        }
    }
    for (int s = 0; s < n_segs; ++s) {
        const int t_seg = ring_next[s];
        if (t_seg < 0) continue;
        for (int t = 0; t < k; ++t) {
            const int64_t row = row0[t_seg] + worst[t_seg * k + t];
            const float *src = stage + ((size_t)s * k + t) * (maxld + 1);
            memcpy(pop + (size_t)row * ld[t_seg], src, sizeof(float) * (size_t)D[t_seg]);
            fit[row] = src[maxld];
        }
    }
    free(stage);
    free(best);
    free(worst);
}

/* ---- CPU baseline (FP64 island loop, threads over islands) ------------------------------ */
typedef struct {
    int i0, i1, P, D, ld, func_id, gens;
    double F, CR, lb, ub;
    const double *o, *M;
    uint64_t seed;
    uint32_t gen0;
    double *pop, *fit;
    int err;
} island_job;

static void *island_worker(void *arg)
{
    island_job *j = (island_job *)arg;
    const int P = j->P, l = j->ld, D = j->D;
    double *cand = (double *)calloc((size_t)P * l, sizeof(double));
    double *cfit = (double *)malloc(sizeof(double) * (size_t)P);
    int *perm = (int *)malloc(sizeof(int) * (size_t)P);
    for (int i = 0; i < P; ++i) perm[i] = i;
    const int st = 4;
    for (int isl = j->i0; isl < j->i1; ++isl) {
        double *pop = j->pop + (size_t)isl * P * l;
        double *fit = j->fit + (size_t)isl * P;
        for (int g = 0; g < j->gens; ++g) {
            speo_oracle_draws dr;
            memset(&dr, 0, sizeof dr);
            dr.key[0] = (uint32_t)j->seed;
            dr.key[1] = (uint32_t)(j->seed >> 32);
            dr.gen = j->gen0 + (uint32_t)g;
            dr.pos0 = (int64_t)isl * P;
            j->err |= speo_oracle_de_generate_f64(cand, pop, l, D, P, 1, perm, &j->CR, &j->F, &st,
                                                  NULL, j->lb, j->ub, &dr);
            for (int i = 0; i < P; ++i)
                cfit[i] = speo_oracle_objective_f64(j->func_id, cand + (size_t)i * l, j->o, j->M, D);
            speo_oracle_select_f64(pop, fit, cand, cfit, P, l, D, NULL);
        }
    }
    free(cand);
    free(cfit);
    free(perm);
    return NULL;
}

static void ring_migrate_f64(int n, int P, int D, int ld, int k, double *pop, double *fit)
{
    float *ff = (float *)malloc(sizeof(float) * (size_t)n * P);
    int *best = (int *)malloc(sizeof(int) * (size_t)n * k), *worst = (int *)malloc(sizeof(int) * (size_t)n * k);
    double *stage = (double *)malloc(sizeof(double) * (size_t)n * k * (D + 1));
    for (int i = 0; i < n * P; ++i) ff[i] = (float)fit[i];
    for (int s = 0; s < n; ++s) {
        seg_extremes(ff, (int64_t)s * P, P, k, best + s * k, worst + s * k);
        for (int t = 0; t < k; ++t) {
            const size_t row = (size_t)s * P + best[s * k + t];
            memcpy(stage + ((size_t)s * k + t) * (D + 1), pop + row * ld, sizeof(double) * (size_t)D);
            stage[((size_t)s * k + t) * (D + 1) + D] = fit[row];
        }
    }
    for (int s = 0; s < n; ++s) {
        const int d = (s + 1) % n;
        for (int t = 0; t < k; ++t) {
            const size_t row = (size_t)d * P + worst[d * k + t];
            memcpy(pop + row * ld, stage + ((size_t)s * k + t) * (D + 1), sizeof(double) * (size_t)D);
            fit[row] = stage[((size_t)s * k + t) * (D + 1) + D];
        }
    }
    free(ff); free(best); free(worst); free(stage);
}

int64_t speo_oracle_run_islands_f64(int n_islands, int P, int D, int ld, int func_id,
                                    double F, double CR, double lb, double ub,
                                    const double *o, const double *M, uint64_t seed,
                                    uint32_t gen0, int gens, int interval, int k_migrate,
                                    double *pop, double *fit, int threads)
{
    if (threads < 1) threads = 1;
    if (threads > n_islands) threads = n_islands;
    int done = 0;
    while (done < gens) {
        /* run up to the next migration point (generation counts are 1-based) */
        int g_abs = (int)gen0 + done;
        int until = gens - done;
        if (interval > 0) {
            const int to_next = interval - (g_abs % interval);
            if (to_next < until) until = to_next;
        }
        pthread_t *tid = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)threads);
        island_job *jobs = (island_job *)malloc(sizeof(island_job) * (size_t)threads);
        for (int t = 0; t < threads; ++t) {
            island_job *j = &jobs[t];
            j->i0 = (int)((int64_t)n_islands * t / threads);
            j->i1 = (int)((int64_t)n_islands * (t + 1) / threads);
            j->P = P; j->D = D; j->ld = ld; j->func_id = func_id; j->gens = until;
            j->F = F; j->CR = CR; j->lb = lb; j->ub = ub; j->o = o; j->M = M;
            j->seed = seed; j->gen0 = (uint32_t)g_abs; j->pop = pop; j->fit = fit; j->err = 0;
            pthread_create(&tid[t], NULL, island_worker, j);
        }
        for (int t = 0; t < threads; ++t) pthread_join(tid[t], NULL);
        free(tid);
        free(jobs);
        done += until;
        if (interval > 0 && ((int)gen0 + done) % interval == 0 && k_migrate > 0 && n_islands > 1)
            ring_migrate_f64(n_islands, P, D, ld, k_migrate, pop, fit);
    }
    return (int64_t)gens * n_islands * P;
}

/* ---- surrogate MLP --------------------------------------------------------------------- */
int speo_oracle_mlp_nparams(int din, int h) { return h * din + h + h * h + h + h + 1; }

typedef struct { const float *W1, *b1, *W2, *b2, *w3, *b3; } mlp_view;

static mlp_view mlp_split(const float *theta, int din, int h)
{
    mlp_view v;
    v.W1 = theta;
    v.b1 = v.W1 + (size_t)h * din;
    v.W2 = v.b1 + h;
    v.b2 = v.W2 + (size_t)h * h;
    v.w3 = v.b2 + h;
    v.b3 = v.w3 + h;
    return v;
}

/* forward of one row; keeps pre-activations z1, z2 (length h) */
static double mlp_row(mlp_view p, int din, int h, float in_scale, const float *x, double *z1, double *z2)
{
    for (int j = 0; j < h; ++j) {
        double a = p.b1[j];
        for (int k = 0; k < din; ++k) a += (double)p.W1[(size_t)j * din + k] * ((double)x[k] * (double)in_scale);
        z1[j] = a;
    }
    for (int j = 0; j < h; ++j) {
        double a = p.b2[j];
        for (int k = 0; k < h; ++k) a += (double)p.W2[(size_t)j * h + k] * (z1[k] > 0 ? z1[k] : 0.0);
        z2[j] = a;
    }
    double y = p.b3[0];
    for (int j = 0; j < h; ++j) y += (double)p.w3[j] * (z2[j] > 0 ? z2[j] : 0.0);
    return y;
}

void speo_oracle_mlp_forward(const float *theta, int din, int h, float in_scale, const float *X, int n, int ldx,
                             double *y)
{
    mlp_view p = mlp_split(theta, din, h);
    double *z1 = (double *)malloc(sizeof(double) * (size_t)h), *z2 = (double *)malloc(sizeof(double) * (size_t)h);
    for (int i = 0; i < n; ++i) y[i] = mlp_row(p, din, h, in_scale, X + (size_t)i * ldx, z1, z2);
    free(z1);
    free(z2);
}

double speo_oracle_mlp_loss_grad(const float *theta, int din, int h, float in_scale, const float *X, int n, int ldx,
                                 const float *t, double *grad)
{
    mlp_view p = mlp_split(theta, din, h);
    const int np = speo_oracle_mlp_nparams(din, h);
    double *gW1 = grad, *gb1 = gW1 + (size_t)h * din, *gW2 = gb1 + h, *gb2 = gW2 + (size_t)h * h, *gw3 = gb2 + h,
           *gb3 = gw3 + h;
    memset(grad, 0, sizeof(double) * (size_t)np);
    double *z1 = (double *)malloc(sizeof(double) * (size_t)h), *z2 = (double *)malloc(sizeof(double) * (size_t)h);
    double *dz2 = (double *)malloc(sizeof(double) * (size_t)h), *dz1 = (double *)malloc(sizeof(double) * (size_t)h);
    double loss = 0.0;
    for (int i = 0; i < n; ++i) {
        const float *x = X + (size_t)i * ldx;
        const double y = mlp_row(p, din, h, in_scale, x, z1, z2);
        const double e = y - (double)t[i];
        loss += e * e;
        const double dy = 2.0 * e / n;
        gb3[0] += dy;
        for (int j = 0; j < h; ++j) {
            const double a2 = z2[j] > 0 ? z2[j] : 0.0;
            gw3[j] += dy * a2;
            dz2[j] = z2[j] > 0 ? dy * p.w3[j] : 0.0;
        }
        for (int j = 0; j < h; ++j) {
            gb2[j] += dz2[j];
            for (int k = 0; k < h; ++k) gW2[(size_t)j * h + k] += dz2[j] * (z1[k] > 0 ? z1[k] : 0.0);
        }
        for (int k = 0; k < h; ++k) {
            double a = 0.0;
            for (int j = 0; j < h; ++j) a += dz2[j] * (double)p.W2[(size_t)j * h + k];
            dz1[k] = z1[k] > 0 ? a : 0.0;
        }
        for (int j = 0; j < h; ++j) {
            gb1[j] += dz1[j];
            for (int k = 0; k < din; ++k) gW1[(size_t)j * din + k] += dz1[j] * ((double)x[k] * (double)in_scale);
        }
    }
    free(z1); free(z2); free(dz1); free(dz2);
    return loss / n;
}

void speo_oracle_adam(float *theta, float *m, float *v, const float *g, int n, float lr, float beta1, float beta2,
                      float eps, int step)
{
    const float c1 = 1.0f - powf(beta1, (float)step), c2 = 1.0f - powf(beta2, (float)step);
    for (int i = 0; i < n; ++i) {
        m[i] = beta1 * m[i] + (1.0f - beta1) * g[i];
        v[i] = beta2 * v[i] + (1.0f - beta2) * g[i] * g[i];
        const float mh = m[i] / c1, vh = v[i] / c2;
        theta[i] -= lr * mh / (sqrtf(vh) + eps);
    }
}
