/*
 * oracle_de_impl.h -- precision-generic body of the DE generate restatement.
 * TEST INFRASTRUCTURE ONLY (see speo_oracle.h). Included twice by speo_oracle.c with
 *   REAL = float  / FMA = fmaf / SFX = _f32
 *   REAL = double / FMA = fma  / SFX = _f64
 * Restates global_DE_GenerateNewPopulation (kernel_DE_CUDA.cu:172-289) and
 * device_CheckBound (kernel_DE_CUDA.cu:160-170).
 */

/* device_CheckBound, kernel_DE_CUDA.cu:160-170: reflect until inside [lb, ub]. The
 * reference loops forever on +-inf; here the loop stops after SPEO_BOUND_ITERS rounds,
 * sets SPEO_DEVERR_BOUND_LIMIT and returns lb (same bound in the CUDA kernel). */
static inline REAL CAT(check_bound, SFX)(REAL v, REAL lb, REAL ub, int *err)
{
    int it = 0;
    while ((v < lb) || (v > ub)) {
        if (v < lb) v = lb + (lb - v);
        if (v > ub) v = ub - (v - ub);
        if (++it >= SPEO_BOUND_ITERS) { *err |= SPEO_DEVERR_BOUND_LIMIT; v = lb; break; }
    }
    return v;
}

/* One mutant element for strategy `st` (kernel_DE_CUDA.cu:243-276). Terms are added left to
 * to right, each F*(a-b) fused into the running sum: v = fma(F, a-b, v). */
static inline REAL CAT(mutant, SFX)(int st, REAL F, REAL xi, REAL xb, const REAL *xr)
{
    REAL v;
    switch (st) {
    case 0: v = FMA(F, xr[0] - xr[1], xi); break;
    case 1: v = FMA(F, xr[0] - xr[1], xi); v = FMA(F, xr[2] - xr[3], v); break;
    case 2: v = FMA(F, xb - xi, xi); v = FMA(F, xr[0] - xr[1], v); break;
    case 3: v = FMA(F, xb - xi, xi); v = FMA(F, xr[0] - xr[1], v); v = FMA(F, xr[1] - xr[2], v); break;
    case 4: v = FMA(F, xr[1] - xr[2], xr[0]); break;
    case 5: v = FMA(F, xr[1] - xr[2], xr[0]); v = FMA(F, xr[3] - xr[4], v); break;
    case 6: v = FMA(F, xr[0] - xr[1], xb); break;
    case 7: v = FMA(F, xr[0] - xr[1], xb); v = FMA(F, xr[2] - xr[3], v); break;
    case 8: v = FMA(F, xr[0] - xi, xi); v = FMA(F, xr[1] - xr[2], v); break;
    default: v = xi; break;
    }
    return v;
}

int CAT(speo_oracle_de_generate, SFX)(REAL *cand, const REAL *pop, int ld, int dim,
                                      int island_size, int subisland_num, const int *perm,
                                      const REAL *de_CR, const REAL *de_F, const int *de_strategy,
                                      const int *best_id, REAL lb, REAL ub,
                                      const speo_oracle_draws *draws)
{
    int err = 0;
    const int S = island_size / subisland_num;           /* kernel_DE_CUDA.cu:178 */
    const int np2 = next_pow2_dim(dim);                   /* kernel_DE_CUDA.cu:179 */
    const int loop_times = np2 / 32;                      /* kernel_DE_CUDA.cu:180 */
    for (int pos = 0; pos < island_size; ++pos) {
        draw_cursor cur;
        cursor_begin(&cur, draws, pos);
        const int sel = perm[pos];                        /* kernel_DE_CUDA.cu:177 */
        const int isl = pos / S;                          /* kernel_DE_CUDA.cu:181 */
        int r[5];
        /* kernel_DE_CUDA.cu:187-212, including its sequential (not full) distinctness check */
        for (int i = 0; i < 5; ++i) {
            r[i] = draw_index(&cur, S, (int)sizeof(REAL));
            if (r[i] == S) r[i]--;
            for (int j = 0; j < i; ++j) {
                int guard = 0;
                while (r[i] == r[j]) {
                    r[i] = draw_index(&cur, S, (int)sizeof(REAL));
                    if (++guard >= SPEO_REDRAW_ITERS) { err |= SPEO_DEVERR_REDRAW_LIMIT; break; }
                }
            }
            if (r[i] == S) r[i]--;
        }
        for (int i = 0; i < 5; ++i) r[i] = perm[r[i] + isl * S];   /* :213-216 */
        const int jrand = draw_index(&cur, dim, (int)sizeof(REAL)); /* :218 */
        const REAL F = de_F[isl], CR = de_CR[isl];
        const int st = de_strategy[isl];
        const int b = best_id ? best_id[isl] : sel;
        const REAL *xi = pop + (size_t)sel * ld;
        const REAL *xb = pop + (size_t)b * ld;
        for (int c = 0; c < loop_times; ++c) {                       /* :229-287 */
            for (int lane = 0; lane < 32; ++lane) {
                const int e = lane + 32 * c;
                const double u = draw_cr(&cur, draws, pos, e, lane);
                if (e >= dim) continue;
                REAL v;
                if (e == jrand || (REAL)u < CR) {
                    REAL xr[5];
                    for (int i = 0; i < 5; ++i) xr[i] = pop[(size_t)r[i] * ld + e];
                    v = CAT(mutant, SFX)(st, F, xi[e], xb[e], xr);
                } else {
                    v = xi[e];
                }
                v = CAT(check_bound, SFX)(v, lb, ub, &err);
                cand[(size_t)sel * ld + e] = v;
            }
        }
        cursor_end(&cur, draws, pos);
    }
    return err;
}

void CAT(speo_oracle_select, SFX)(REAL *pop, REAL *pop_fit, const REAL *cand, const REAL *cand_fit,
                                  int n, int ld, int dim, uint8_t *sel)
{
    /* kernel_DE_CUDA.cu:305-327 */
    for (int i = 0; i < n; ++i) {
        const int win = cand_fit[i] < pop_fit[i];
        if (sel) sel[i] = (uint8_t)win;
        if (win) {
            memcpy(pop + (size_t)i * ld, cand + (size_t)i * ld, sizeof(REAL) * (size_t)dim);
            pop_fit[i] = cand_fit[i];
        }
    }
}
