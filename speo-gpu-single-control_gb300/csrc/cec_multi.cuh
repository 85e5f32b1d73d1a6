// cec_multi.cuh -- CEC2014 hybrid (17-22) and composition (23-30) functions: their tables and
// the per-row pieces the evaluation kernels share.
//
// Hybrid functions hf01..hf06 (CUDA_EA_library/CEC2014.cc:954-1207): z = M (x - o), y_i =
// z[S_i - 1] (S 1-based), y cut into groups of ceil(gp_g D) coordinates (the last takes the
// rest); group g is the body of id fid_g on y_g * rate(fid_g) + fixed shift(fid_g), with the
// group's own length; f = sum over the groups.
// Composition functions cf01..cf08 (CEC2014.cc:1209-1369): component c is the body of fid_c on
// rate(fid_c) M_c (x - o_c) (+ fixed shift; cf01's fifth and cf02's first component without
// M_c), rescaled as num * f / den; cf07 / cf08 take the hybrids hf01-03 / hf04-06 on (o_c, M_c,
// S_c). cf_cal (:1481-1520) adds bias_c = 100 c and mixes the components with weights
// w_c = S_c^-1/2 exp(-S_c / (2 D delta_c^2)), S_c = sum_j (x_j - o_cj)^2.
// The bodies are those of the single-component ids (schwefel = 10, rastrigin = 8, with those
// ids' rates and fixed shifts), so every piece runs through RowAcc / row_push / row_finish.
#pragma once

#include "common.cuh"

namespace speo {

__host__ __device__ __forceinline__ bool func_multi(int f) { return f >= 17 && f <= 30; }
__host__ __device__ __forceinline__ bool func_composition(int f) { return f >= 23 && f <= 30; }
__host__ __device__ __forceinline__ bool func_any(int f) { return func_supported(f) || func_multi(f); }
// Components: one shift / matrix (/ shuffle) each (CEC2014.cc:306-333).
__host__ __device__ __forceinline__ int func_components(int f)
{
    switch (f) {
    case 23: case 26: case 27: case 28: return 5;
    case 24: case 25: case 29: case 30: return 3;
    default: return 1;
    }
}
__host__ __device__ __forceinline__ bool func_uses_shuffle(int f) { return (f >= 17 && f <= 22) || f == 29 || f == 30; }

// ---- hybrids: h = 0..5 for hf01..hf06 ---------------------------------------------------------
__host__ __device__ __forceinline__ int hybrid_groups(int h) { return h < 2 ? 3 : h < 4 ? 4 : 5; }
__host__ __device__ __forceinline__ double hybrid_gp(int h, int g)
{
    switch (h) {
    case 0: case 1: return g < 2 ? 0.3 : 0.4;
    case 2: case 3: return g < 2 ? 0.2 : 0.3;
    case 4: return g == 0 ? 0.1 : g < 4 ? 0.2 : 0.3;
    default: return g == 0 ? 0.1 : 0.2;
    }
}
__host__ __device__ __forceinline__ int hybrid_fid(int h, int g)
{
    constexpr int8_t t[6][5] = {{10, 8, 1, 0, 0},   {2, 14, 8, 0, 0},    {7, 6, 4, 16, 0},
                                {14, 3, 15, 8, 0},  {16, 14, 4, 10, 1},  {12, 13, 15, 10, 5}};
    return t[h][g];
}
// Group g's length at dimension D: ceil(gp_g D) in double for all but the last, which takes the
// rest (CEC2014.cc:961-972). Returns false if some group would be empty (D too small).
__host__ __device__ __forceinline__ bool hybrid_split(int h, int D, int &start, int &len, int g)
{
    const int n = hybrid_groups(h);
    int s = 0;
    for (int i = 0; i < g; ++i) s += (int)ceil(hybrid_gp(h, i) * (double)D);
    start = s;
    len = g < n - 1 ? (int)ceil(hybrid_gp(h, g) * (double)D) : D - s;
    return len >= 1 && start + len <= D;
}
__host__ __device__ __forceinline__ bool hybrid_dim_ok(int h, int D)
{
    for (int g = 0; g < hybrid_groups(h); ++g) {
        int s, l;
        if (!hybrid_split(h, D, s, l, g)) return false;
    }
    return true;
}
// The hybrid index (0..5) of component c of f, or -1.
__host__ __device__ __forceinline__ int multi_hybrid(int f, int c)
{
    if (f >= 17 && f <= 22) return f - 17;
    if (f == 29) return c;
    if (f == 30) return 3 + c;
    return -1;
}
// Whether every hybrid of f is defined at dimension D.
__host__ __device__ __forceinline__ bool multi_dim_ok(int f, int D)
{
    for (int c = 0; c < func_components(f); ++c) {
        const int h = multi_hybrid(f, c);
        if (h >= 0 && !hybrid_dim_ok(h, D)) return false;
    }
    return true;
}

// ---- compositions 23-28: component c ---------------------------------------------------------
struct CompPiece {
    int fid;      // body
    bool rotated;
    double num, den;  // fit = num * f / den; den = 0: unscaled
};
__host__ __device__ __forceinline__ CompPiece comp_piece(int f, int c)
{
    switch (f) {
    case 23: {  // cf01
        constexpr int8_t fid[5] = {4, 1, 2, 3, 1};
        constexpr double den[5] = {1e+4, 1e+10, 1e+30, 1e+10, 1e+10};
        return {fid[c], c != 4, 10000.0, den[c]};
    }
    case 24: {  // cf02
        constexpr int8_t fid[3] = {10, 8, 14};
        return {fid[c], c != 0, 0.0, 0.0};
    }
    case 25: {  // cf03
        constexpr int8_t fid[3] = {10, 8, 1};
        constexpr double den[3] = {4e+3, 1e+3, 1e+10};
        return {fid[c], true, 1000.0, den[c]};
    }
    case 26: {  // cf04
        constexpr int8_t fid[5] = {10, 13, 1, 6, 7};
        constexpr double den[5] = {4e+3, 1e+3, 1e+10, 400.0, 100.0};
        return {fid[c], true, 1000.0, den[c]};
    }
    case 27: {  // cf05
        constexpr int8_t fid[5] = {14, 8, 10, 6, 1};
        constexpr double den[5] = {1000.0, 1e+3, 4e+3, 400.0, 1e+10};
        return {fid[c], true, 10000.0, den[c]};
    }
    default: {  // 28, cf06
        constexpr int8_t fid[5] = {15, 13, 10, 16, 1};
        constexpr double den[5] = {4e+3, 1e+3, 4e+3, 2e+7, 1e+10};
        return {fid[c], true, 10000.0, den[c]};
    }
    }
}
__host__ __device__ __forceinline__ double comp_delta(int f, int c)
{
    switch (f) {
    case 23: case 28: return 10.0 * (c + 1);
    case 24: return 20.0;
    case 26: return 10.0;
    case 27: return c < 3 ? 10.0 : 20.0;
    default: return 10.0 + 20.0 * c;  // 25, 29, 30: 10, 30, 50
    }
}

template <typename T> __device__ __forceinline__ T rate_of(int fid)
{
    return sizeof(T) == 4 ? (T)func_scale(fid) : (T)func_scale_f64(fid);
}

// One hybrid of one row: z (the rotated, unshuffled row, D values in shared memory), s0 the
// 0-based shuffle (shared memory). All lanes call it together; the value is valid on every lane.
template <typename T>
__device__ __noinline__ T hybrid_row_warp(const T *z, const int *s0, int h, int D, int lane)
{
    T total = T(0);
    const int n = hybrid_groups(h);
    for (int g = 0; g < n; ++g) {
        int g0, len;
        if (!hybrid_split(h, D, g0, len, g)) return __longlong_as_double(0x7ff8000000000000LL);
        const int fid = hybrid_fid(h, g);
        const T rate = rate_of<T>(fid), fs = func_fixed_shift<T>(fid);
        RowAcc<T> a;
        for (int j = lane; j < len; j += 32) {
            const int jn = j + 1 < len ? j + 1 : 0;
            row_push(a, fid, j, z[s0[g0 + j]] * rate + fs, z[s0[g0 + jn]] * rate + fs, len);
        }
        a.s1 = warp_sum(a.s1);
        a.s2 = warp_sum(a.s2);
        a.p = warp_prod(a.p);
        total += row_finish(a, fid, len);
    }
    return total;
}

// cf_cal (CEC2014.cc:1481-1520): sum_c w_c / w_sum * (fit_c + 100 c). FP64 follows the reference
// formula (1e99 for S_c = 0, equal weights when every w_c underflows); FP32 forms the same
// normalised weights from logarithms, exp(l_c - max l), l_c = -ln(S_c) / 2 - S_c / (2 D delta_c^2),
// so that weights the reference keeps (FP64 underflows only past S_c / (2 D delta^2) ~ 745) do
// not underflow in binary32; S_c = 0 gives that component (or those components, equally) weight 1.
template <typename T>
__device__ __forceinline__ T comp_combine(int f, int D, const T *fit, const T *S)
{
    const int n = func_components(f);
    if constexpr (sizeof(T) == 8) {
        double w[5], w_max = 0.0, w_sum = 0.0;
        for (int c = 0; c < n; ++c) {
            const double dl = comp_delta(f, c);
            w[c] = S[c] != 0.0 ? pow(1.0 / S[c], 0.5) * exp(-S[c] / 2.0 / D / (dl * dl)) : 1.0e99;
            if (w[c] > w_max) w_max = w[c];
        }
        for (int c = 0; c < n; ++c) w_sum += w[c];
        if (w_max == 0.0) {
            for (int c = 0; c < n; ++c) w[c] = 1.0;
            w_sum = n;
        }
        double r = 0.0;
        for (int c = 0; c < n; ++c) r += w[c] / w_sum * (fit[c] + 100.0 * c);
        return r;
    } else {
        int zeros = 0;
        for (int c = 0; c < n; ++c) zeros += S[c] == 0.f;
        float r = 0.f;
        if (zeros) {
            for (int c = 0; c < n; ++c)
                if (S[c] == 0.f) r += (fit[c] + 100.f * c) / (float)zeros;
            return r;
        }
        float l[5], m = -__int_as_float(0x7f800000);
        for (int c = 0; c < n; ++c) {
            const float dl = (float)comp_delta(f, c);
            l[c] = -0.5f * logf(S[c]) - S[c] / (2.f * (float)D * dl * dl);
            m = fmaxf(m, l[c]);
        }
        float e[5], es = 0.f;
        for (int c = 0; c < n; ++c) { e[c] = expf(l[c] - m); es += e[c]; }
        for (int c = 0; c < n; ++c) r += e[c] / es * (fit[c] + 100.f * c);
        return r;
    }
}

}  // namespace speo
