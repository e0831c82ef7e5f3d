// Table-driven FP64 elementary functions of the device code, each after
// P. T. P. Tang's table-driven method (argument reduced against a table
// point, short Taylor polynomial for the remainder, product with the
// tabulated value).  Checked against the host's libm by hbt_check_math
// (include/hbt_check.h, tests/test_math_gpu.py).
#pragma once

// Table of cos and sin of 2 pi k / 512, k = 0..511, for table_cos, filled
// by each CTA of the FP64-form same-event kernels.
constexpr int COS_TABLE = 512;
__device__ __forceinline__ void fill_cos_table(double2 *cs) {
    for (int k = threadIdx.x; k < COS_TABLE; k += blockDim.x) {
        double sn, cn;
        sincospi(k / 256.0, &sn, &cn);
        cs[k] = make_double2(cn, sn);
    }
}

// cos(x), table-driven (the argument reduction of P. T. P. Tang's
// table-driven elementary functions): x = k (2 pi / 512) + d with
// k = rint(x 512 / 2 pi) and d from a two-part split of 2 pi / 512 (the
// leading part has 26 significant bits, so k times it is exact for
// |k| < 2^27), |d| <= pi / 512 = 6.2e-3; then
//   cos x = cos(2 pi k / 512) cos d - sin(2 pi k / 512) sin d
// with cos d to d^4 and sin d to d^5 from their Taylor series (truncation
// below 1e-16 and 1e-18).  |x| >= 2^20 (never on this path: |q.dx| / hbarC
// is a few hundred at most) falls back to cos().
__device__ __forceinline__ double table_cos(const double2 *cs, double x) {
    if (!(fabs(x) < 1048576.0)) return cos(x);
    const double kd = rint(x * 81.48733086305042);          // 512 / (2 pi)
    double d = __fma_rn(-kd, 0.01227184641174972, x);       // leading part
    d = __fma_rn(-kd, -1.086645907356806e-10, d);           // 2 pi / 512 - leading part
    const int k = __double2int_rn(kd) & (COS_TABLE - 1);
    const double d2 = d * d;
    const double cd = __fma_rn(d2, __fma_rn(d2, 1.0 / 24.0, -0.5), 1.0);
    const double sd = d * __fma_rn(d2, __fma_rn(d2, 1.0 / 120.0, -1.0 / 6.0), 1.0);
    const double2 e = cs[k];
    return __fma_rn(e.x, cd, -(e.y * sd));
}

// Table of 2^(j / 64), j = 0..63, for table_exp, filled by each CTA that
// uses it.
constexpr int EXP_TABLE = 64;
__device__ __forceinline__ void fill_exp_table(double *t) {
    for (int k = threadIdx.x; k < EXP_TABLE; k += blockDim.x) t[k] = exp2(k / 64.0);
}

// exp(x), table-driven: n = rint(x 64 / ln 2), x = n (ln 2 / 64) + r with r
// from a two-part split of ln 2 / 64 (the leading part has 28 significant
// bits, so n times it is exact for |n| < 2^25), |r| <= ln 2 / 128 = 5.4e-3;
// with j = n mod 64 and m = floor(n / 64),
//   exp x = 2^m 2^(j / 64) (1 + r + r^2 / 2 + ... + r^5 / 120)
// (truncation below 4e-17 relative), 2^m added to the exponent field.
// Outside |x| < 700 (where 2^m could leave the normal range) it calls exp().
__device__ __forceinline__ double table_exp(const double *t, double x) {
    if (!(fabs(x) < 700.0)) return exp(x);
    const double nd = rint(x * 92.33248261689366);             // 64 / ln 2
    double r = __fma_rn(-nd, 0x1.62e42ff000000p-7, x);         // leading part
    r = __fma_rn(-nd, -6.563929801064195e-13, r);              // ln 2 / 64 - leading part
    const int n = __double2int_rn(nd);
    double p = __fma_rn(r, 1.0 / 120.0, 1.0 / 24.0);
    p = __fma_rn(p, r, 1.0 / 6.0);
    p = __fma_rn(p, r, 0.5);
    p = __fma_rn(p, r, 1.0);
    p = __fma_rn(p, r, 1.0);
    const double v = t[n & (EXP_TABLE - 1)] * p;
    return __hiloint2double(__double2hiint(v) + ((n >> 6) * (1 << 20)), __double2loint(v));
}
