// Table-driven FP64 elementary functions of the device code, each after
// P. T. P. Tang's table-driven method (argument reduced against a table
// point, short Taylor polynomial for the remainder, product with the
// tabulated value).  Checked against the host's libm by hbt_check_math
// (include/hbt_check.h, tests/test_math_gpu.py).
#pragma once

#include <cmath>
#include <cstring>

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

// Constants of table_cos for one scale h: it returns cos(h ph) of a phase
// ph (h = 1 / hbarC for the pair numerators, h = 1 for a plain cos), with
// the product h ph never rounded.  Filled on the host by make_cos_scale.
struct CosScale {
    double c1;       // h 512 / (2 pi): table points per unit of ph
    double s1, s2;   // (2 pi / 512) / h = s1 + s2, s1 with 26 significant bits
    double h;        // h, and the Taylor coefficients of cos(h d'), sin(h d')
    double c2, c4;   //   -h^2 / 2, h^4 / 24
    double s3, s5;   //   -h^3 / 6, h^5 / 120
    unsigned lim_hi; // high word of L, the largest power of two with L c1 < 2^27
};

// (2 pi / 512) / h is formed in double-double arithmetic (2 pi as a
// two-part constant, the division's remainder taken exactly with an FMA),
// then split into s1, its leading 26 significant bits (the low 27 bits of
// the significand cleared, so that k s1 is exact for |k| < 2^27), and the
// rest s2: s1 + s2 holds the step to about 2^-79 relative.
static inline CosScale make_cos_scale(double h) {
    CosScale k;
    const double t_hi = 6.283185307179586 / 512.0, t_lo = 2.4492935982947064e-16 / 512.0;
    const double q1 = t_hi / h;
    const double q2 = (std::fma(-q1, h, t_hi) + t_lo) / h;
    unsigned long long bits;
    std::memcpy(&bits, &q1, sizeof bits);
    bits &= ~((1ull << 27) - 1);
    std::memcpy(&k.s1, &bits, sizeof bits);
    k.s2 = (q1 - k.s1) + q2;
    k.c1 = h * (512.0 / 6.283185307179586);
    k.h = h;
    k.c2 = -0.5 * h * h;
    k.c4 = h * h * h * h / 24.0;
    k.s3 = -h * h * h / 6.0;
    k.s5 = h * h * h * h * h / 120.0;
    int m = 40;
    while (m > -40 && std::ldexp(1.0, m) * k.c1 >= 134217728.0) m--;
    k.lim_hi = (unsigned)(1023 + m) << 20;
    return k;
}

// cos(h ph), table-driven (the argument reduction of P. T. P. Tang's
// table-driven elementary functions, done on ph itself): ph = k s + d' with
// s = (2 pi / 512) / h, k the integer nearest to ph c1 (the exact product,
// rounded once by an FMA against 1.5 2^52, whose low word then holds k) and
// d' from the two-part split of s, so that d = h d' is at most pi / 512 =
// 6.2e-3 in magnitude; then
//   cos(h ph) = cos(2 pi k / 512) cos d - sin(2 pi k / 512) sin d
// with cos d to d^4 and sin d to d^5 from their Taylor series in d'
// (truncation below 1e-16 and 1e-18).  |ph| >= L (k could reach 2^27;
// never on the pair path, where |q.dx| / hbarC is a few hundred at most) and
// NaN fall back to cos(h ph).
__device__ __forceinline__ double table_cos(const double2 *cs, const CosScale &k, double ph) {
    if (!(((unsigned)__double2hiint(ph) & 0x7fffffffu) < k.lim_hi)) return cos(k.h * ph);
    const double t = __fma_rn(ph, k.c1, 6755399441055744.0);  // 1.5 2^52
    const double kd = t - 6755399441055744.0;
    double d = __fma_rn(-kd, k.s1, ph);
    d = __fma_rn(-kd, k.s2, d);
    const int j = __double2loint(t) & (COS_TABLE - 1);
    const double d2 = d * d;
    const double cd = __fma_rn(d2, __fma_rn(d2, k.c4, k.c2), 1.0);
    const double sd = d * __fma_rn(d2, __fma_rn(d2, k.s5, k.s3), k.h);
    const double2 e = cs[j];
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
