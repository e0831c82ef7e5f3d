// Screened pair binning of one tile pair (device code shared by the grid
// kernels of hbt_fast.cu and the persistent batch kernel of hbt_batch.cu).
//
// GB300 runs FP64 at 1/58 of its FP32 rate, so every pair is first screened
// in FP32 and only the pairs that are binned pay for more work:
//
//  A. Prefilter (every pair, ~30 FP32 operations).  Rejects only pairs
//     certainly outside the window: q_out^2 + q_side^2 = q_x^2 + q_y^2 in
//     real arithmetic, so a binned pair has q_x^2 + q_y^2 <= 2 Q^2, and
//     |q_long| <= Q (with the boost: |S_E dq_z - S_z dq_E| <= Q sqrt(M^2),
//     no division), Q = max(-lo, hi); each test carries the FP32 rounding of
//     its inputs (2.01 u per sum) and a relative margin.  Other pairs are
//     queued.
//  B. Window screen and bins, per warp on 32 queued pairs with all lanes
//     active.  From FP32 copies of the momenta: K_perp^2, q_out, q_side,
//     q_long and a rigorous bound on how far each lies from the value the
//     reference computes in FP64 (error analysis below).  A pair is dropped
//     when a window check fails by more than its bound; the bin indices are
//     decided in FP32 when every truncation is farther from its edge than
//     its bound (they are then the reference's indices exactly), K_phi
//     likewise with atan2f; any pair with an undecided window, index or
//     angle runs the reference-order FP64 chain of hbt_chain.cuh instead.
//     Same-event pairs that pass go to a second per-warp queue, so the FP64
//     work of stage C again runs on 32 pairs at a time.
//  C. Histogram update.  Mixed pairs add 1 to their denominator bin.
//     Same-event pairs add q_out, q_side, q_long and cos(q.dx / hbarC):
//       FP64 form  - the phase q.dx and its cos in FP64 (table_cos,
//                    hbt_math.cuh, of the unrounded product with 1/hbarC);
//                    q_out, q_side, q_long from algebraically identical
//                    expressions (q_out = (q_x S_x + q_y S_y) / |S|, ...) in
//                    double-float on the FP32 pipe, from the FP64 sums and
//                    differences (values64);
//       FP32W form - each FP64 column split once per tile into hi + lo
//                    FP32 parts; differences and the phase in double-float
//                    arithmetic on the FP32 pipe, q values in FP32, cos by
//                    quadrant reduction and FP32 Taylor polynomials
//                    (values32_split); added with one float4 vector atomic
//                    into FP32 partial bins (two arrays, even and odd warps:
//                    partials_of) that are merged into the FP64 bins with
//                    Kahan compensation.
//     In the FP32-weight form a pair is evaluated as stored (i, j) and
//     oriented afterwards: swapping first and second negates every momentum
//     and position difference, so it negates q_out, q_side, q_long exactly
//     (IEEE rounding is symmetric in sign) and leaves the phase and its cos
//     unchanged.
//  D. Pairs left undecided in B go to a third per-warp queue; the reference
//     chain runs on them 32 at a time.
//
// Error analysis (u = 2^-24).  Inputs are FP64 values v rounded once to
// FP32: |v32 - v| <= u|v|.  For s = a +- b in FP32, |s - S| <= 2.01 u A with
// A = |a| + |b| and S the exact sum of the FP64 inputs.  Products, sums, the
// reciprocal square root (rsqrtf: at most 2 ulp) and the approximate
// divisions used only inside the bounds (__fdividef: at most 2 ulp, the
// bounds carry a 1e-4 relative margin for it) propagate this as coded in
// screen_windows() and decide_bins(); every bound is then doubled and widened
// by the rounding of the FP32 copies of the constants, which also covers the
// FP64 reference's own rounding (2^-29 times smaller).
#pragma once

#include <type_traits>

#include "hbt_chain.cuh"
#include "hbt_math.cuh"

namespace hbt {
namespace tile {

using namespace chain;

constexpr float U = 5.9604645e-8f;  // 2^-24
constexpr int FT = 128;             // tile edge (particles) for both lists
constexpr int QCAP = 64;            // per-warp compaction queue

// FP32 screen quantities of one pair and their error bounds.
struct Q {
    float sx, sy, Ax, Ay, k2, ek2;
    float qo, eqo, qs, eqs, ql, eql;
};

// 0: certainly outside [lo, hi], 1: certainly inside, 2: undecided.
__device__ __forceinline__ int window_class(const Screen &S, float v, float err) {
    const float e = 2.0f * err + S.win_slack;
    if (v + e < S.lo || v - e > S.hi) return 0;
    if (v - e > S.lo && v + e < S.hi) return 1;
    return 2;
}

// Stage A: false only when the pair certainly lies outside the q window.
// a, b: FP32 momenta (px, py, pz, E); ga, gb: (|px| + |py|, |pz|) of each.
template <bool BOOST>
__device__ __forceinline__ bool prefilter(const Screen &S, float4 a, float2 ga, float4 b,
                                          float2 gb) {
    const float dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
    // |q_T| > sqrt(2) Q: |(dx, dy) - (q_x, q_y)| <= 2.01 u (|a.x|+|a.y|+|b.x|+|b.y|)
    const float t = __fmaf_rn(dx, dx, dy * dy);
    if (t > __fmaf_rn(S.pqt_c, ga.x + gb.x, S.pqt2)) return false;
    const float Az = ga.y + gb.y;
    if (BOOST) {
        // q_long = (S_E dz - S_z dE) / sqrt((S_E - S_z)(S_E + S_z)); reject
        // when (|nl| - e_nl)^2 > Q^2 * upper bound of (S_E - S_z)(S_E + S_z)
        const float sE = a.w + b.w, sz = a.z + b.z, dE = a.w - b.w;
        const float nl = __fmaf_rn(sE, dz, -(sz * dE));
        const float low = fabsf(nl) - 17.0f * U * sE * Az;
        const float em = 3.1f * U * (sE + Az);
        const float m = sE - sz, p = sE + sz;
        if (m > em && low > 0.0f &&
            low * low > S.pq2 * ((m + em) * (p + em)) * (1.0f + 1e-5f))
            return false;
    } else {
        if (fabsf(dz) > __fmaf_rn(2.1f * U, Az, S.pq)) return false;
    }
    return true;
}

// Stage B, K_T part: fills q's transverse sums and K_perp^2 with its bound;
// 0 the K_T cut certainly fails, 1 certainly passes, 2 undecided.
__device__ __forceinline__ int screen_kt(const Screen &S, float4 a, float4 b, Q &q) {
    q.sx = a.x + b.x;
    q.sy = a.y + b.y;
    q.Ax = fabsf(a.x) + fabsf(b.x);
    q.Ay = fabsf(a.y) + fabsf(b.y);
    q.k2 = __fmaf_rn(q.sx, q.sx, q.sy * q.sy);
    // |k2 - (S_x^2 + S_y^2)|
    q.ek2 = 6.1f * U * __fmaf_rn(q.Ax, fabsf(q.sx), q.Ay * fabsf(q.sy)) + 3.1f * U * q.k2 +
            1e-13f * __fmaf_rn(q.Ax, q.Ax, q.Ay * q.Ay);
    // K_T window (reference rejects Kp2 < KT_min^2 or Kp2 > KT_max^2)
    const float ekt = 2.0f * q.ek2 + S.kt_slack;
    if ((S.kt_lo4 > 0.0f && q.k2 + ekt < S.kt_lo4) || q.k2 - ekt > S.kt_hi4) return 0;
    return ((S.kt_lo4 == 0.0f || q.k2 - ekt > S.kt_lo4) && q.k2 + ekt < S.kt_hi4) ? 1 : 2;
}

// Stage B, LCMS part (after screen_kt): q_out, q_side, q_long and their
// bounds; 0 a window certainly fails, 1 all certainly pass, 2 undecided.
template <bool BOOST>
__device__ __forceinline__ int screen_lcms(const Screen &S, float4 a, float4 b, Q &q) {
    const float dx = a.x - b.x, dy = a.y - b.y;
    const float AA = __fmaf_rn(q.Ax, q.Ax, q.Ay * q.Ay);
    const float rel_k2 = __fdividef(q.ek2, q.k2) * 1.0001f;
    if (!(q.k2 > 0.0f) || !(rel_k2 <= 0.05f)) return 2;  // |S| too small for the bounds
    const float inv = rsqrtf(q.k2);
    const float rel_inv = 0.53f * rel_k2 + 4.5f * U;
    const float eN = 9.0f * U * AA;
    const float no = __fmaf_rn(dx, q.sx, dy * q.sy);
    const float ns = __fmaf_rn(dy, q.sx, -(dx * q.sy));
    q.qo = no * inv;
    q.eqo = __fmaf_rn(fabsf(no), rel_inv, eN) * inv + U * fabsf(q.qo);
    q.qs = ns * inv;
    q.eqs = __fmaf_rn(fabsf(ns), rel_inv, eN) * inv + U * fabsf(q.qs);
    const float dz = a.z - b.z;
    const float Az = fabsf(a.z) + fabsf(b.z);
    if (BOOST) {
        const float sE = a.w + b.w, sz = a.z + b.z, dE = a.w - b.w;
        const float AE = fabsf(a.w) + fabsf(b.w);
        const float m = sE - sz, p = sE + sz;
        const float e0 = 2.01f * U * (AE + Az);
        const float rel_m2 =
            (__fdividef(e0 + U * fabsf(m), m) + __fdividef(e0 + U * fabsf(p), p)) * 1.0001f +
            1.01f * U;
        if (!(m > 0.0f) || !(p > 0.0f) || !(rel_m2 <= 0.05f)) return 2;
        const float rl = rsqrtf(m * p);
        const float rel_rl = 0.53f * rel_m2 + 4.5f * U;
        const float nl = __fmaf_rn(sE, dz, -(sz * dE));
        q.ql = nl * rl;
        q.eql = __fmaf_rn(fabsf(nl), rel_rl, 17.0f * U * AE * Az) * rl + U * fabsf(q.ql);
    } else {
        q.ql = dz;
        q.eql = 2.1f * U * Az;
    }
    const int wo = window_class(S, q.qo, q.eqo), ws = window_class(S, q.qs, q.eqs),
              wl = window_class(S, q.ql, q.eql);
    if (wo == 0 || ws == 0 || wl == 0) return 0;
    if (wo == 2 || ws == 2 || wl == 2) return 2;
    return 1;
}

// Stage B: window checks.  Returns 0 (reject), 1 (all windows certainly
// passed), 2 (undecided).  The K_T and LCMS parts of screen_kt and
// screen_lcms in one function (the forms without q_inv histograms keep it
// whole: split, their register allocation spilled more).
template <bool BOOST>
__device__ __forceinline__ int screen_windows(const Screen &S, float4 a, float4 b, Q &q) {
    q.sx = a.x + b.x;
    q.sy = a.y + b.y;
    const float dx = a.x - b.x, dy = a.y - b.y;
    q.Ax = fabsf(a.x) + fabsf(b.x);
    q.Ay = fabsf(a.y) + fabsf(b.y);
    q.k2 = __fmaf_rn(q.sx, q.sx, q.sy * q.sy);
    const float AA = __fmaf_rn(q.Ax, q.Ax, q.Ay * q.Ay);
    // |k2 - (S_x^2 + S_y^2)|
    q.ek2 = 6.1f * U * __fmaf_rn(q.Ax, fabsf(q.sx), q.Ay * fabsf(q.sy)) + 3.1f * U * q.k2 +
            1e-13f * AA;
    // K_T window (reference rejects Kp2 < KT_min^2 or Kp2 > KT_max^2)
    const float ekt = 2.0f * q.ek2 + S.kt_slack;
    if ((S.kt_lo4 > 0.0f && q.k2 + ekt < S.kt_lo4) || q.k2 - ekt > S.kt_hi4) return 0;
    int cls = ((S.kt_lo4 == 0.0f || q.k2 - ekt > S.kt_lo4) && q.k2 + ekt < S.kt_hi4) ? 1 : 2;
    const float rel_k2 = __fdividef(q.ek2, q.k2) * 1.0001f;
    if (!(q.k2 > 0.0f) || !(rel_k2 <= 0.05f)) return 2;  // |S| too small for the bounds
    const float inv = rsqrtf(q.k2);
    const float rel_inv = 0.53f * rel_k2 + 4.5f * U;
    const float eN = 9.0f * U * AA;
    const float no = __fmaf_rn(dx, q.sx, dy * q.sy);
    const float ns = __fmaf_rn(dy, q.sx, -(dx * q.sy));
    q.qo = no * inv;
    q.eqo = __fmaf_rn(fabsf(no), rel_inv, eN) * inv + U * fabsf(q.qo);
    q.qs = ns * inv;
    q.eqs = __fmaf_rn(fabsf(ns), rel_inv, eN) * inv + U * fabsf(q.qs);
    const float dz = a.z - b.z;
    const float Az = fabsf(a.z) + fabsf(b.z);
    if (BOOST) {
        const float sE = a.w + b.w, sz = a.z + b.z, dE = a.w - b.w;
        const float AE = fabsf(a.w) + fabsf(b.w);
        const float m = sE - sz, p = sE + sz;
        const float e0 = 2.01f * U * (AE + Az);
        const float rel_m2 =
            (__fdividef(e0 + U * fabsf(m), m) + __fdividef(e0 + U * fabsf(p), p)) * 1.0001f +
            1.01f * U;
        if (!(m > 0.0f) || !(p > 0.0f) || !(rel_m2 <= 0.05f)) return 2;
        const float rl = rsqrtf(m * p);
        const float rel_rl = 0.53f * rel_m2 + 4.5f * U;
        const float nl = __fmaf_rn(sE, dz, -(sz * dE));
        q.ql = nl * rl;
        q.eql = __fmaf_rn(fabsf(nl), rel_rl, 17.0f * U * AE * Az) * rl + U * fabsf(q.ql);
    } else {
        q.ql = dz;
        q.eql = 2.1f * U * Az;
    }
    const int wo = window_class(S, q.qo, q.eqo), ws = window_class(S, q.qs, q.eqs),
              wl = window_class(S, q.ql, q.eql);
    if (wo == 0 || ws == 0 || wl == 0) return 0;
    if (wo == 2 || ws == 2 || wl == 2) return 2;
    return cls;
}

// floor((v - base) / delta_q) when certain, else -1.
__device__ __forceinline__ int q_index(const Screen &S, float v, float err) {
    const float t = (v - S.base) * S.inv_dq;
    const float et = (2.0f * err + S.win_slack) * S.inv_dq + 4.0f * U * fabsf(t) +
                     2.0f * U * (fabsf(v) + fabsf(S.base)) * S.inv_dq + S.t_slack;
    const float k = floorf(t);
    const float fr = t - k;
    if (!(fr > et) || !(fr < 1.0f - et) || k < 0.0f || k >= (float)S.qnpts) return -1;
    return (int)k;
}

// Stage B: K_T and q bin indices of a pair whose windows all passed.
// Returns false when any index is undecided.
__device__ __forceinline__ bool decide_bins(const Screen &S, const Q &q, int &iK, int &bin) {
    const float inv = rsqrtf(q.k2);
    const float kp = 0.5f * q.k2 * inv;  // |S|/2 = K_perp
    const float ekp = 0.5f * q.ek2 * inv * 1.1f + 8.0f * U * kp;
    const float t = (kp - S.KT_min) * S.inv_dKT;
    const float et = 2.0f * ekp * S.inv_dKT + 4.0f * U * (fabsf(t) + S.KT_min * S.inv_dKT) +
                     S.kt_t_slack;
    const float k = floorf(t);
    const float fr = t - k;
    if (!(fr > et) || !(fr < 1.0f - et) || k < 0.0f || k >= (float)S.n_KT) return false;
    iK = (int)k;
    const int io = q_index(S, q.qo, q.eqo), is = q_index(S, q.qs, q.eqs),
              il = q_index(S, q.ql, q.eql);
    if (io < 0 || is < 0 || il < 0) return false;
    bin = (io * S.qnpts + is) * S.qnpts + il;
    return true;
}

// q_inv^2 = q_x^2 + q_y^2 + q_z^2 - q_E^2 of a pair in FP32 (a, b: FP32
// momenta) and a bound on its distance from the reference's FP64 value
// -(q_E q_E - q_x q_x - q_y q_y - q_z q_z): each difference lies within
// e = 2.01 u (|a| + |b|) of the exact difference of the FP64 inputs, so its
// square within e (2 |d| + e); the FMA chain rounds four times, each below
// u times the sum of squares; the reference's own FP64 rounding is 2^-29
// times smaller and covered by a fifth u.
__device__ __forceinline__ void qinv2_bound(float4 a, float4 b, float &t, float &et) {
    const float dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z, dE = a.w - b.w;
    const float ex = 2.01f * U * (fabsf(a.x) + fabsf(b.x));
    const float ey = 2.01f * U * (fabsf(a.y) + fabsf(b.y));
    const float ez = 2.01f * U * (fabsf(a.z) + fabsf(b.z));
    const float eE = 2.01f * U * (fabsf(a.w) + fabsf(b.w));
    t = __fmaf_rn(dx, dx, __fmaf_rn(dy, dy, __fmaf_rn(dz, dz, -(dE * dE))));
    const float s2 = __fmaf_rn(dx, dx, __fmaf_rn(dy, dy, __fmaf_rn(dz, dz, dE * dE)));
    et = (ex * (2.0f * fabsf(dx) + ex) + ey * (2.0f * fabsf(dy) + ey) +
          ez * (2.0f * fabsf(dz) + ez) + eE * (2.0f * fabsf(dE) + eE)) * 1.0001f +
         5.0f * U * s2 + 1e-30f;
}

// Stage A for q_inv: false only when q_inv is certainly above the window
// (q_inv^2 lower bound above the square of the upper bound).
__device__ __forceinline__ bool prefilter_qinv(const Screen &S, float4 a, float4 b) {
    float t, et;
    qinv2_bound(a, b, t, et);
    return !(t - et > S.qi_hi2);
}

// Stage B for q_inv: 0 no q_inv event (q_inv outside the window or NaN),
// 1 event in q_inv bin k (certain), 2 undecided.
__device__ __forceinline__ int qinv_class(const Screen &S, float4 a, float4 b, int &k) {
    float t, et;
    qinv2_bound(a, b, t, et);
    if (t + et < 0.0f) return 0;  // the reference's q_inv is NaN: fails both bounds
    if (!(t - et > 0.0f)) return 2;
    const float qf = __fsqrt_rn(t);
    // |sqrt(t) - sqrt(T)| = |t - T| / (sqrt(t) + sqrt(T)) <= et / (sqrt(t) + sqrt(t - et))
    const float err = __fdividef(et, qf + __fsqrt_rn(t - et)) * 1.0001f + U * qf;
    const int w = window_class(S, qf, err);
    if (w != 1) return w;
    k = q_index(S, qf, err);
    return k < 0 ? 2 : 1;
}

// K_T bin from the FP32 screen values (after screen_kt): >= 0 certain,
// -1 undecided.
__device__ __forceinline__ int kt_index(const Screen &S, const Q &q) {
    const float inv = rsqrtf(q.k2);
    const float kp = 0.5f * q.k2 * inv;  // |S|/2 = K_perp
    const float ekp = 0.5f * q.ek2 * inv * 1.1f + 8.0f * U * kp;
    const float t = (kp - S.KT_min) * S.inv_dKT;
    const float et = 2.0f * ekp * S.inv_dKT + 4.0f * U * (fabsf(t) + S.KT_min * S.inv_dKT) +
                     S.kt_t_slack;
    const float k = floorf(t);
    const float fr = t - k;
    if (!(q.k2 > 0.0f) || !(__fdividef(q.ek2, q.k2) <= 0.05f)) return -1;
    if (!(fr > et) || !(fr < 1.0f - et) || k < 0.0f || k >= (float)S.n_KT) return -1;
    return (int)k;
}

// K_phi bin from the FP32 screen values: >= 0 certain, -2 undecided.
__device__ __forceinline__ int kphi_screen(const Screen &S, const Q &q) {
    const float phi = atan2f(q.sy, q.sx);
    // angle error from the inputs, atan2f (3 ulp), psi_ref rounding, wrap
    const float e = 2.02f * U * __fdividef(__fmaf_rn(q.Ax, fabsf(q.sy), q.Ay * fabsf(q.sx)), q.k2) +
                    1.0e-6f + S.psi_slack;
    float d = phi - S.psi;
    if (d < 0.0f) d += S.two_pi;
    // pairs within the host's deferral zone go to the reference chain too
    const float ed = 2.0f * e + 1.0e-6f + S.kphi_tol;
    if (!(d > ed) || !(d < S.two_pi - ed)) return -2;
    const float r = d * S.inv_dKphi;
    const float er = ed * S.inv_dKphi + 4.0f * U * r;
    const float k = floorf(r);
    const float fr = r - k;
    if (!(fr > er) || !(fr < 1.0f - er) || k < 0.0f || k >= (float)S.n_Kphi) return -2;
    return (int)k;
}

// Summed values of the FP32-weight form.  The momentum sums and differences
// are taken in FP64 (no cancellation), then q_out, q_side, q_long follow in
// FP32 (relative error a few 1e-7).  cos: the phase is computed and reduced
// to [-pi, pi] in FP64 (Cody-Waite with a two-part 2 pi), then to
// [-pi/4, pi/4] by quadrant in FP32, where Taylor polynomials of cos (to
// x^8) and sin (to x^9) are accurate to 3e-8 and 2e-9: error < 2e-7.
template <bool BOOST>
__device__ __forceinline__ float4 values32(const Grid &g, const double *a, const double *b) {
    const double dx = a[0] - b[0], dy = a[1] - b[1];
    const double dz = a[2] - b[2], dE = a[3] - b[3];
    const float fsx = (float)(a[0] + b[0]), fsy = (float)(a[1] + b[1]);
    const float fdx = (float)dx, fdy = (float)dy, fdz = (float)dz;
    const float inv = rsqrtf(__fmaf_rn(fsx, fsx, fsy * fsy));
    float4 v;
    v.x = __fmaf_rn(fdx, fsx, fdy * fsy) * inv;
    v.y = __fmaf_rn(fdy, fsx, -(fdx * fsy)) * inv;
    if (BOOST) {
        const float sE = (float)(a[3] + b[3]), sz = (float)(a[2] + b[2]), fdE = (float)dE;
        v.z = __fmaf_rn(sE, fdz, -(sz * fdE)) * rsqrtf((sE - sz) * (sE + sz));
    } else {
        v.z = fdz;
    }
    const double ph = g.hbarC_inv * (dE * (a[7] - b[7]) - dx * (a[4] - b[4]) -
                                     dy * (a[5] - b[5]) - dz * (a[6] - b[6]));
    const double k = rint(ph * 0.15915494309189535);  // 1 / (2 pi)
    double r = __fma_rn(-k, 6.283185307179586, ph);   // 2 pi, leading double
    r = __fma_rn(-k, 2.4492935982947064e-16, r);      // 2 pi - leading double
    const float rf = (float)r;
    const float j = rintf(rf * 0.63661977f);           // 2 / pi
    float x = __fmaf_rn(-j, 1.5707963f, rf);           // pi/2 = 1.5707963 + 4.37114e-8
    x = __fmaf_rn(-j, -4.37113883e-8f, x);
    const float x2 = x * x;
    const float c = __fmaf_rn(x2, __fmaf_rn(x2, __fmaf_rn(x2, __fmaf_rn(x2, 2.48015873e-5f,
                                                                      -1.38888889e-3f),
                                                          4.16666667e-2f),
                                            -0.5f),
                              1.0f);
    const float s = x * __fmaf_rn(x2, __fmaf_rn(x2, __fmaf_rn(x2, __fmaf_rn(x2, 2.75573192e-6f,
                                                                          -1.98412698e-4f),
                                                              8.33333333e-3f),
                                                -1.66666667e-1f),
                                  1.0f);
    const int quad = ((int)j) & 3;  // cos(x + j pi/2)
    v.w = quad == 0 ? c : quad == 1 ? -s : quad == 2 ? -c : s;
    return v;
}

// ---- double-float arithmetic (value = hi + lo, two FP32 numbers) on the
// FP32 pipe, for the FP32-weight form's per-pair values.  The error-free
// transformations are Knuth's two-sum and the FMA two-product (as in
// Dekker's and Shewchuk's double-length arithmetic).
struct FF {
    float h, l;
};

// Exact FP32 -> FP64 conversion of a normal FP32 value or zero through its
// bits, on the integer pipe (the conversion instruction runs on the FP64
// pipe): the exponent
// rebiased by 1023 - 127 = 896, the significand moved up by 29 bits.  FP32
// subnormals (below 1.2e-38, which the low parts of these values never
// reach but at zero) give a signed zero; infinities and NaN are not
// handled (the values of binned pairs are finite).
__device__ __forceinline__ double f32_to_f64_bits(float f) {
    const unsigned u = __float_as_uint(f), m = u & 0x7fffffffu, sign = u & 0x80000000u;
    const bool normal = m >= 0x00800000u;
    const unsigned hi = normal ? ((m >> 3) + (896u << 20)) | sign : sign;
    return __hiloint2double((int)hi, normal ? (int)(m << 29) : 0);
}

__device__ __forceinline__ FF two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return FF{s, e};
}

// a + b with |a| >= |b| (or a == 0).
__device__ __forceinline__ FF fast_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    return FF{s, __fsub_rn(b, __fsub_rn(s, a))};
}

// (ah + al) - (bh + bl) of two split FP64 values.  A split holds its value
// to 2^-48 relative; the high parts' difference is exact (two-sum) and the
// low parts add one FP32 rounding of a term below 2^-47 of the inputs.
__device__ __forceinline__ FF ff_diff(float2 a, float2 b) {
    const FF s = two_sum(a.x, -b.x);
    return two_sum(s.h, __fadd_rn(s.l, __fsub_rn(a.y, b.y)));
}

__device__ __forceinline__ FF ff_mul(FF a, FF b) {
    const float p = __fmul_rn(a.h, b.h);
    float e = __fmaf_rn(a.h, b.h, -p);
    e = __fmaf_rn(a.h, b.l, e);
    e = __fmaf_rn(a.l, b.h, e);
    return fast_two_sum(p, e);
}

__device__ __forceinline__ FF ff_add(FF a, FF b) {
    const FF s = two_sum(a.h, b.h);
    return two_sum(s.h, __fadd_rn(s.l, __fadd_rn(a.l, b.l)));
}

__device__ __forceinline__ FF ff_neg(FF a) { return FF{-a.h, -a.l}; }

// Splits an FP64 value into hi = nearest FP32 and lo = nearest FP32 to the
// rest (done once per particle and tile).
__device__ __forceinline__ float2 split(double x) {
    const float h = (float)x;
    return make_float2(h, (float)(x - (double)h));
}

// cos of a phase given as a double-float: reduction by quadrant with pi/2
// split into three parts (12 + 12 significant bits and the rest, so that
// j times either leading part is exact for |j| < 2^11), then the FP32
// Taylor polynomials of values32.  Absolute error below 2e-7.
__device__ __forceinline__ float ff_cos(FF ph) {
    const float j = rintf(ph.h * 0.63661977f);  // 2 / pi
    float x;
    if (fabsf(j) < 2048.0f) {
        const float t1 = __fmaf_rn(-j, 1.57080078125f, ph.h);       // exact
        const FF t2 = two_sum(t1, __fmul_rn(-j, -4.453584551811218e-06f));
        x = __fadd_rn(t2.h, __fadd_rn(t2.l, __fmaf_rn(-j, -8.705515752716053e-10f, ph.l)));
    } else {
        // never on this path (|q.dx| / hbarC is a few hundred at most)
        const double r = (double)ph.h + (double)ph.l;
        const double k = rint(r * 0.6366197723675814);
        x = (float)(r - k * 1.5707963267948966);
        return cosf(x + (float)(fmod(k, 4.0)) * 1.5707964f);
    }
    const float x2 = __fmul_rn(x, x);
    const float c = __fmaf_rn(x2, __fmaf_rn(x2, __fmaf_rn(x2, __fmaf_rn(x2, 2.48015873e-5f,
                                                                    -1.38888889e-3f),
                                                        4.16666667e-2f),
                                          -0.5f),
                              1.0f);
    const float s = x * __fmaf_rn(x2, __fmaf_rn(x2, __fmaf_rn(x2, __fmaf_rn(x2, 2.75573192e-6f,
                                                                        -1.98412698e-4f),
                                                            8.33333333e-3f),
                                              -1.66666667e-1f),
                                1.0f);
    const int quad = ((int)j) & 3;  // cos(x + j pi/2)
    return quad == 0 ? c : quad == 1 ? -s : quad == 2 ? -c : s;
}

// Summed values of the FP32-weight form from split FP64 inputs, all on the
// FP32 pipe: momentum and position differences in double-float (their
// rounding relative to the difference, not to the momenta), q_out, q_side,
// q_long in FP32 (a few 1e-7 relative), the phase (q.dx)/hbarC in
// double-float and its cos by ff_cos.  a, b: the eight split columns of the
// pair's first and second particle.
template <bool BOOST>
__device__ __forceinline__ float4 values32_split(const Screen &S, const float2 *a,
                                                 const float2 *b) {
    const FF dx = ff_diff(a[0], b[0]), dy = ff_diff(a[1], b[1]);
    const FF dz = ff_diff(a[2], b[2]), dE = ff_diff(a[3], b[3]);
    const float sx = __fadd_rn(__fadd_rn(a[0].x, b[0].x), __fadd_rn(a[0].y, b[0].y));
    const float sy = __fadd_rn(__fadd_rn(a[1].x, b[1].x), __fadd_rn(a[1].y, b[1].y));
    const float inv = rsqrtf(__fmaf_rn(sx, sx, sy * sy));
    float4 v;
    v.x = __fmaf_rn(dx.h, sx, dy.h * sy) * inv;
    v.y = __fmaf_rn(dy.h, sx, -(dx.h * sy)) * inv;
    if (BOOST) {
        const float sE = __fadd_rn(__fadd_rn(a[3].x, b[3].x), __fadd_rn(a[3].y, b[3].y));
        const float sz = __fadd_rn(__fadd_rn(a[2].x, b[2].x), __fadd_rn(a[2].y, b[2].y));
        v.z = __fmaf_rn(sE, dz.h, -(sz * dE.h)) * rsqrtf((sE - sz) * (sE + sz));
    } else {
        v.z = dz.h;
    }
    FF ph = ff_mul(dE, ff_diff(a[7], b[7]));
    ph = ff_add(ph, ff_neg(ff_mul(dx, ff_diff(a[4], b[4]))));
    ph = ff_add(ph, ff_neg(ff_mul(dy, ff_diff(a[5], b[5]))));
    ph = ff_add(ph, ff_neg(ff_mul(dz, ff_diff(a[6], b[6]))));
    ph = ff_mul(ph, FF{S.hc_h, S.hc_l});
    v.w = ff_cos(ph);
    return v;
}

// ---- Double-float form (HBT_PRECISION_DF64): the summed values of a binned
// same-event pair to FP64-class accuracy with FP32-pipe arithmetic.  The
// inputs are split columns; the four momentum columns are split after
// subtracting an FP32 offset per tile (the momentum of the tile's first
// row), so their splitting error is 2^-48 of the distance to that row (the
// tiles are compact in momentum) instead of 2^-48 of the momentum, which
// would be the largest term of the phase error.

// a + b of two split values.
__device__ __forceinline__ FF ff_sum(float2 a, float2 b) {
    const FF s = two_sum(a.x, b.x);
    return two_sum(s.h, __fadd_rn(s.l, __fadd_rn(a.y, b.y)));
}

__device__ __forceinline__ FF ff_mul_f(FF a, float b) {
    const float p = __fmul_rn(a.h, b);
    float e = __fmaf_rn(a.h, b, -p);
    e = __fmaf_rn(a.l, b, e);
    return fast_two_sum(p, e);
}

// 1 / sqrt(x): the FP32 estimate y0 and one Newton step carried in
// double-float.  With u = x y0^2 = 1 + e (|e| ~ 2^-22, u.h - 1 exact),
// 1 / sqrt(x) = y0 (1 - e / 2 + 3 e^2 / 8 - ...): relative error about 2^-46.
__device__ __forceinline__ FF ff_rsqrt(FF x) {
    const float y0 = rsqrtf(x.h);
    const FF u = ff_mul_f(ff_mul_f(x, y0), y0);
    const float e = __fadd_rn(__fsub_rn(u.h, 1.0f), u.l);
    return fast_two_sum(y0, __fmul_rn(__fmul_rn(y0, e), __fmaf_rn(0.375f, e, -0.5f)));
}

// Table of cos(k / 64) and sin(k / 64), |k| <= 51, as split pairs
// (cos hi, cos lo, sin hi, sin lo), filled by each CTA of the double-float
// same-event kernels from the FP64 sincos.
constexpr int DF_TABLE_HALF = 51;
constexpr int DF_TABLE = 2 * DF_TABLE_HALF + 1;
__device__ __forceinline__ void fill_df_table(float4 *t) {
    for (int k = threadIdx.x; k < DF_TABLE; k += blockDim.x) {
        double s, c;
        sincos((k - DF_TABLE_HALF) / 64.0, &s, &c);
        const float2 cc = split(c), ss = split(s);
        t[k] = make_float4(cc.x, cc.y, ss.x, ss.y);
    }
}

// cos of a double-float phase, to about 5e-15 absolute (the table's 48-bit
// values), for |ph| < 3200 (|q.dx| / hbarC is a few hundred at most; beyond,
// the FP64 cos).  Cody-Waite reduction by quarter periods x = ph - j pi / 2
// with pi / 2 in four FP32 parts: the first two have 12 significant bits
// (j times them is exact for |j| < 2^11), the third goes through an FMA
// two-product and the fourth is below 2^-57, so x carries about 2^-48
// absolute error; |x| <= pi / 4.  Then the table point t = k / 64 nearest x
// (exact in FP32) and d = x - t, |d| <= 1 / 128:
//   cos(x + j pi / 2) = A cos d + B sin d,
// (A, B) = (C, -S), (-S, -C), (-C, S), (S, C) for j mod 4 = 0..3 with
// C = cos t, S = sin t; cos d - 1 = -d^2 / 2 + d^4 / 24 and
// sin d - d = d^3 (-1 / 6 + d^2 / 120) (truncations below 3.2e-16 and
// 4e-19), the d^2 and d^3 terms in double-float.
__device__ __forceinline__ double df_cos(const float4 *tab, FF ph) {
    const float j = rintf(ph.h * 0.63661977f);  // 2 / pi
    if (!(fabsf(j) < 2048.0f)) return cos((double)ph.h + (double)ph.l);
    const float t1 = __fmaf_rn(-j, 1.57080078125f, ph.h);  // exact
    const FF s1 = two_sum(t1, __fmul_rn(-j, -4.453584551811218e-06f));  // product exact
    const float p3 = __fmul_rn(-j, -8.705515752716053e-10f);
    const float e3 = __fmaf_rn(-j, -8.705515752716053e-10f, -p3);
    const FF s2 = two_sum(s1.h, p3);
    const FF u = two_sum(s2.h, ph.l);
    const float rest = __fadd_rn(__fadd_rn(s1.l, s2.l),
                                 __fadd_rn(e3, __fmul_rn(-j, 5.721188916458728e-18f)));
    const FF x = fast_two_sum(u.h, __fadd_rn(u.l, rest));
    const float k = rintf(x.h * 64.0f);
    const FF dd = two_sum(__fsub_rn(x.h, k * 0.015625f), x.l);  // x.h - k / 64 exact
    const FF d2 = ff_mul(dd, dd);
    const float c4 = __fmul_rn(__fmul_rn(d2.h, d2.h), 1.0f / 24.0f);
    const FF cm = {__fmul_rn(d2.h, -0.5f), __fadd_rn(__fmul_rn(d2.l, -0.5f), c4)};
    // -1 / 6 as a split pair, plus d^2 / 120
    const FF kq = fast_two_sum(-0.1666666716337204f,
                               __fadd_rn(4.967053879312289e-09f, d2.h * (1.0f / 120.0f)));
    const FF sd = ff_add(dd, ff_mul(ff_mul(d2, dd), kq));
    const float4 e = tab[(int)k + DF_TABLE_HALF];
    const int quad = ((int)j) & 3;
    FF A, B;
    if (quad == 0) {
        A = FF{e.x, e.y};
        B = FF{-e.z, -e.w};
    } else if (quad == 1) {
        A = FF{-e.z, -e.w};
        B = FF{-e.x, -e.y};
    } else if (quad == 2) {
        A = FF{-e.x, -e.y};
        B = FF{e.z, e.w};
    } else {
        A = FF{e.z, e.w};
        B = FF{e.x, e.y};
    }
    const FF r = ff_add(A, ff_add(ff_mul(A, cm), ff_mul(B, sd)));
    return (double)r.h + (double)r.l;
}

// hi + lo rounded once to FP64: with the conversion instructions (the
// double-float form, whose FP64 pipe has room), or on the integer pipe (the
// FP64 form, whose FP64 pipe is the busiest).
__device__ __forceinline__ double ff_double(FF a) { return (double)a.h + (double)a.l; }
__device__ __forceinline__ double ff_double_bits(FF a) {
    return f32_to_f64_bits(a.h) + f32_to_f64_bits(a.l);
}

// x as hi + lo, two FP32 values formed from its bits on the integer pipe:
// hi is x with the significand truncated to 24 bits, lo the remaining 29
// bits truncated to 24, so that |x - hi - lo| < 2^-46 |x| (both parts carry
// the sign of x).  For x = 0 or 2^-100 <= |x| < 2^100 (momenta, their sums
// and differences); a lo part below the FP32 normal range (2^-126) is
// dropped, and magnitudes outside the range give zero.
__device__ __forceinline__ FF f64_to_ff_bits(double x) {
    const unsigned hw = (unsigned)__double2hiint(x), lw = (unsigned)__double2loint(x);
    const unsigned sign = hw & 0x80000000u, ae = hw & 0x7fffffffu;
    const bool in_range = ae - ((1023u - 100u) << 20) < (200u << 20);
    // hi: the exponent rebiased by 1023 - 127 = 896, the top 23 explicit bits
    const unsigned hb = __funnelshift_l(lw, ae - (896u << 20), 3) | sign;
    // lo: the low 29 bits r, worth r 2^(E - 1075); its leading bit is bit
    // 31 - clz(r), so the FP32 exponent field is E - 917 - clz(r)
    const unsigned r = lw & 0x1fffffffu;
    const int lz = __clz(r);
    const int e = (int)(ae >> 20) - 917 - lz;
    const unsigned lb = (r != 0u && e > 0)
                            ? ((unsigned)e << 23) | (((r << (lz & 31)) >> 8) & 0x7fffffu) | sign
                            : sign;
    return in_range ? FF{__uint_as_float(hb), __uint_as_float(lb)} : FF{0.0f, 0.0f};
}

// q_out, q_side, q_long of a pair in double-float arithmetic from its
// momentum differences dp and sums sp (px, py, pz, E; sp[2], sp[3] only
// with the boost): q_out = (dx sx + dy sy) / |s_T|, q_side = (dy sx - dx sy)
// / |s_T| and, with the longitudinal boost, q_long = (sE dz - sz dE) /
// sqrt(sE^2 - sz^2) (algebraically the reference's expressions), each
// operation in double-float: about 1e-14 relative, or 2^-45 of |dp_T| in
// absolute terms where q_out or q_side cancels.
template <bool BOOST>
__device__ __forceinline__ void ff_lcms(const FF *dp, const FF *sp, FF &vo, FF &vs, FF &vl) {
    const FF inv = ff_rsqrt(ff_add(ff_mul(sp[0], sp[0]), ff_mul(sp[1], sp[1])));
    vo = ff_mul(ff_add(ff_mul(dp[0], sp[0]), ff_mul(dp[1], sp[1])), inv);
    vs = ff_mul(ff_add(ff_mul(dp[1], sp[0]), ff_neg(ff_mul(dp[0], sp[1]))), inv);
    vl = dp[2];
    if (BOOST) {
        const FF m2 = ff_mul(ff_add(sp[3], ff_neg(sp[2])), ff_add(sp[3], sp[2]));
        vl = ff_mul(ff_add(ff_mul(sp[3], dp[2]), ff_neg(ff_mul(sp[2], dp[3]))), ff_rsqrt(m2));
    }
}

// Summed values of a binned pair in the double-float form, for the pair as
// stored (first = a from the i-tile, second = b from the j-tile): a, b are
// the eight split columns (momenta relative to the tiles' offsets oa, ob),
// results as FP64, q_out, q_side, q_long negated when `neg` (the pair's
// reference orientation is (b, a)).  The expressions of ff_lcms and
// values64 from the split columns, each operation in double-float; q_out, q_side, q_long to about 1e-15 relative,
// the phase to 2^-48 of its terms.
template <bool BOOST>
__device__ __forceinline__ void values_df(const Screen &S, const float4 *tab, const float2 *a,
                                          const float2 *b, const float *oa, const float *ob,
                                          bool neg, double &qo, double &qs, double &ql,
                                          double &w) {
    FF dp[4], sp[4], vo, vs, vl;
#pragma unroll
    for (int f = 0; f < 4; f++) {
        dp[f] = ff_add(ff_diff(a[f], b[f]), two_sum(oa[f], -ob[f]));
        if (f < 2 || BOOST) sp[f] = ff_add(ff_sum(a[f], b[f]), two_sum(oa[f], ob[f]));
    }
    ff_lcms<BOOST>(dp, sp, vo, vs, vl);
    if (neg) {
        vo = ff_neg(vo);
        vs = ff_neg(vs);
        vl = ff_neg(vl);
    }
    qo = ff_double(vo);
    qs = ff_double(vs);
    ql = ff_double(vl);
    FF ph = ff_mul(dp[3], ff_diff(a[7], b[7]));
    ph = ff_add(ph, ff_neg(ff_mul(dp[0], ff_diff(a[4], b[4]))));
    ph = ff_add(ph, ff_neg(ff_mul(dp[1], ff_diff(a[5], b[5]))));
    ph = ff_add(ph, ff_neg(ff_mul(dp[2], ff_diff(a[6], b[6]))));
    w = df_cos(tab, ff_mul(ph, FF{S.hc_h, S.hc_l}));
}

// FP64 summed values of an accepted same-event pair (algebraically the
// reference's q_out, q_side, q_long and cos(q.dx / hbarC)).  The momentum
// differences and sums are FP64 (one rounding each, so that cancelling sums
// stay exact to the last bits), and so are the phase q.dx and its cos
// (table_cos of the unrounded product with 1/hbarC, 3e-16).  q_out, q_side
// and the boosted q_long, which are only summed, follow in double-float on
// the FP32 pipe (ff_lcms: about 1e-14 relative) from the FP64 sums and
// differences split on the integer pipe, and come back as FP64 with one
// addition each.  The longitudinal sums sz = p_z1 + p_z2 and sE = E_1 + E_2
// (used with the boost only) come in as double-float sums of the particles'
// split values (2^-47 of the sum: sE does not cancel, and sz enters q_long
// through sz dE and M_T^2 = (sE - sz)(sE + sz), where its absolute error
// stays below 1e-14 GeV).  Of the FP64 pipe, which bounds this form, a
// binned pair then takes 27 to 29 instructions instead of 55.
template <bool BOOST>
__device__ __forceinline__ void values64(const Grid &g, const double2 *cs, const double *a,
                                         const double *b, FF sz, FF sE, double &qo, double &qs,
                                         double &ql, double &w) {
    const double dx = a[0] - b[0], dy = a[1] - b[1];
    const double dz = a[2] - b[2], dE = a[3] - b[3];
    FF dp[4] = {f64_to_ff_bits(dx), f64_to_ff_bits(dy), f64_to_ff_bits(dz), f64_to_ff_bits(dE)};
    FF sp[4];
    sp[0] = f64_to_ff_bits(a[0] + b[0]);
    sp[1] = f64_to_ff_bits(a[1] + b[1]);
    sp[2] = sz;
    sp[3] = sE;
    FF vo, vs, vl;
    ff_lcms<BOOST>(dp, sp, vo, vs, vl);
    qo = ff_double_bits(vo);
    qs = ff_double_bits(vs);
    ql = BOOST ? ff_double_bits(vl) : dz;
    // q.dx = dE dt - dx dX - dy dY - dz dZ, accumulated with fused
    // multiply-adds (one rounding per term)
    double ph = dE * (a[7] - b[7]);
    ph = __fma_rn(-dx, a[4] - b[4], ph);
    ph = __fma_rn(-dy, a[5] - b[5], ph);
    ph = __fma_rn(-dz, a[6] - b[6], ph);
    w = table_cos(cs, g.cph, ph);
}

// Shared memory of one tile pair; E2 is the entry of the second same-event
// queue (uint2, or uint4 when q_inv histograms are binned too).
template <class E2>
struct TileSmemT {
    // same-event tiles: FP64 columns (FP64 form) or split columns (hi, lo
    // FP32 pairs, FP32-weight form), px py pz E x y z t
    double si[8][FT];
    double sj[8][FT];
    float4 fi[FT];     // FP32 momenta of the i-tile
    float4 fj[FT];     // FP32 momenta of the j-tile
    float2 gi[FT];     // (|px| + |py|, |pz|) of the i-tile (prefilter)
    float2 gj[FT];
    // FP64 form: FP32 low parts of p_z and E (their high parts are fi, fj's
    // z and w), for the longitudinal sums in double-float
    float2 li[FT], lj[FT];
    unsigned queue[FT / 32][QCAP];
    // same-event pairs that passed the window screen: x = (i, j, swap,
    // undecided, slot) bits, y = q bin (bin_entry); with q_inv, x = (i, j,
    // swap, undecided, 3-D event, q_inv event) bits, y = q bin, z = slot |
    // K_T bin << 16, w = q_inv bin
    E2 queue2[FT / 32][QCAP];
    // pairs the screen left undecided, (i, j, swap) bits: the reference
    // chain runs on them 32 at a time (inline, a warp would run it for the
    // one or two lanes holding such a pair)
    unsigned queue3[FT / 32][QCAP];
    unsigned oi[FT], oj[FT];  // original list positions (pair orientation)
    float offi[4], offj[4];   // double-float form: the tiles' momentum offsets
};
using TileSmem = TileSmemT<uint2>;
template <bool QINV>
using SmemFor = TileSmemT<typename std::conditional<QINV, uint4, uint2>::type>;

// Entry of the second same-event queue.
__device__ __forceinline__ uint2 bin_entry(unsigned e, bool undecided, int slot, int bin) {
    return make_uint2((e & 0x1ffffu) | (undecided ? 1u << 17 : 0u) | ((unsigned)slot << 18),
                      (unsigned)bin);
}

// Appends this lane's entry to the warp queue when `take`, and runs
// `process(entry, true)` on 32 queued entries whenever 32 are waiting (all
// lanes of the warp call this in step; `count` is warp-uniform).
template <class T, class F>
__device__ __forceinline__ void enqueue(T *q, int &count, bool take, T entry, int lane,
                                        F &process) {
    const unsigned m = __ballot_sync(0xffffffffu, take);
    if (!m) return;
    if (take) q[count + __popc(m & ((1u << lane) - 1u))] = entry;
    count += __popc(m);
    __syncwarp();
    if (count >= 32) {
        process(q[lane], true);
        __syncwarp();
        if (lane < count - 32) q[lane] = q[32 + lane];
        __syncwarp();
        count -= 32;
    }
}

// Runs `process(entry, valid)` on the entries left in the queue, all lanes
// in step (lanes beyond the count pass valid = false).
template <class T, class F>
__device__ __forceinline__ void drain(T *q, int count, int lane, F &process) {
    if (count > 0) process(q[lane < count ? lane : 0], lane < count);
    __syncwarp();
}

// Sum of x over the lanes in `peers` (the lanes of the warp holding the
// same key, from __match_any_sync), left in the group's lowest lane: a tree
// over the lanes' ranks in their group, log2(group size) shuffle rounds
// (each lane adds its next remaining peer's value, then the odd ranks drop
// out and the ranks halve).  Called by all 32 lanes.
__device__ __forceinline__ double sum_peers(unsigned peers, double x) {
    const int lane = threadIdx.x & 31;
    unsigned rest = peers & (0xfffffffeu << lane);  // peers above this lane
    int rank = __popc(peers & ((1u << lane) - 1u));
    while (__any_sync(0xffffffffu, rest != 0u)) {
        const int next = __ffs(rest);  // 1-based, 0: none left
        const double t = __shfl_sync(0xffffffffu, x, next ? next - 1 : lane);
        if (next) x += t;
        rest &= ~__ballot_sync(0xffffffffu, rank & 1);
        rank >>= 1;
    }
    return x;
}

// One q_inv histogram update per group of lanes with the same bin (`key`,
// 0xffffffff: no update): the q_inv histogram has only n_KT x qnpts bins,
// which the pairs of a warp share, so per-pair atomics would queue on a few
// addresses.  num: add q_inv and cos (numerator, same-event) or only the
// count (denominator, mixed-event).  Called by all 32 lanes.
__device__ __forceinline__ void qinv_update(const Device &d, unsigned key, double qv, double wv,
                                            bool num) {
    const unsigned peers = __match_any_sync(0xffffffffu, key);
    const int lane = threadIdx.x & 31;
    const bool leader = (peers & ((1u << lane) - 1u)) == 0u && key != 0xffffffffu;
    if (num) {
        const double sq = sum_peers(peers, qv), sw = sum_peers(peers, wv);
        if (leader) {
            atomicAdd(&d.h.qi_sums[key].q, sq);
            atomicAdd(&d.h.qi_sums[key].w, sw);
            atomicAdd(d.h.qi_cnt + key, (unsigned long long)__popc(peers));
        }
    } else if (leader) {
        atomicAdd(d.h.qi_den + key, (unsigned long long)__popc(peers));
    }
}

// A mixed-event pair the screens left undecided: the reference chain
// decides.  Out of line: it runs for a few pairs per thousand, and inlined
// its registers would crowd the screen's (the kernel spilled 420 bytes).
static __device__ __noinline__ void undecided_mixed_pair(const Device &d, const double *const *l1,
                                                         const double *const *l2, long long i,
                                                         long long j, long long n1, long long n2) {
    const Chain ch = pair_chain<true>(d.g, l1[0][i], l1[1][i], l1[2][i], l1[3][i], l2[0][j],
                                      l2[1][j], l2[2][j], l2[3][j], nullptr, nullptr);
    consume<true, MODE_FAST>(d, i, j, n2, n1, ch);
}

// A same-event pair of the FP32-weight form that the screens left
// undecided: the reference chain decides; a binned pair adds its FP32
// values to the partials.  Out of line, for the same reason.
template <bool BOOST>
__device__ __noinline__ void undecided_pair32(const Device &d, const double *A, const double *B,
                                              long long i, long long j, long long n) {
    const Chain full = pair_chain<false>(d.g, A[0], A[1], A[2], A[3], B[0], B[1], B[2], B[3],
                                         A + 4, B + 4);
    if (full.ev3 != 1) {
        consume<false, MODE_FAST>(d, i, j, n, n, full);
    } else {
        const long long at = (long long)full.slot * d.g.q3 + full.bin;
        atomicAdd(partials_of(d) + at, values32<BOOST>(d.g, A, B));
        atomicAdd(d.h.cnt + at, 1ull);
    }
}

// A same-event pair of the FP64 or double-float form that the screens left
// undecided: the reference chain decides and bins it with FP64 values.  Out
// of line, so that the chain's registers do not spill in the pair loop.
static __device__ __noinline__ void undecided_pair64(const Device &d, const double *A,
                                                     const double *B, long long i, long long j,
                                                     long long n) {
    const Chain full = pair_chain<false>(d.g, A[0], A[1], A[2], A[3], B[0], B[1], B[2], B[3],
                                         A + 4, B + 4);
    consume<false, MODE_FAST>(d, i, j, n, n, full);
}

// A pair the screens left undecided, under ordered cap admission (COUNT
// or ORDER mode): the reference chain decides; the pair is counted or
// admitted at its position in the caller's lists (row, col).  Out of line,
// like the fast-mode helpers above.
template <bool MIXED, int MODE>
__device__ __noinline__ void undecided_pair_ordered(const Device &d, const double *A,
                                                    const double *B, long long row,
                                                    long long col, long long rows,
                                                    long long cols) {
    const Chain full = pair_chain<MIXED>(d.g, A[0], A[1], A[2], A[3], B[0], B[1], B[2], B[3],
                                         MIXED ? nullptr : A + 4, MIXED ? nullptr : B + 4);
    consume<MIXED, MODE>(d, row, col, cols, rows, full);
}

// Ordered cap admission of a pair the screen decided (slot, row in the
// caller's order): COUNT adds it to its row's survivor count and returns
// false; ORDER returns true when its row lies before the slot's cut row
// (the cut row itself is admitted pair by pair by k_straddle).
template <int MODE>
__device__ __forceinline__ bool admit(const Device &d, int slot, long long row, long long rows) {
    if (MODE == MODE_FAST) return true;
    if (MODE == MODE_COUNT) {
        atomicAdd(d.caps.rowcnt + (long long)slot * rows + row, 1u);
        return false;
    }
    return row < d.caps.row_cut[slot];
}

// Same-event pairs of the tiles starting at i0 and j0 (i0 <= j0) of one list
// of n particles with columns c = px py pz E x y z t.  Every unordered pair
// is visited once (position j > i); it is oriented as the reference orients
// it, q = p_first - p_second with `first` the particle earlier in the
// caller's list: orig[k] is that original index of row k, or nullptr when
// the rows are in the caller's order.  MODE selects the admission: FAST bins
// every pair; COUNT and ORDER are the two passes of ordered cap admission,
// which see each pair at its row (the earlier of its two positions in the
// caller's list).  QINV: the pairs also go to the q_inv histograms
// (invariant_radius_flag, src/HBT_correlation.cpp:331-356): a pair is kept
// when its 3-D window or its q_inv window can pass, and its q_inv bin is
// decided in FP32 with an error bound like the 3-D bins (qinv_class).
// Called by all FT threads of the CTA; the caller syncs before reusing `sm`.
template <bool AZ, bool BOOST, int PREC, int MODE = MODE_FAST, bool QINV = false>
__device__ __forceinline__ void same_tile_pair(const Device &d, SmemFor<QINV> &sm,
                                               const double2 *cs,
                                               const double *const *c, const unsigned *orig,
                                               long long n, long long i0, long long j0) {
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    // split columns of the FP32-weight form, in the FP64 tiles' place
    float2(*spi)[FT] = reinterpret_cast<float2(*)[FT]>(&sm.si[0][0]);
    float2(*spj)[FT] = reinterpret_cast<float2(*)[FT]>(&sm.sj[0][0]);
    if (PREC == 0) {
        for (int f = 0; f < 8; f++) {
            sm.si[f][tid] = (i0 + tid < n) ? c[f][i0 + tid] : 0.0;
            sm.sj[f][tid] = (j0 + tid < n) ? c[f][j0 + tid] : 0.0;
        }
        sm.fi[tid] = make_float4((float)sm.si[0][tid], (float)sm.si[1][tid], (float)sm.si[2][tid],
                                 (float)sm.si[3][tid]);
        sm.fj[tid] = make_float4((float)sm.sj[0][tid], (float)sm.sj[1][tid], (float)sm.sj[2][tid],
                                 (float)sm.sj[3][tid]);
        if (BOOST) {
            sm.li[tid] = make_float2((float)(sm.si[2][tid] - (double)sm.fi[tid].z),
                                     (float)(sm.si[3][tid] - (double)sm.fi[tid].w));
            sm.lj[tid] = make_float2((float)(sm.sj[2][tid] - (double)sm.fj[tid].z),
                                     (float)(sm.sj[3][tid] - (double)sm.fj[tid].w));
        }
    } else if (PREC == 1) {
        for (int f = 0; f < 8; f++) {
            spi[f][tid] = split((i0 + tid < n) ? c[f][i0 + tid] : 0.0);
            spj[f][tid] = split((j0 + tid < n) ? c[f][j0 + tid] : 0.0);
        }
        // the high parts are the FP32 roundings of the momenta
        sm.fi[tid] = make_float4(spi[0][tid].x, spi[1][tid].x, spi[2][tid].x, spi[3][tid].x);
        sm.fj[tid] = make_float4(spj[0][tid].x, spj[1][tid].x, spj[2][tid].x, spj[3][tid].x);
    } else {
        // double-float form: momenta split relative to the tile's first row
        double vi[8], vj[8];
        for (int f = 0; f < 8; f++) {
            vi[f] = (i0 + tid < n) ? c[f][i0 + tid] : 0.0;
            vj[f] = (j0 + tid < n) ? c[f][j0 + tid] : 0.0;
        }
        for (int f = 0; f < 4; f++) {
            const float oi = (float)c[f][i0], oj = (float)c[f][j0];
            if (tid == 0) {
                sm.offi[f] = oi;
                sm.offj[f] = oj;
            }
            spi[f][tid] = split(vi[f] - (double)oi);
            spj[f][tid] = split(vj[f] - (double)oj);
        }
        for (int f = 4; f < 8; f++) {
            spi[f][tid] = split(vi[f]);
            spj[f][tid] = split(vj[f]);
        }
        sm.fi[tid] = make_float4((float)vi[0], (float)vi[1], (float)vi[2], (float)vi[3]);
        sm.fj[tid] = make_float4((float)vj[0], (float)vj[1], (float)vj[2], (float)vj[3]);
    }
    sm.oi[tid] = orig ? (i0 + tid < n ? orig[i0 + tid] : 0u) : (unsigned)(i0 + tid);
    sm.oj[tid] = orig ? (j0 + tid < n ? orig[j0 + tid] : 0u) : (unsigned)(j0 + tid);
    sm.gi[tid] = make_float2(fabsf(sm.fi[tid].x) + fabsf(sm.fi[tid].y), fabsf(sm.fi[tid].z));
    sm.gj[tid] = make_float2(fabsf(sm.fj[tid].x) + fabsf(sm.fj[tid].y), fabsf(sm.fj[tid].z));
    __syncthreads();
    const Screen &S = d.s;
    // warp w takes the tile's rows w, w + 4, w + 8, ...: the rows are sorted
    // in momentum space, so interleaving spreads each warp's rows over the
    // tile and evens out the binned pairs (the FP64 work) between warps
    const int il = lane * (FT / 32) + w;
    const long long i = i0 + il;
    const float4 a = sm.fi[il];
    const float2 ga = sm.gi[il];
    const unsigned oa = sm.oi[il];
    const int jend = (int)min((long long)FT, n - j0);
    unsigned *q = sm.queue[w];
    auto *q2 = sm.queue2[w];
    int count = 0, count2 = 0;

    // the q_inv form's stages exist only in its instantiation: a lambda that
    // captures the queue counters by reference, even unused, would take
    // their addresses and push them to local memory in the other forms
    if constexpr (QINV) {
        // stage C with q_inv histograms, for 32 screened pairs: the 3-D event
        // and the q_inv event of each pair (cos(q.dx) computed once for both)
        unsigned *q3 = sm.queue3[w];
        int count3 = 0;
        // the pairs left undecided, 32 at a time: the reference chain
        // decides both events
        auto chains_q = [&](unsigned e, bool valid) {
            if (!valid) return;
            const int qi = e & 0xff, qj = (e >> 8) & 0xff;
            const bool swap = (e >> 16) & 1u;
            double A[8], B[8];  // first and second particle of the pair
#pragma unroll
            for (int f = 0; f < 8; f++) {
                const double u = PREC == 0 ? sm.si[f][qi] : c[f][i0 + qi];
                const double v = PREC == 0 ? sm.sj[f][qj] : c[f][j0 + qj];
                A[f] = swap ? v : u;
                B[f] = swap ? u : v;
            }
            if (MODE == MODE_FAST) {
                undecided_pair_ordered<false, MODE_FAST>(d, A, B, i0 + qi, j0 + qj, n, n);
            } else {
                const long long oa = sm.oi[qi], ob = sm.oj[qj];
                const long long row = oa < ob ? oa : ob, col = oa < ob ? ob : oa;
                undecided_pair_ordered<false, MODE>(d, A, B, row, col, n, n);
            }
        };
        auto values_q = [&](uint4 e4, bool valid) {
            // this lane's q_inv event, added per group of lanes at the end
            unsigned qkey = 0xffffffffu;
            double qsum = 0.0, qw = 0.0;
            const unsigned e = e4.x;
            const int qi = e & 0xff, qj = (e >> 8) & 0xff;
            const bool swap = (e >> 16) & 1u;
            bool has3 = valid && ((e >> 18) & 1u), hasq = valid && ((e >> 19) & 1u);
            const int bin = (int)e4.y, slot = (int)(e4.z & 0xffffu), iK = (int)(e4.z >> 16);
            const int kq = (int)e4.w;
            double A[8], B[8];  // first and second particle of the pair
#pragma unroll
            for (int f = 0; f < 8; f++) {
                const double u = PREC == 0 ? sm.si[f][qi] : c[f][i0 + qi];
                const double v = PREC == 0 ? sm.sj[f][qj] : c[f][j0 + qj];
                A[f] = swap ? v : u;
                B[f] = swap ? u : v;
            }
            const long long oa = sm.oi[qi], ob = sm.oj[qj];
            const long long row = oa < ob ? oa : ob;
            // undecided: both events wait for the reference chain (stage D)
            const bool undecided = valid && ((e >> 17) & 1u);
            if (undecided) has3 = hasq = false;
            if (MODE != MODE_FAST) {
                has3 = has3 && admit<MODE>(d, slot, row, n);
                hasq = hasq && admit<MODE>(d, d.g.n_slots + iK, row, n);
            }
            if (has3 || hasq) {
                const long long at = (long long)slot * d.g.q3 + bin;
                double wq;
                if (PREC == 1) {
                    float2 a[8], b[8];
#pragma unroll
                    for (int f = 0; f < 8; f++) {
                        a[f] = spi[f][qi];
                        b[f] = spj[f][qj];
                    }
                    float4 v = values32_split<BOOST>(d.s, a, b);
                    if (swap) {
                        v.x = -v.x;
                        v.y = -v.y;
                        v.z = -v.z;
                    }
                    if (has3) {
                        atomicAdd(partials_of(d) + at, v);
                        atomicAdd(d.h.cnt + at, 1ull);
                    }
                    wq = v.w;
                } else {
                    double vo, vs, vl;
                    if (PREC == 0) {
                        FF sz = {0.0f, 0.0f}, sE = {0.0f, 0.0f};
                        if (BOOST) {
                            const float4 fa = sm.fi[qi], fb = sm.fj[qj];
                            const float2 la = sm.li[qi], lb = sm.lj[qj];
                            sz = ff_sum(make_float2(fa.z, la.x), make_float2(fb.z, lb.x));
                            sE = ff_sum(make_float2(fa.w, la.y), make_float2(fb.w, lb.y));
                        }
                        values64<BOOST>(d.g, cs, A, B, sz, sE, vo, vs, vl, wq);
                    } else {
                        float2 a[8], b[8];
#pragma unroll
                        for (int f = 0; f < 8; f++) {
                            a[f] = spi[f][qi];
                            b[f] = spj[f][qj];
                        }
                        values_df<BOOST>(d.s, reinterpret_cast<const float4 *>(cs), a, b,
                                         sm.offi, sm.offj, swap, vo, vs, vl, wq);
                    }
                    if (has3) {
                        Sums *h = d.h.sums + at;
                        atomicAdd(&h->qo, vo);
                        atomicAdd(&h->qs, vs);
                        atomicAdd(&h->ql, vl);
                        atomicAdd(&h->w, wq);
                        atomicAdd(d.h.cnt + at, 1ull);
                    }
                }
                if (hasq) {
                    // the reference's q_inv expression (FP64, same order, no
                    // contraction): the summed value equals the oracle's
                    const double q_x = A[0] - B[0], q_y = A[1] - B[1], q_z = A[2] - B[2];
                    const double q_E = A[3] - B[3];
                    qsum = sqrt(-(q_E * q_E - q_x * q_x - q_y * q_y - q_z * q_z));
                    qw = wq;
                    qkey = (unsigned)(iK * d.g.qnpts + kq);
                }
            }
            qinv_update(d, qkey, qsum, qw, true);
            enqueue(q3, count3, undecided, e & 0x1ffffu, lane, chains_q);
        };

        // stage B with q_inv histograms: the K_T window and bin, the 3-D
        // windows and bins, and the q_inv window and bin of each pair; a pair
        // with any of them undecided goes to the reference chain as a whole
        auto screen_q = [&](unsigned e, bool valid) {
            const int qi = e & 0xff, qj = (e >> 8) & 0xff;
            const bool swap = (e >> 16) & 1u;
            const float4 fa = swap ? sm.fj[qj] : sm.fi[qi], fb = swap ? sm.fi[qi] : sm.fj[qj];
            Q s;
            int c3 = 0, cq = 0, iK = -1, bin = 0, slot = -1, kq = 0;
            bool und = false;
            if (valid) {
                const int kt = screen_kt(S, fa, fb, s);
                if (kt != 0) {
                    c3 = screen_lcms<BOOST>(S, fa, fb, s);
                    cq = qinv_class(S, fa, fb, kq);
                    if (c3 == 1 || cq == 1) {
                        iK = kt == 1 ? kt_index(S, s) : -1;
                        und = iK < 0;
                    }
                    if (c3 == 1 && !und) {
                        int iK2 = 0;
                        if (decide_bins(S, s, iK2, bin)) {
                            slot = iK2;
                            if (AZ) {
                                const int ip = kphi_screen(S, s);
                                slot = ip < 0 ? -1 : iK2 * d.g.n_Kphi + ip;
                            }
                        }
                        und = slot < 0;
                    }
                    und = und || c3 == 2 || cq == 2;
                }
            }
            const bool take = valid && (und || c3 == 1 || cq == 1);
            const unsigned x = e | (und ? 1u << 17 : 0u) | (!und && c3 == 1 ? 1u << 18 : 0u) |
                               (!und && cq == 1 ? 1u << 19 : 0u);
            const uint4 ent = make_uint4(x, (unsigned)bin,
                                         (unsigned)(slot < 0 ? 0 : slot) |
                                             ((unsigned)(iK < 0 ? 0 : iK) << 16),
                                         (unsigned)kq);
            enqueue(q2, count2, take, ent, lane, values_q);
        };

        for (int jj = 0; jj < jend; jj++) {
            const long long j = j0 + jj;
            const bool swap = oa > sm.oj[jj];
            const bool take = i < n && j > i &&
                              (prefilter<BOOST>(S, a, ga, sm.fj[jj], sm.gj[jj]) ||
                               prefilter_qinv(S, a, sm.fj[jj]));
            enqueue(q, count, take,
                    (unsigned)il | ((unsigned)jj << 8) | ((swap ? 1u : 0u) << 16), lane,
                    screen_q);
        }
        drain(q, count, lane, screen_q);
        drain(q2, count2, lane, values_q);
        drain(q3, count3, lane, chains_q);
    } else {
        unsigned *q3 = sm.queue3[w];
        int count3 = 0;
        // stage D for 32 pairs the screen left undecided: the reference chain
        // decides them (and may hand a K_phi edge to the host), from the FP64
        // tile or (FP32-weight and double-float forms) the FP64 columns
        auto chains = [&](unsigned e, bool valid) {
            if (!valid) return;
            const int qi = e & 0xff, qj = (e >> 8) & 0xff;
            const bool swap = (e >> 16) & 1u;
            double A[8], B[8];  // first and second particle of the pair
#pragma unroll
            for (int f = 0; f < 8; f++) {
                const double u = PREC == 0 ? sm.si[f][qi] : c[f][i0 + qi];
                const double v = PREC == 0 ? sm.sj[f][qj] : c[f][j0 + qj];
                A[f] = swap ? v : u;
                B[f] = swap ? u : v;
            }
            if (MODE != MODE_FAST) {
                const long long oa = sm.oi[qi], ob = sm.oj[qj];
                const long long row = oa < ob ? oa : ob, col = oa < ob ? ob : oa;
                undecided_pair_ordered<false, MODE>(d, A, B, row, col, n, n);
                return;
            }
            if (PREC == 1)
                undecided_pair32<BOOST>(d, A, B, i0 + qi, j0 + qj, n);
            else
                undecided_pair64(d, A, B, i0 + qi, j0 + qj, n);
        };

        // stage C for one decided pair: its values into its bin
        auto decided = [&](uint2 e2) {
            const unsigned e = e2.x;
            const int qi = e & 0xff, qj = (e >> 8) & 0xff;
            const bool swap = (e >> 16) & 1u;
            const int slot = (int)(e >> 18);
            const int bin = (int)e2.y;
            if (MODE != MODE_FAST) {
                const long long oa = sm.oi[qi], ob = sm.oj[qj];
                const long long row = oa < ob ? oa : ob;
                if (!admit<MODE>(d, slot, row, n)) return;
            }
            if (PREC == 1) {
                // the pair as stored (i, j); swapping first and second negates
                // q_out, q_side, q_long exactly and leaves the phase unchanged
                float2 a[8], b[8];
#pragma unroll
                for (int f = 0; f < 8; f++) {
                    a[f] = spi[f][qi];
                    b[f] = spj[f][qj];
                }
                float4 v = values32_split<BOOST>(d.s, a, b);
                if (swap) {
                    v.x = -v.x;
                    v.y = -v.y;
                    v.z = -v.z;
                }
                const long long at = (long long)slot * d.g.q3 + bin;
                atomicAdd(partials_of(d) + at, v);
                atomicAdd(d.h.cnt + at, 1ull);
                return;
            }
            double vo, vs, vl, vw;
            if (PREC == 2) {
                float2 a[8], b[8];
#pragma unroll
                for (int f = 0; f < 8; f++) {
                    a[f] = spi[f][qi];
                    b[f] = spj[f][qj];
                }
                values_df<BOOST>(d.s, reinterpret_cast<const float4 *>(cs), a, b, sm.offi, sm.offj,
                                 swap, vo, vs, vl, vw);
            } else {
                // the pair in the reference's orientation, from the FP64 tile
                // (the two rows chosen once, then read column by column)
                const double *ra = swap ? &sm.sj[0][qj] : &sm.si[0][qi];
                const double *rb = swap ? &sm.si[0][qi] : &sm.sj[0][qj];
                double A[8], B[8];
#pragma unroll
                for (int f = 0; f < 8; f++) {
                    A[f] = ra[f * FT];
                    B[f] = rb[f * FT];
                }
                FF sz = {0.0f, 0.0f}, sE = {0.0f, 0.0f};
                if (BOOST) {
                    const float4 fa = sm.fi[qi], fb = sm.fj[qj];
                    const float2 la = sm.li[qi], lb = sm.lj[qj];
                    sz = ff_sum(make_float2(fa.z, la.x), make_float2(fb.z, lb.x));
                    sE = ff_sum(make_float2(fa.w, la.y), make_float2(fb.w, lb.y));
                }
                values64<BOOST>(d.g, cs, A, B, sz, sE, vo, vs, vl, vw);
            }
            const long long at = (long long)slot * d.g.q3 + bin;
            Sums *h = d.h.sums + at;
            atomicAdd(&h->qo, vo);
            atomicAdd(&h->qs, vs);
            atomicAdd(&h->ql, vl);
            atomicAdd(&h->w, vw);
            atomicAdd(d.h.cnt + at, 1ull);
        };

        // stage C for 32 screened pairs (all lanes of the warp in step): the
        // decided pairs' values, then the undecided ones to stage D's queue
        // (last, so that stage D runs with nothing of stage C live)
        auto values = [&](uint2 e2, bool valid) {
            const bool undecided = valid && ((e2.x >> 17) & 1u);
            if (valid && !undecided) decided(e2);
            enqueue(q3, count3, undecided, e2.x & 0x1ffffu, lane, chains);
        };

        // stage B for 32 prefiltered pairs: window screen and bins; the pairs
        // inside the window (or undecided) go to the second queue
        auto screen = [&](unsigned e, bool valid) {
            const int qi = e & 0xff, qj = (e >> 8) & 0xff;
            const bool swap = (e >> 16) & 1u;
            Q s;
            int wcls = 0;
            if (valid)
                wcls = swap ? screen_windows<BOOST>(S, sm.fj[qj], sm.fi[qi], s)
                            : screen_windows<BOOST>(S, sm.fi[qi], sm.fj[qj], s);
            int iK = 0, bin = 0, slot = -1;
            if (wcls == 1 && decide_bins(S, s, iK, bin)) {
                slot = iK;
                if (AZ) {
                    const int ip = kphi_screen(S, s);
                    slot = ip < 0 ? -1 : iK * d.g.n_Kphi + ip;
                }
            }
            enqueue(q2, count2, wcls != 0, bin_entry(e, slot < 0, slot < 0 ? 0 : slot, bin), lane,
                    values);
        };

        for (int jj = 0; jj < jend; jj++) {
            const long long j = j0 + jj;
            const bool swap = oa > sm.oj[jj];
            const bool take = i < n && j > i && prefilter<BOOST>(S, a, ga, sm.fj[jj], sm.gj[jj]);
            enqueue(q, count, take,
                    (unsigned)il | ((unsigned)jj << 8) | ((swap ? 1u : 0u) << 16), lane, screen);
        }
        drain(q, count, lane, screen);
        drain(q2, count2, lane, values);
        drain(q3, count3, lane, chains);
    }
}

// Mixed-event pairs of the list-1 tile at i0 (n1 particles, columns l1 =
// px py pz E) and the list-2 tile at j0 (n2 particles, columns l2).  Under
// ordered cap admission (MODE COUNT / ORDER) a pair's row and column are
// its positions in the caller's lists, orig1 / orig2 (nullptr: the rows are
// in the caller's order).
template <bool AZ, bool BOOST, int MODE = MODE_FAST, bool QINV = false, class SM = TileSmem>
__device__ __forceinline__ void mixed_tile_pair(const Device &d, SM &sm,
                                                const double *const *l1, long long n1,
                                                const double *const *l2, long long n2,
                                                long long i0, long long j0,
                                                const unsigned *orig1 = nullptr,
                                                const unsigned *orig2 = nullptr,
                                                long long row_base = 0) {
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    sm.fi[tid] = (i0 + tid < n1) ? make_float4((float)l1[0][i0 + tid], (float)l1[1][i0 + tid],
                                               (float)l1[2][i0 + tid], (float)l1[3][i0 + tid])
                                 : make_float4(0.f, 0.f, 0.f, 1.f);
    sm.fj[tid] = (j0 + tid < n2) ? make_float4((float)l2[0][j0 + tid], (float)l2[1][j0 + tid],
                                               (float)l2[2][j0 + tid], (float)l2[3][j0 + tid])
                                 : make_float4(0.f, 0.f, 0.f, 1.f);
    sm.gi[tid] = make_float2(fabsf(sm.fi[tid].x) + fabsf(sm.fi[tid].y), fabsf(sm.fi[tid].z));
    sm.gj[tid] = make_float2(fabsf(sm.fj[tid].x) + fabsf(sm.fj[tid].y), fabsf(sm.fj[tid].z));
    __syncthreads();
    const Screen &S = d.s;
    const int il = lane * (FT / 32) + w;  // interleaved rows, as in same_tile_pair
    const bool active = i0 + il < n1;
    const float4 a = sm.fi[il];
    const float2 ga = sm.gi[il];
    const int jend = (int)min((long long)FT, n2 - j0);
    unsigned *q = sm.queue[w];
    int count = 0;
    // ordered admission: row stride of the survivor counts and key stride of
    // the deferrals (several jobs admitted together, or this job alone)
    const long long rows = d.caps.rows_total ? d.caps.rows_total : n1;
    const long long cols = d.caps.cols_key ? d.caps.cols_key : n2;

    // pairs the screen left undecided, 32 at a time: the reference chain
    // decides (inline, a warp would run it for one or two lanes)
    unsigned *q3 = sm.queue3[w];
    int count3 = 0;
    auto chains = [&](unsigned e, bool valid) {
        if (!valid) return;
        const int qi = e & 0xff, qj = (e >> 8) & 0xff;
        if (MODE != MODE_FAST) {
            const long long row = row_base + (orig1 ? (long long)orig1[i0 + qi] : i0 + qi);
            const long long col = orig2 ? (long long)orig2[j0 + qj] : j0 + qj;
            const double A[4] = {l1[0][i0 + qi], l1[1][i0 + qi], l1[2][i0 + qi], l1[3][i0 + qi]};
            const double B[4] = {l2[0][j0 + qj], l2[1][j0 + qj], l2[2][j0 + qj], l2[3][j0 + qj]};
            undecided_pair_ordered<true, MODE>(d, A, B, row, col, rows, cols);
        } else {
            undecided_mixed_pair(d, l1, l2, i0 + qi, j0 + qj, n1, n2);
        }
    };

    // one screened pair: its denominator bin, or undecided (true)
    auto screened = [&](unsigned e) -> bool {
        const int qi = e & 0xff, qj = (e >> 8) & 0xff;
        Q s;
        const int wcls = screen_windows<BOOST>(S, sm.fi[qi], sm.fj[qj], s);
        if (wcls == 0) return false;
        int iK = 0, bin = 0, slot = -1;
        if (wcls == 1 && decide_bins(S, s, iK, bin)) {
            slot = iK;
            if (AZ) {
                const int ip = kphi_screen(S, s);
                slot = ip < 0 ? -1 : iK * d.g.n_Kphi + ip;
            }
        }
        if (slot < 0) return true;
        if (MODE != MODE_FAST) {
            const long long row = row_base + (orig1 ? (long long)orig1[i0 + qi] : i0 + qi);
            if (!admit<MODE>(d, slot, row, rows)) return false;
        }
        atomicAdd(d.h.den + (long long)slot * d.g.q3 + bin, 1ull);
        return false;
    };

    // 32 prefiltered pairs (all lanes of the warp in step)
    auto process = [&](unsigned e, bool valid) {
        const bool undecided = valid && screened(e);
        enqueue(q3, count3, undecided, e, lane, chains);
    };

    if constexpr (QINV) {
        // with q_inv histograms: the 3-D and the q_inv denominator events
        auto process_q = [&](unsigned e, bool valid) {
            const int qi = e & 0xff, qj = (e >> 8) & 0xff;
            unsigned qkey = 0xffffffffu;  // this lane's q_inv denominator bin
            bool undecided = false;       // both events wait for the chain
            if (valid) {
                Q s;
                const int kt = screen_kt(S, sm.fi[qi], sm.fj[qj], s);
                int c3 = 0, cq = 0, kq = 0, iK = -1, bin = 0, slot = -1;
                if (kt != 0) {
                    c3 = screen_lcms<BOOST>(S, sm.fi[qi], sm.fj[qj], s);
                    cq = qinv_class(S, sm.fi[qi], sm.fj[qj], kq);
                }
                bool und = false;
                if (c3 == 1 || cq == 1) {
                    iK = kt == 1 ? kt_index(S, s) : -1;
                    und = iK < 0;
                }
                if (c3 == 1 && !und) {
                    int iK2 = 0;
                    if (decide_bins(S, s, iK2, bin)) {
                        slot = iK2;
                        if (AZ) {
                            const int ip = kphi_screen(S, s);
                            slot = ip < 0 ? -1 : iK2 * d.g.n_Kphi + ip;
                        }
                    }
                    und = slot < 0;
                }
                und = und || c3 == 2 || cq == 2;
                const long long row = row_base + (orig1 ? (long long)orig1[i0 + qi] : i0 + qi);
                undecided = und;
                if (!und) {
                    bool h3 = c3 == 1, hq = cq == 1;
                    if (MODE != MODE_FAST) {
                        h3 = h3 && admit<MODE>(d, slot, row, rows);
                        hq = hq && admit<MODE>(d, d.g.n_slots + iK, row, rows);
                    }
                    if (h3) atomicAdd(d.h.den + (long long)slot * d.g.q3 + bin, 1ull);
                    if (hq) qkey = (unsigned)(iK * d.g.qnpts + kq);
                }
            }
            qinv_update(d, qkey, 0.0, 0.0, false);
            enqueue(q3, count3, undecided, e, lane, chains);
        };

        for (int jj = 0; jj < jend; jj++) {
            const bool take = active && (prefilter<BOOST>(S, a, ga, sm.fj[jj], sm.gj[jj]) ||
                                         prefilter_qinv(S, a, sm.fj[jj]));
            enqueue(q, count, take, (unsigned)il | ((unsigned)jj << 8), lane, process_q);
        }
        drain(q, count, lane, process_q);
        drain(q3, count3, lane, chains);
    } else {
        for (int jj = 0; jj < jend; jj++) {
            const bool take = active && prefilter<BOOST>(S, a, ga, sm.fj[jj], sm.gj[jj]);
            enqueue(q, count, take, (unsigned)il | ((unsigned)jj << 8), lane, process);
        }
        drain(q, count, lane, process);
        drain(q3, count3, lane, chains);
    }
}

}  // namespace tile
}  // namespace hbt
