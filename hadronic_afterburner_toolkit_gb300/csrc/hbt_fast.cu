// Screened pair-binning kernels for sm_103a (fast admission mode).
//
// GB300 runs FP64 at 1/58 of its FP32 rate, so every pair is first screened
// in FP32 and only the pairs that are binned pay for FP64 work:
//
//  1. FP32 screen (all pairs).  From FP32 copies of the momenta it computes
//     K_perp^2, q_out, q_side, q_long and a rigorous per-pair bound on how far
//     each may lie from the value the reference computes in FP64 (error
//     analysis below).  A pair is REJECTED when a window check fails by more
//     than its bound, ACCEPTED with its K_T and q bin indices when every
//     window check and every truncation to a bin index is farther from its
//     edge than the bound, and UNCERTAIN otherwise.  Accepted bins are
//     therefore exactly the reference's; uncertain pairs (a few in 10^4 of
//     the binned ones) run the reference-order FP64 chain of hbt_chain.cuh.
//  2. Same-event survivors are compacted per warp in shared memory and
//     processed 32 at a time with full lanes: FP64 q components, the
//     space-time phase and cos(q.dx), then the histogram atomics.  The
//     summed values come from algebraically identical FP64 expressions
//     (q_out = (q_x S_x + q_y S_y) / |S|, ...), so they differ from the
//     reference's per-pair values in the last bits only.
//  3. Mixed-event survivors only add 1 to a denominator bin: accepted pairs
//     do it straight from the screen, with no FP64 arithmetic at all.
//
// K_phi bins (azimuthal_flag = 1) are decided after the screen with an FP32
// atan2f and its error bound; pairs too close to an edge take the FP64
// path, which may in turn hand them to the host's atan2.
//
// Error analysis (u = 2^-24).  Inputs are FP64 values v rounded once to
// FP32: |v32 - v| <= u|v|.  For s = a +- b in FP32, |s - S| <= 2.01 u A with
// A = |a| + |b| and S the exact sum of the FP64 inputs.  Products, sums and
// the reciprocal square root (rsqrtf: at most 2 ulp) propagate this as coded
// in screen_*() below; every bound is then doubled and widened by the
// rounding of the FP32 copies of the constants, which also covers the FP64
// reference's own rounding (2^-29 times smaller).
#include "hbt_chain.cuh"

namespace hbt {
namespace {

using namespace chain;

constexpr float U = 5.9604645e-8f;  // 2^-24
constexpr int FT = 128;             // tile edge (particles) for both lists
constexpr int QCAP = 64;            // per-warp compaction queue

// One FP32 quantity of the screen: the value and its error bound.
struct VE {
    float v, e;
};

// 0: certainly outside [lo, hi], 1: certainly inside, 2: undecided.
__device__ __forceinline__ int window_class(const Screen &S, VE x) {
    const float e = 2.0f * x.e + S.win_slack;
    if (x.v + e < S.lo || x.v - e > S.hi) return 0;
    if (x.v - e > S.lo && x.v + e < S.hi) return 1;
    return 2;
}

// Bin index floor((v - base)/delta_q) if certain, else -1.
__device__ __forceinline__ int bin_index(const Screen &S, VE x) {
    const float t = (x.v - S.base) * S.inv_dq;
    const float et = (2.0f * x.e + S.win_slack) * S.inv_dq + 4.0f * U * fabsf(t) +
                     2.0f * U * (fabsf(x.v) + fabsf(S.base)) * S.inv_dq + S.t_slack;
    const float k = floorf(t - et);
    if (k != floorf(t + et) || k < 0.0f || k >= (float)S.qnpts) return -1;
    return (int)k;
}

// Screen of one pair.  Returns 0 (reject), 1 (accept: iK, bin set), 2
// (undecided).  sx, sy, Ax, Ay, k2 are returned for the K_phi decision.
template <bool BOOST>
__device__ __forceinline__ int screen_pair(const Screen &S, float4 a, float4 b, int &iK,
                                           int &bin, float &sx, float &sy, float &Ax,
                                           float &Ay, float &k2) {
    sx = a.x + b.x;
    sy = a.y + b.y;
    const float dx = a.x - b.x, dy = a.y - b.y;
    Ax = fabsf(a.x) + fabsf(b.x);
    Ay = fabsf(a.y) + fabsf(b.y);
    k2 = __fmaf_rn(sx, sx, sy * sy);
    const float AA = __fmaf_rn(Ax, Ax, Ay * Ay);
    // |k2 - (S_x^2 + S_y^2)|
    const float ek2 = 6.1f * U * __fmaf_rn(Ax, fabsf(sx), Ay * fabsf(sy)) + 3.1f * U * k2 +
                      1e-13f * AA;
    // K_T window: reference rejects 4 Kp2 < 4 KT_min^2 or > 4 KT_max^2
    const float ekt = 2.0f * ek2 + S.kt_slack;
    const bool kt_out = (S.kt_lo4 > 0.0f && k2 + ekt < S.kt_lo4) || (k2 - ekt > S.kt_hi4);
    if (kt_out) return 0;
    int cls = 1;
    if (!((S.kt_lo4 == 0.0f || k2 - ekt > S.kt_lo4) && k2 + ekt < S.kt_hi4)) cls = 2;
    const float rel_k2 = ek2 / k2;
    if (!(k2 > 0.0f) || rel_k2 > 0.05f) return 2;  // bounds below need a usable |S|
    // K_T bin: (|S|/2 - KT_min) / dKT
    {
        const float rk = __fsqrt_rn(k2);
        const float kp = 0.5f * rk;
        const float ekp = 0.5f * (ek2 / rk) + U * kp;
        const float t = (kp - S.KT_min) * S.inv_dKT;
        const float et = 2.0f * ekp * S.inv_dKT + 4.0f * U * (fabsf(t) + S.KT_min * S.inv_dKT) +
                         S.kt_t_slack;
        const float k = floorf(t - et);
        if (k != floorf(t + et) || k < 0.0f || k >= (float)S.n_KT) cls = 2;
        iK = (int)k;
    }
    const float inv = rsqrtf(k2);
    const float rel_inv = 0.53f * rel_k2 + 4.5f * U;
    const float eN = 9.0f * U * AA;
    const float no = __fmaf_rn(dx, sx, dy * sy);
    const float ns = __fmaf_rn(dy, sx, -(dx * sy));
    VE qo, qs, ql;
    qo.v = no * inv;
    qo.e = __fmaf_rn(fabsf(no), rel_inv, eN) * inv + U * fabsf(qo.v);
    qs.v = ns * inv;
    qs.e = __fmaf_rn(fabsf(ns), rel_inv, eN) * inv + U * fabsf(qs.v);
    const float dz = a.z - b.z;
    const float Az = fabsf(a.z) + fabsf(b.z);
    if (BOOST) {
        const float sE = a.w + b.w, sz = a.z + b.z, dE = a.w - b.w;
        const float AE = fabsf(a.w) + fabsf(b.w);
        const float m = sE - sz, p = sE + sz;
        const float em = 2.01f * U * (AE + Az) + U * fabsf(m);
        const float ep = 2.01f * U * (AE + Az) + U * fabsf(p);
        const float rel_m2 = em / m + ep / p + 1.01f * U;
        if (!(m > 0.0f) || !(p > 0.0f) || rel_m2 > 0.05f) return 2;
        const float rl = rsqrtf(m * p);
        const float rel_rl = 0.53f * rel_m2 + 4.5f * U;
        const float nl = __fmaf_rn(sE, dz, -(sz * dE));
        ql.v = nl * rl;
        ql.e = __fmaf_rn(fabsf(nl), rel_rl, 17.0f * U * AE * Az) * rl + U * fabsf(ql.v);
    } else {
        ql.v = dz;
        ql.e = 2.1f * U * Az;
    }
    const int wo = window_class(S, qo), ws = window_class(S, qs), wl = window_class(S, ql);
    if (wo == 0 || ws == 0 || wl == 0) return 0;
    if (wo == 2 || ws == 2 || wl == 2 || cls == 2) return 2;
    const int io = bin_index(S, qo), is = bin_index(S, qs), il = bin_index(S, ql);
    if (io < 0 || is < 0 || il < 0) return 2;
    bin = (io * S.qnpts + is) * S.qnpts + il;
    return 1;
}

// K_phi bin from the FP32 screen values: >= 0 certain, -2 undecided.
__device__ __forceinline__ int kphi_screen(const Screen &S, float sx, float sy, float Ax,
                                           float Ay, float k2) {
    const float phi = atan2f(sy, sx);
    // angle error from the inputs, atan2f (3 ulp), psi_ref rounding, wrap
    const float e = 2.01f * U * __fmaf_rn(Ax, fabsf(sy), Ay * fabsf(sx)) / k2 + 1.0e-6f +
                    S.psi_slack;
    float d = phi - S.psi;
    if (d < 0.0f) d += S.two_pi;
    const float ed = 2.0f * e + 1.0e-6f;
    if (d < ed || d > S.two_pi - ed) return -2;
    const float r = d * S.inv_dKphi;
    const float er = ed * S.inv_dKphi + 4.0f * U * r;
    const float k = floorf(r - er);
    if (k != floorf(r + er) || k < 0.0f || k >= (float)S.n_Kphi) return -2;
    return (int)k;
}

// FP64 summed values of an accepted same-event pair (algebraically the
// reference's q_out, q_side, q_long and cos(q.dx / hbarC)).
template <bool BOOST>
__device__ __forceinline__ void values64(const Grid &g, const double *a, const double *b,
                                         double &qo, double &qs, double &ql, double &w) {
    const double sx = a[0] + b[0], sy = a[1] + b[1];
    const double dx = a[0] - b[0], dy = a[1] - b[1];
    const double dz = a[2] - b[2], dE = a[3] - b[3];
    const double inv = rsqrt(__fma_rn(sx, sx, sy * sy));
    qo = __fma_rn(dx, sx, dy * sy) * inv;
    qs = __fma_rn(dy, sx, -(dx * sy)) * inv;
    if (BOOST) {
        const double sE = a[3] + b[3], sz = a[2] + b[2];
        ql = __fma_rn(sE, dz, -(sz * dE)) * rsqrt((sE - sz) * (sE + sz));
    } else {
        ql = dz;
    }
    const double ph = dE * (a[7] - b[7]) - dx * (a[4] - b[4]) - dy * (a[5] - b[5]) -
                      dz * (a[6] - b[6]);
    w = cos(g.hbarC_inv * ph);
}

// Same-event pairs, FP64 sums.  One CTA per (i-tile <= j-tile); warp w owns
// i = ti*FT + 32w + lane and sweeps the j-tile.
template <bool AZ, bool BOOST>
__global__ void __launch_bounds__(FT) k_same_screened(Device d, long long n, Cols8 c) {
    __shared__ double si[8][FT];
    __shared__ double sj[8][FT];
    __shared__ float4 fj[FT];
    __shared__ uint2 queue[FT / 32][QCAP];
    long long ti, tj;
    tri_tile(blockIdx.x, ti, tj);
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const long long i0 = ti * FT, j0 = tj * FT;
    for (int f = 0; f < 8; f++) {
        si[f][tid] = (i0 + tid < n) ? c.p[f][i0 + tid] : 0.0;
        sj[f][tid] = (j0 + tid < n) ? c.p[f][j0 + tid] : 0.0;
    }
    __syncthreads();
    fj[tid] = make_float4((float)sj[0][tid], (float)sj[1][tid], (float)sj[2][tid],
                          (float)sj[3][tid]);
    __syncthreads();
    const Screen &S = d.s;
    const int il = w * 32 + lane;
    const long long i = i0 + il;
    const float4 a = make_float4((float)si[0][il], (float)si[1][il], (float)si[2][il],
                                 (float)si[3][il]);
    const int jend = (int)min((long long)FT, n - j0);
    uint2 *q = queue[w];
    int count = 0;

    // FP64 stage of one queued pair (all lanes of the warp in step)
    auto process = [&](uint2 e) {
        const int qi = e.x & 0xff, qj = (e.x >> 8) & 0xff, cls = (e.x >> 16) & 0xff;
        double A[8], B[8];
#pragma unroll
        for (int f = 0; f < 8; f++) {
            A[f] = si[f][qi];
            B[f] = sj[f][qj];
        }
        if (cls == 1) {
            const int iK = (int)(e.x >> 24);
            int slot = iK;
            double vo, vs, vl, vw;
            values64<BOOST>(d.g, A, B, vo, vs, vl, vw);
            if (AZ) {
                // K_phi: FP32 first, FP64 (and host) for edge cases
                const float fsx = (float)A[0] + (float)B[0], fsy = (float)A[1] + (float)B[1];
                const float fAx = fabsf((float)A[0]) + fabsf((float)B[0]);
                const float fAy = fabsf((float)A[1]) + fabsf((float)B[1]);
                int ip = kphi_screen(S, fsx, fsy, fAx, fAy, __fmaf_rn(fsx, fsx, fsy * fsy));
                if (ip == -2) {
                    const double Kx = 0.5 * (A[0] + B[0]), Ky = 0.5 * (A[1] + B[1]);
                    ip = kphi_bin(d.g, Kx, Ky);
                    if (ip == -1) return;
                    if (ip == -2) {
                        Chain full = pair_chain<false>(d.g, A[0], A[1], A[2], A[3], B[0], B[1],
                                                       B[2], B[3], A + 4, B + 4);
                        consume<false, MODE_FAST>(d, i0 + qi, j0 + qj, n, n, full);
                        return;
                    }
                }
                slot = iK * d.g.n_Kphi + ip;
            }
            const long long at = (long long)slot * d.g.q3 + e.y;
            Sums *s = d.h.sums + at;
            atomicAdd(&s->qo, vo);
            atomicAdd(&s->qs, vs);
            atomicAdd(&s->ql, vl);
            atomicAdd(&s->w, vw);
            atomicAdd(d.h.cnt + at, 1ull);
        } else {
            const Chain full = pair_chain<false>(d.g, A[0], A[1], A[2], A[3], B[0], B[1], B[2],
                                                 B[3], A + 4, B + 4);
            consume<false, MODE_FAST>(d, i0 + qi, j0 + qj, n, n, full);
        }
    };

    for (int jj = 0; jj < jend; jj++) {
        const long long j = j0 + jj;
        const float4 b = fj[jj];
        int cls = 0, iK = 0, bin = 0;
        float sx, sy, Ax, Ay, k2;
        if (i < n && j > i) cls = screen_pair<BOOST>(S, a, b, iK, bin, sx, sy, Ax, Ay, k2);
        const unsigned m = __ballot_sync(0xffffffffu, cls != 0);
        if (m) {
            if (cls != 0) {
                const int pos = count + __popc(m & ((1u << lane) - 1u));
                q[pos] = make_uint2((unsigned)il | ((unsigned)jj << 8) | ((unsigned)cls << 16) |
                                        ((unsigned)iK << 24),
                                    (unsigned)bin);
            }
            count += __popc(m);
            __syncwarp();
            if (count >= 32) {
                process(q[lane]);
                __syncwarp();
                if (lane < count - 32) q[lane] = q[32 + lane];
                __syncwarp();
                count -= 32;
            }
        }
    }
    if (lane < count) process(q[lane]);
}

// Mixed-event pairs: list1 tile x list2 tile; accepted pairs add 1 to their
// denominator bin straight from the screen.
template <bool AZ, bool BOOST>
__global__ void __launch_bounds__(FT) k_mixed_screened(Device d, long long n1, Cols4 l1,
                                                       long long n2, Cols4 l2, long long tiles1) {
    __shared__ float4 fj[FT];
    const long long ti = blockIdx.x % tiles1, tj = blockIdx.x / tiles1;
    const int tid = threadIdx.x;
    const long long j0 = tj * FT;
    if (j0 + tid < n2)
        fj[tid] = make_float4((float)l2.p[0][j0 + tid], (float)l2.p[1][j0 + tid],
                              (float)l2.p[2][j0 + tid], (float)l2.p[3][j0 + tid]);
    __syncthreads();
    const long long i = ti * FT + tid;
    if (i >= n1) return;
    const float4 a = make_float4((float)l1.p[0][i], (float)l1.p[1][i], (float)l1.p[2][i],
                                 (float)l1.p[3][i]);
    const Screen &S = d.s;
    const int jend = (int)min((long long)FT, n2 - j0);
    for (int jj = 0; jj < jend; jj++) {
        int iK = 0, bin = 0;
        float sx, sy, Ax, Ay, k2;
        int cls = screen_pair<BOOST>(S, a, fj[jj], iK, bin, sx, sy, Ax, Ay, k2);
        int slot = iK;
        if (AZ && cls == 1) {
            const int ip = kphi_screen(S, sx, sy, Ax, Ay, k2);
            if (ip < 0)
                cls = 2;
            else
                slot = iK * d.g.n_Kphi + ip;
        }
        if (cls == 1) {
            atomicAdd(d.h.den + (long long)slot * d.g.q3 + bin, 1ull);
        } else if (cls == 2) {
            const long long j = j0 + jj;
            const Chain ch = pair_chain<true>(d.g, l1.p[0][i], l1.p[1][i], l1.p[2][i], l1.p[3][i],
                                              l2.p[0][j], l2.p[1][j], l2.p[2][j], l2.p[3][j],
                                              nullptr, nullptr);
            consume<true, MODE_FAST>(d, i, j, n2, n1, ch);
        }
    }
}

}  // namespace

cudaError_t launch_same_fast(const Device &d, long long n, const double *const *c8,
                             cudaStream_t st) {
    if (n < 2) return cudaSuccess;
    const long long nt = (n + FT - 1) / FT;
    const long long blocks = nt * (nt + 1) / 2;
    if (blocks > 0x7fffffffLL) return cudaErrorInvalidValue;
    Cols8 c;
    for (int f = 0; f < 8; f++) c.p[f] = c8[f];
    const bool az = d.g.azimuthal, boost = d.g.boost;
    if (az && boost)
        k_same_screened<true, true><<<(unsigned)blocks, FT, 0, st>>>(d, n, c);
    else if (az)
        k_same_screened<true, false><<<(unsigned)blocks, FT, 0, st>>>(d, n, c);
    else if (boost)
        k_same_screened<false, true><<<(unsigned)blocks, FT, 0, st>>>(d, n, c);
    else
        k_same_screened<false, false><<<(unsigned)blocks, FT, 0, st>>>(d, n, c);
    return cudaGetLastError();
}

cudaError_t launch_mixed_fast(const Device &d, long long n1, const double *const *l1,
                              long long n2, const double *const *l2, cudaStream_t st) {
    if (n1 < 1 || n2 < 1) return cudaSuccess;
    const long long t1 = (n1 + FT - 1) / FT, t2 = (n2 + FT - 1) / FT;
    const long long blocks = t1 * t2;
    if (blocks > 0x7fffffffLL) return cudaErrorInvalidValue;
    Cols4 a, b;
    for (int f = 0; f < 4; f++) {
        a.p[f] = l1[f];
        b.p[f] = l2[f];
    }
    const bool az = d.g.azimuthal, boost = d.g.boost;
    if (az && boost)
        k_mixed_screened<true, true><<<(unsigned)blocks, FT, 0, st>>>(d, n1, a, n2, b, t1);
    else if (az)
        k_mixed_screened<true, false><<<(unsigned)blocks, FT, 0, st>>>(d, n1, a, n2, b, t1);
    else if (boost)
        k_mixed_screened<false, true><<<(unsigned)blocks, FT, 0, st>>>(d, n1, a, n2, b, t1);
    else
        k_mixed_screened<false, false><<<(unsigned)blocks, FT, 0, st>>>(d, n1, a, n2, b, t1);
    return cudaGetLastError();
}

}  // namespace hbt
