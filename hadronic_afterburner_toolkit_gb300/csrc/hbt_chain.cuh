// Device-side pieces shared by the pair-binning kernels: the reference's
// FP64 decision chain, histogram updates, K_phi deferrals and the
// admission-mode dispatch.  Included by hbt_kernels.cu and hbt_fast.cu.
#pragma once

#include "hbt_engine.cuh"

namespace hbt {
namespace chain {

constexpr int TILE = 128;

struct Cols8 {
    const double *p[8];  // px py pz E x y z t
};
struct Cols4 {
    const double *p[4];  // px py pz E
};

// Result of one pair's decision chain.
struct Chain {
    int iK;       // K_T bin, -1: K_T cut failed (or anomaly)
    int qi_k;     // q_inv bin, -1: no q_inv event
    int ev3;      // 0: no 3-D event, 1: event in `slot`, 2: K_phi deferred
    int slot;     // 3-D slot
    int bin;      // (iqout*qnpts + iqside)*qnpts + iqlong
    int anomaly;  // NaN LCMS component / K_T index out of range
    double qinv, qo, qs, ql, phase, Kx, Ky;
};

// K_phi bin of the pair (src/HBT_correlation.cpp:408-423): -1 out of
// range, -2 within kphi_tol of an edge or of the 0 / 2 pi wrap (the host
// decides those with the C library's atan2).
__device__ __forceinline__ int kphi_bin(const Grid &g, double Kx, double Ky) {
    const double phi = atan2(Ky, Kx);
    double d = phi - g.psi_ref;
    if (fabs(d) <= g.kphi_tol || fabs(d - g.two_pi) <= g.kphi_tol) return -2;
    while (d < 0.) d += g.two_pi;
    while (d > g.two_pi) d -= g.two_pi;
    if (d <= g.kphi_tol || g.two_pi - d <= g.kphi_tol) return -2;
    const double r = d / g.dKphi;
    const double nearest = rint(r);
    if (fabs(r - nearest) * g.dKphi <= g.kphi_tol) return -2;
    const int ip = static_cast<int>(r);
    if (ip < 0 || ip >= g.n_Kphi) return -1;
    return ip;
}

// The reference's per-pair chain.  MIXED selects the mixed-event variant
// (inclusive upper window bounds, q_inv index check, no space-time phase).
template <bool MIXED>
__device__ __forceinline__ Chain pair_chain(const Grid &g, double apx, double apy,
                                            double apz, double aE, double bpx,
                                            double bpy, double bpz, double bE,
                                            const double *ax, const double *bx) {
    Chain c;
    c.iK = -1;
    c.qi_k = -1;
    c.ev3 = 0;
    c.anomaly = 0;
    const double K_z = 0.5 * (apz + bpz);
    const double K_E = 0.5 * (aE + bE);
    const double K_x = 0.5 * (apx + bpx);
    const double K_y = 0.5 * (apy + bpy);
    const double Kp2 = K_x * K_x + K_y * K_y;
    if (Kp2 < g.KT_min_sq || Kp2 > g.KT_max_sq) return c;
    const double Kp = sqrt(Kp2);
    const int iK = static_cast<int>((Kp - g.KT_min) / g.dKT);
    if (iK < 0 || iK >= g.n_KT) {
        c.anomaly = 1;
        return c;
    }
    c.iK = iK;
    const double q_x = apx - bpx;
    const double q_y = apy - bpy;
    const double q_z = apz - bpz;
    const double q_E = aE - bE;
    if (!MIXED) {
        // x, y, z, t differences for the phase (q.dx)/hbarC
        const double dt = ax[3] - bx[3];
        const double dx = ax[0] - bx[0];
        const double dy = ax[1] - bx[1];
        const double dz = ax[2] - bx[2];
        c.phase = g.hbarC_inv * (q_E * dt - q_x * dx - q_y * dy - q_z * dz);
    }
    if (g.qinv) {
        const double qinv = sqrt(-(q_E * q_E - q_x * q_x - q_y * q_y - q_z * q_z));
        if (qinv > g.q_lo && qinv < g.q_hi) {
            const int k = static_cast<int>((qinv - g.q_base) / g.delta_q);
            if (k < g.qnpts) {
                c.qi_k = k;
                c.qinv = qinv;
            } else if (!MIXED) {
                // the reference indexes past its array here (no check on the
                // numerator side); never reached for a window inside the grid
                c.anomaly = 1;
            }
        }
    }
    const double cphi = K_x / Kp;
    const double sphi = K_y / Kp;
    const double qo = q_x * cphi + q_y * sphi;
    if (qo != qo) {
        c.anomaly = 1;
        return c;
    }
    if (qo < g.q_lo || (MIXED ? qo >= g.q_hi : qo > g.q_hi)) return c;
    const int io = static_cast<int>((qo - g.q_base) / g.delta_q);
    if (io >= g.qnpts) return c;
    const double qs = q_y * cphi - q_x * sphi;
    if (qs != qs) {
        c.anomaly = 1;
        return c;
    }
    if (qs < g.q_lo || (MIXED ? qs >= g.q_hi : qs > g.q_hi)) return c;
    const int is = static_cast<int>((qs - g.q_base) / g.delta_q);
    if (is >= g.qnpts) return c;
    double ql = q_z;
    if (g.boost) {
        const double Mt = sqrt(K_E * K_E - K_z * K_z);
        const double gamma = K_E / Mt;
        const double beta = K_z / K_E;
        ql = gamma * (q_z - beta * q_E);
    }
    if (ql != ql) {
        c.anomaly = 1;
        return c;
    }
    if (ql < g.q_lo || (MIXED ? ql >= g.q_hi : ql > g.q_hi)) return c;
    const int il = static_cast<int>((ql - g.q_base) / g.delta_q);
    if (il >= g.qnpts) return c;
    c.bin = (io * g.qnpts + is) * g.qnpts + il;
    c.qo = qo;
    c.qs = qs;
    c.ql = ql;
    c.Kx = K_x;
    c.Ky = K_y;
    if (g.azimuthal) {
        const int ip = kphi_bin(g, K_x, K_y);
        if (ip == -1) return c;
        if (ip == -2) {
            c.ev3 = 2;
            return c;
        }
        c.slot = iK * g.n_Kphi + ip;
    } else {
        c.slot = iK;
    }
    c.ev3 = 1;
    return c;
}

// Histogram updates ---------------------------------------------------------

__device__ __forceinline__ void bin_num3(const Device &d, int slot, int bin,
                                         const Chain &c) {
    const long long at = (long long)slot * d.g.q3 + bin;
    Sums *s = d.h.sums + at;
    atomicAdd(&s->qo, c.qo);
    atomicAdd(&s->qs, c.qs);
    atomicAdd(&s->ql, c.ql);
    atomicAdd(&s->w, cos(c.phase));
    atomicAdd(d.h.cnt + at, 1ull);
}

__device__ __forceinline__ void bin_den3(const Device &d, int slot, int bin) {
    atomicAdd(d.h.den + (long long)slot * d.g.q3 + bin, 1ull);
}

__device__ __forceinline__ void bin_num_qinv(const Device &d, const Chain &c) {
    const int at = c.iK * d.g.qnpts + c.qi_k;
    atomicAdd(&d.h.qi_sums[at].q, c.qinv);
    atomicAdd(&d.h.qi_sums[at].w, cos(c.phase));
    atomicAdd(d.h.qi_cnt + at, 1ull);
}

__device__ __forceinline__ void bin_den_qinv(const Device &d, const Chain &c) {
    atomicAdd(d.h.qi_den + c.iK * d.g.qnpts + c.qi_k, 1ull);
}

template <bool MIXED>
__device__ __forceinline__ void push_deferral(const Device &d, long long i, long long j,
                                              const Chain &c) {
    const unsigned k = atomicAdd(d.n_defer, 1u);
    atomicAdd(d.stats + STAT_DEFER, 1ull);
    if (k < d.defer_cap) {
        Deferral r;
        r.i = i;
        r.j = j;
        r.Kx = c.Kx;
        r.Ky = c.Ky;
        r.psi = d.g.psi_ref;
        r.mixed = MIXED ? 1 : 0;
        r.pad = 0;
        r.qo = c.qo;
        r.qs = c.qs;
        r.ql = c.ql;
        r.cosw = MIXED ? 0.0 : cos(c.phase);
        r.iK = c.iK;
        r.bin = c.bin;
        d.defer[k] = r;
    } else {
        atomicAdd(d.stats + STAT_ERROR, 1ull);
    }
}

// Slot of a deferred pair from the host-resolved table (-1: skip).
__device__ __forceinline__ int resolved_slot(const Device &d, long long key, int iK) {
    int lo = 0, hi = d.caps.n_resolved - 1;
    while (lo <= hi) {
        const int mid = (lo + hi) >> 1;
        const long long k = d.caps.resolved[mid].key;
        if (k == key) {
            const int ip = d.caps.resolved[mid].iphi;
            return ip < 0 ? -1 : iK * d.g.n_Kphi + ip;
        }
        if (k < key)
            lo = mid + 1;
        else
            hi = mid - 1;
    }
    atomicAdd(d.stats + STAT_ERROR, 1ull);
    return -1;
}

// Consumes one pair's chain according to the admission mode.
template <bool MIXED, int MODE>
__device__ __forceinline__ void consume(const Device &d, long long i, long long j,
                                        long long cols, long long rows, const Chain &c) {
    if (c.anomaly) atomicAdd(d.stats + STAT_ANOMALY, 1ull);
    if (c.iK < 0) return;
    const int ns = d.g.n_slots;
    if (c.qi_k >= 0) {
        const int b = ns + c.iK;
        if (MODE == MODE_FAST) {
            if (MIXED)
                bin_den_qinv(d, c);
            else
                bin_num_qinv(d, c);
        } else if (MODE == MODE_COUNT) {
            atomicAdd(d.caps.rowcnt + (long long)b * rows + i, 1u);
        } else if (i < d.caps.row_cut[b]) {
            if (MIXED)
                bin_den_qinv(d, c);
            else
                bin_num_qinv(d, c);
        }
    }
    if (c.ev3 == 0) return;
    int slot = c.slot;
    if (c.ev3 == 2) {
        if (MODE != MODE_ORDER) {
            push_deferral<MIXED>(d, i, j, c);
            return;
        }
        slot = resolved_slot(d, i * cols + j, c.iK);
        if (slot < 0) return;
    }
    if (MODE == MODE_FAST) {
        if (MIXED)
            bin_den3(d, slot, c.bin);
        else
            bin_num3(d, slot, c.bin, c);
    } else if (MODE == MODE_COUNT) {
        atomicAdd(d.caps.rowcnt + (long long)slot * rows + i, 1u);
    } else if (i < d.caps.row_cut[slot]) {
        if (MIXED)
            bin_den3(d, slot, c.bin);
        else
            bin_num3(d, slot, c.bin, c);
    }
}

__device__ __forceinline__ void tri_tile(long long k, long long &ti, long long &tj) {
    long long b = (long long)((sqrt(8.0 * (double)k + 1.0) - 1.0) * 0.5);
    while (b * (b + 1) / 2 > k) b--;
    while ((b + 1) * (b + 2) / 2 <= k) b++;
    tj = b;
    ti = k - b * (b + 1) / 2;
}

}  // namespace chain
}  // namespace hbt
