// CPU oracle for the HBT pair-binning path - TEST INFRASTRUCTURE ONLY.
//
// A sequential restatement of the reference's algorithm in
// src/HBT_correlation.cpp (chunshen1987/hadronic_afterburner_toolkit).  Every
// floating-point expression that decides a bin keeps the reference's operand
// order; the file is compiled with -ffp-contract=off so no multiply-add is
// fused.  Only tests/ and the benchmark's CPU-baseline leg load it.
#include "hbt_oracle.h"

#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

namespace {

const double kHbarC = 0.197327053;  // GeV fm (src/parameters.h:4)

struct Hist {
    // 3-D histograms, [slot][iqout][iqside][iqlong]
    std::vector<double> cnt, qo, qs, ql, num, den;
    // sum of |cos(q.dx)| per 3-D bin: the scale of the numerator's rounding
    // (precision comparisons); not part of the reference's output
    std::vector<double> anum;
    // 1-D q_inv histograms, [iKT][iq]
    std::vector<double> qi_sum, qi_num, qi_cnt, qi_den;
    // pair counters per slot (3-D) and per K_T bin (q_inv)
    std::vector<unsigned long long> c_num, c_den, c_num_qi, c_den_qi;
    unsigned long long anomalies = 0;

    void init(int64_t nbins, int n_slots, int n_KT, int qnpts) {
        cnt.assign(nbins, 0.0);
        qo.assign(nbins, 0.0);
        qs.assign(nbins, 0.0);
        ql.assign(nbins, 0.0);
        num.assign(nbins, 0.0);
        den.assign(nbins, 0.0);
        anum.assign(nbins, 0.0);
        qi_sum.assign((int64_t)n_KT * qnpts, 0.0);
        qi_num.assign((int64_t)n_KT * qnpts, 0.0);
        qi_cnt.assign((int64_t)n_KT * qnpts, 0.0);
        qi_den.assign((int64_t)n_KT * qnpts, 0.0);
        c_num.assign(n_slots, 0);
        c_den.assign(n_slots, 0);
        c_num_qi.assign(n_KT, 0);
        c_den_qi.assign(n_KT, 0);
        anomalies = 0;
    }
    void add(const Hist &o) {
        for (size_t i = 0; i < cnt.size(); i++) {
            cnt[i] += o.cnt[i];
            qo[i] += o.qo[i];
            qs[i] += o.qs[i];
            ql[i] += o.ql[i];
            num[i] += o.num[i];
            den[i] += o.den[i];
            anum[i] += o.anum[i];
        }
        for (size_t i = 0; i < qi_sum.size(); i++) {
            qi_sum[i] += o.qi_sum[i];
            qi_num[i] += o.qi_num[i];
            qi_cnt[i] += o.qi_cnt[i];
            qi_den[i] += o.qi_den[i];
        }
        for (size_t i = 0; i < c_num.size(); i++) {
            c_num[i] += o.c_num[i];
            c_den[i] += o.c_den[i];
        }
        for (size_t i = 0; i < c_num_qi.size(); i++) {
            c_num_qi[i] += o.c_num_qi[i];
            c_den_qi[i] += o.c_den_qi[i];
        }
        anomalies += o.anomalies;
    }
};

struct P8 {
    double px, py, pz, E, x, y, z, t;
};

}  // namespace

struct orc_ctx {
    orc_params p;
    // constants derived exactly as HBT_correlation::HBT_correlation
    // (src/HBT_correlation.cpp:25-61)
    double delta_q, dKT, dKphi;
    double q_lo, q_hi, q_base;  // window bounds and bin origin (:342-345)
    double KT_min_sq, KT_max_sq;
    double hbarC_inv;
    unsigned long long cap, cap_qinv;
    int n_slots;
    int64_t q3;
    std::vector<double> KT_array, Kphi_array, q_grid;
    double psi_ref = 0.0;
    Hist h;
    // per-thread partial histograms of the multi-threaded loops, merged into
    // h before anything reads h; pend_* bound the pairs they hold
    std::vector<Hist> part;
    unsigned long long pend_num = 0, pend_den = 0;
    unsigned long long pairs_same = 0, pairs_mixed = 0;
    std::mt19937 gen;
    std::uniform_real_distribution<double> u01{0.0, 1.0};
    std::uniform_int_distribution<int> uint_dist;  // [0, INT_MAX]
};

namespace {

void flush_parts(const orc_ctx *cc) {
    orc_ctx *c = const_cast<orc_ctx *>(cc);
    for (auto &x : c->part) c->h.add(x);
    c->part.clear();
    c->pend_num = c->pend_den = 0;
}

void ensure_parts(orc_ctx *c, int nthreads) {
    if ((int)c->part.size() == nthreads) return;
    flush_parts(c);
    c->part.resize(nthreads);
    for (auto &x : c->part) x.init(c->n_slots * c->q3, c->n_slots, c->p.n_KT, c->p.qnpts);
}

inline int slot_of(const orc_ctx &c, int iK, int iphi) {
    return c.p.azimuthal_flag ? iK * c.p.n_Kphi + iphi : iK;
}

// Azimuthal bin of the pair (src/HBT_correlation.cpp:408-423).  Returns -1
// when the index leaves [0, n_Kphi) (the reference warns and skips).
inline int kphi_bin(const orc_ctx &c, double Kx, double Ky) {
    double phi = atan2(Ky, Kx);
    double d = phi - c.psi_ref;
    while (d < 0.) d += 2. * M_PI;
    while (d > 2. * M_PI) d -= 2. * M_PI;
    int ip = static_cast<int>(d / c.dKphi);
    if (ip < 0 || ip >= c.p.n_Kphi) return -1;
    return ip;
}

// One same-event pair: src/HBT_correlation.cpp:311-458.
inline void same_pair(const orc_ctx &c, Hist &h, const P8 &a, const P8 &b,
                      bool capped) {
    const double K_z = 0.5 * (a.pz + b.pz);
    const double K_E = 0.5 * (a.E + b.E);
    const double K_x = 0.5 * (a.px + b.px);
    const double K_y = 0.5 * (a.py + b.py);
    const double Kp2 = K_x * K_x + K_y * K_y;
    if (Kp2 < c.KT_min_sq || Kp2 > c.KT_max_sq) return;
    const double Kp = sqrt(Kp2);
    const int iK = static_cast<int>((Kp - c.p.KT_min) / c.dKT);
    if (iK < 0 || iK >= c.p.n_KT) {
        h.anomalies++;
        return;
    }
    const double q_x = a.px - b.px;
    const double q_y = a.py - b.py;
    const double q_z = a.pz - b.pz;
    const double q_E = a.E - b.E;
    const double q_inv = sqrt(-(q_E * q_E - q_x * q_x - q_y * q_y - q_z * q_z));
    const double dt = a.t - b.t;
    const double dx = a.x - b.x;
    const double dy = a.y - b.y;
    const double dz = a.z - b.z;

    if (c.p.invariant_radius_flag == 1) {
        if (!capped || h.c_num_qi[iK] < c.cap_qinv) {
            if (q_inv > c.q_lo && q_inv < c.q_hi) {
                const int k = static_cast<int>((q_inv - c.q_base) / c.delta_q);
                h.c_num_qi[iK]++;
                const double w =
                    cos(c.hbarC_inv * (q_E * dt - q_x * dx - q_y * dy - q_z * dz));
                const int64_t at = (int64_t)iK * c.p.qnpts + k;
                h.qi_cnt[at]++;
                h.qi_sum[at] += q_inv;
                h.qi_num[at] += w;
            }
        }
    }

    const double cphi = K_x / Kp;
    const double sphi = K_y / Kp;
    const double q_o = q_x * cphi + q_y * sphi;
    if (q_o != q_o) {
        h.anomalies++;
        return;
    }
    if (q_o < c.q_lo || q_o > c.q_hi) return;
    const int io = static_cast<int>((q_o - c.q_base) / c.delta_q);
    if (io >= c.p.qnpts) return;

    const double q_s = q_y * cphi - q_x * sphi;
    if (q_s != q_s) {
        h.anomalies++;
        return;
    }
    if (q_s < c.q_lo || q_s > c.q_hi) return;
    const int is = static_cast<int>((q_s - c.q_base) / c.delta_q);
    if (is >= c.p.qnpts) return;

    double q_l = q_z;
    if (c.p.long_comoving_boost) {
        const double Mt = sqrt(K_E * K_E - K_z * K_z);
        const double gamma = K_E / Mt;
        const double beta = K_z / K_E;
        q_l = gamma * (q_z - beta * q_E);
    }
    if (q_l != q_l) {
        h.anomalies++;
        return;
    }
    if (q_l < c.q_lo || q_l > c.q_hi) return;
    const int il = static_cast<int>((q_l - c.q_base) / c.delta_q);
    if (il >= c.p.qnpts) return;

    int iphi = 0;
    if (c.p.azimuthal_flag) {
        iphi = kphi_bin(c, K_x, K_y);
        if (iphi < 0) return;
    }
    const int s = slot_of(c, iK, iphi);
    if (capped && h.c_num[s] > c.cap) return;
    h.c_num[s]++;

    const double w = cos(c.hbarC_inv * (q_E * dt - q_x * dx - q_y * dy - q_z * dz));
    const int64_t at = s * c.q3 + ((int64_t)io * c.p.qnpts + is) * c.p.qnpts + il;
    h.cnt[at]++;
    h.qo[at] += q_o;
    h.qs[at] += q_s;
    h.ql[at] += q_l;
    h.num[at] += w;
    h.anum[at] += fabs(w);
}

// One mixed-event pair: src/HBT_correlation.cpp:574-687.  Note the
// inclusive (>=) upper window bounds and the q_inv index check.
inline void mixed_pair(const orc_ctx &c, Hist &h, const double *a,
                       const double *b, bool capped) {
    // a, b: {px, py, pz, E}
    const double K_z = 0.5 * (a[2] + b[2]);
    const double K_E = 0.5 * (a[3] + b[3]);
    const double K_x = 0.5 * (a[0] + b[0]);
    const double K_y = 0.5 * (a[1] + b[1]);
    const double Kp2 = K_x * K_x + K_y * K_y;
    if (Kp2 < c.KT_min_sq || Kp2 > c.KT_max_sq) return;
    const double Kp = sqrt(Kp2);
    const int iK = static_cast<int>((Kp - c.p.KT_min) / c.dKT);
    if (iK < 0 || iK >= c.p.n_KT) {
        h.anomalies++;
        return;
    }
    const double q_z = a[2] - b[2];
    const double q_E = a[3] - b[3];
    const double q_x = a[0] - b[0];
    const double q_y = a[1] - b[1];
    const double q_inv = sqrt(-(q_E * q_E - q_x * q_x - q_y * q_y - q_z * q_z));

    if (c.p.invariant_radius_flag == 1) {
        if (q_inv > c.q_lo && q_inv < c.q_hi) {
            const int k = static_cast<int>((q_inv - c.q_base) / c.delta_q);
            if (k < c.p.qnpts && (!capped || h.c_den_qi[iK] < c.cap_qinv)) {
                h.c_den_qi[iK]++;
                h.qi_den[(int64_t)iK * c.p.qnpts + k] += 1.0;
            }
        }
    }

    const double cphi = K_x / Kp;
    const double sphi = K_y / Kp;
    const double q_o = q_x * cphi + q_y * sphi;
    if (q_o != q_o) {
        h.anomalies++;
        return;
    }
    if (q_o < c.q_lo || q_o >= c.q_hi) return;
    const int io = static_cast<int>((q_o - c.q_base) / c.delta_q);
    if (io >= c.p.qnpts) return;
    const double q_s = q_y * cphi - q_x * sphi;
    if (q_s != q_s) {
        h.anomalies++;
        return;
    }
    if (q_s < c.q_lo || q_s >= c.q_hi) return;
    const int is = static_cast<int>((q_s - c.q_base) / c.delta_q);
    if (is >= c.p.qnpts) return;
    double q_l = q_z;
    if (c.p.long_comoving_boost) {
        const double Mt = sqrt(K_E * K_E - K_z * K_z);
        const double gamma = K_E / Mt;
        const double beta = K_z / K_E;
        q_l = gamma * (q_z - beta * q_E);
    }
    if (q_l != q_l) {
        h.anomalies++;
        return;
    }
    if (q_l < c.q_lo || q_l >= c.q_hi) return;
    const int il = static_cast<int>((q_l - c.q_base) / c.delta_q);
    if (il >= c.p.qnpts) return;

    int iphi = 0;
    if (c.p.azimuthal_flag) {
        iphi = kphi_bin(c, K_x, K_y);
        if (iphi < 0) return;
    }
    const int s = slot_of(c, iK, iphi);
    if (capped && h.c_den[s] > c.cap) return;
    h.c_den[s]++;
    h.den[s * c.q3 + ((int64_t)io * c.p.qnpts + is) * c.p.qnpts + il] += 1.0;
}

inline P8 load8(const double *const *cols, int64_t i) {
    return P8{cols[0][i], cols[1][i], cols[2][i], cols[3][i],
              cols[4][i], cols[5][i], cols[6][i], cols[7][i]};
}

void same_rows(const orc_ctx &c, Hist &h, int64_t n, const double *const *cols,
               int64_t first, int64_t stride, bool capped) {
    for (int64_t i = first; i < n; i += stride) {
        const P8 a = load8(cols, i);
        for (int64_t j = i + 1; j < n; j++) same_pair(c, h, a, load8(cols, j), capped);
    }
}

void mixed_rows(const orc_ctx &c, Hist &h, int64_t n1, const double *const *l1,
                int64_t n2, const double *const *l2, int64_t first,
                int64_t stride, bool capped) {
    for (int64_t i = first; i < n1; i += stride) {
        const double a[4] = {l1[0][i], l1[1][i], l1[2][i], l1[3][i]};
        for (int64_t j = 0; j < n2; j++) {
            const double b[4] = {l2[0][j], l2[1][j], l2[2][j], l2[3][j]};
            mixed_pair(c, h, a, b, capped);
        }
    }
}

// True when no cap check can reject any of `pairs` more pairs.
bool caps_cannot_bind(const orc_ctx &c, const std::vector<unsigned long long> &ctr,
                      const std::vector<unsigned long long> &ctr_qi,
                      unsigned long long pairs) {
    for (unsigned long long v : ctr)
        if (v + pairs > c.cap) return false;
    if (c.p.invariant_radius_flag == 1)
        for (unsigned long long v : ctr_qi)
            if (v + pairs >= c.cap_qinv) return false;
    return true;
}

void gather(const double *const *cols, const int64_t *off, int ev, double ycut_min,
            double ycut_max, std::vector<double> (&out)[8]) {
    for (int64_t k = off[ev]; k < off[ev + 1]; k++) {
        const double E = cols[3][k];
        const double pz = cols[2][k];
        const double ratio = pz / E;
        if (ratio > ycut_min && ratio < ycut_max)
            for (int f = 0; f < 8; f++) out[f].push_back(cols[f][k]);
    }
}

}  // namespace

extern "C" {

orc_ctx *orc_create(const orc_params *p) {
    orc_ctx *c = new orc_ctx();
    c->p = *p;
    c->delta_q = (p->q_max - p->q_min) / (p->qnpts - 1);
    for (int i = 0; i < p->qnpts; i++) c->q_grid.push_back(p->q_min + i * c->delta_q);
    c->q_lo = p->q_min - c->delta_q / 2. + 1e-8;
    c->q_hi = p->q_max + c->delta_q / 2. - 1e-8;
    c->q_base = p->q_min - c->delta_q / 2.;
    c->dKT = (p->KT_max - p->KT_min) / (p->n_KT - 1);
    c->dKphi = 2 * M_PI / p->n_Kphi;
    for (int i = 0; i < p->n_KT; i++) c->KT_array.push_back(p->KT_min + i * c->dKT);
    for (int i = 0; i < p->n_Kphi; i++) c->Kphi_array.push_back(i * c->dKphi);
    c->KT_min_sq = p->KT_min * p->KT_min;
    c->KT_max_sq = p->KT_max * p->KT_max;
    c->hbarC_inv = 1. / kHbarC;
    c->cap = static_cast<unsigned long long>(p->needed_number_of_pairs);
    c->cap_qinv = 50 * c->cap;
    c->n_slots = p->azimuthal_flag ? p->n_KT * p->n_Kphi : p->n_KT;
    c->q3 = (int64_t)p->qnpts * p->qnpts * p->qnpts;
    c->h.init(c->n_slots * c->q3, c->n_slots, p->n_KT, p->qnpts);
    c->gen.seed(static_cast<std::mt19937::result_type>(p->seed));
    return c;
}

void orc_destroy(orc_ctx *c) { delete c; }

void orc_rapidity_shift(int64_t n, double *E, double *pz, double shift) {
    for (int64_t i = 0; i < n; i++) {
        const double e = E[i] * cosh(shift) + pz[i] * sinh(shift);
        const double z = pz[i] * cosh(shift) + E[i] * sinh(shift);
        E[i] = e;
        pz[i] = z;
    }
}

void orc_set_psi_ref(orc_ctx *c, double psi) { c->psi_ref = psi; }
double orc_get_psi_ref(const orc_ctx *c) { return c->psi_ref; }

double orc_event_plane_angle(int64_t n, const double *px, const double *py,
                             int32_t n_order) {
    double re = 0.0, im = 0.0;
    for (int64_t i = 0; i < n; i++) {
        const double phi = atan2(py[i], px[i]);
        re += cos(n_order * phi);
        im += sin(n_order * phi);
    }
    return atan2(im, re) / n_order;
}

void orc_bin_same(orc_ctx *c, int64_t n, const double *const *cols8) {
    flush_parts(c);
    c->pairs_same += (unsigned long long)(n * (n - 1) / 2);
    same_rows(*c, c->h, n, cols8, 0, 1, true);
}

void orc_bin_mixed(orc_ctx *c, int64_t n1, const double *const *l1, int64_t n2,
                   const double *const *l2) {
    flush_parts(c);
    c->pairs_mixed += (unsigned long long)(n1 * n2);
    mixed_rows(*c, c->h, n1, l1, n2, l2, 0, 1, true);
}

void orc_bin_same_mt(orc_ctx *c, int64_t n, const double *const *cols8,
                     int32_t nthreads) {
    const unsigned long long pairs = (unsigned long long)(n * (n - 1) / 2);
    if (nthreads <= 1 ||
        !caps_cannot_bind(*c, c->h.c_num, c->h.c_num_qi, pairs + c->pend_num)) {
        flush_parts(c);
        orc_bin_same(c, n, cols8);
        return;
    }
    ensure_parts(c, nthreads);
    c->pairs_same += pairs;
    c->pend_num += pairs;
    std::vector<std::thread> th;
    for (int t = 0; t < nthreads; t++)
        th.emplace_back([&, t] { same_rows(*c, c->part[t], n, cols8, t, nthreads, false); });
    for (auto &x : th) x.join();
}

void orc_bin_mixed_mt(orc_ctx *c, int64_t n1, const double *const *l1, int64_t n2,
                      const double *const *l2, int32_t nthreads) {
    const unsigned long long pairs = (unsigned long long)(n1 * n2);
    if (nthreads <= 1 ||
        !caps_cannot_bind(*c, c->h.c_den, c->h.c_den_qi, pairs + c->pend_den)) {
        flush_parts(c);
        orc_bin_mixed(c, n1, l1, n2, l2);
        return;
    }
    ensure_parts(c, nthreads);
    c->pairs_mixed += pairs;
    c->pend_den += pairs;
    std::vector<std::thread> th;
    for (int t = 0; t < nthreads; t++)
        th.emplace_back(
            [&, t] { mixed_rows(*c, c->part[t], n1, l1, n2, l2, t, nthreads, false); });
    for (auto &x : th) x.join();
}

void orc_process_buffer(orc_ctx *c, int32_t nev, const int64_t *off,
                        const double *const *cols, int32_t mixed_nev,
                        const int64_t *moff, const double *const *mcols) {
    const double ycut_max = tanh(c->p.HBTrap_max);
    const double ycut_min = tanh(c->p.HBTrap_min);
    if (c->p.azimuthal_flag == 1) {
        // psi_ref from every particle of the buffer (:181-183, :233-249)
        c->psi_ref = orc_event_plane_angle(off[nev], cols[0], cols[1], 2);
    }
    // same-event pairs over the concatenated buffer (:190-194, :251-290)
    {
        std::vector<double> g[8];
        for (int e = 0; e < nev; e++) gather(cols, off, e, ycut_min, ycut_max, g);
        const double *gp[8];
        for (int f = 0; f < 8; f++) gp[f] = g[f].data();
        orc_bin_same(c, (int64_t)g[0].size(), gp);
    }
    // mixed-event pairs (:197-217, :464-558)
    const int nmix = c->p.number_of_mixed_events > 0 ? c->p.number_of_mixed_events
                                                     : mixed_nev / 2 + 1;
    for (int iev = 0; iev < nev; iev++) {
        std::vector<int> partners(nmix, 0);
        for (int k = 0; k < nmix; k++) {
            int id = c->uint_dist(c->gen) % mixed_nev;
            while (iev == id && mixed_nev != 1) id = c->uint_dist(c->gen) % mixed_nev;
            partners[k] = id;
        }
        std::vector<double> l1[8], l2[4];
        gather(cols, off, iev, ycut_min, ycut_max, l1);
        for (int k = 0; k < nmix; k++) {
            const double rot = c->u01(c->gen) * 2 * M_PI;
            const double cr = cos(rot);
            const double sr = sin(rot);
            const int m = partners[k];
            for (int64_t q = moff[m]; q < moff[m + 1]; q++) {
                const double E = mcols[3][q];
                const double pz = mcols[2][q];
                const double ratio = pz / E;
                if (ratio > ycut_min && ratio < ycut_max) {
                    const double px = mcols[0][q];
                    const double py = mcols[1][q];
                    l2[0].push_back(px * cr - py * sr);
                    l2[1].push_back(px * sr + py * cr);
                    l2[2].push_back(pz);
                    l2[3].push_back(E);
                }
            }
        }
        const double *a[4] = {l1[0].data(), l1[1].data(), l1[2].data(), l1[3].data()};
        const double *b[4] = {l2[0].data(), l2[1].data(), l2[2].data(), l2[3].data()};
        orc_bin_mixed(c, (int64_t)l1[0].size(), a, (int64_t)l2[0].size(), b);
    }
}

int32_t orc_mixed_partners(const orc_ctx *c, int32_t mixed_nev) {
    return c->p.number_of_mixed_events > 0 ? c->p.number_of_mixed_events : mixed_nev / 2 + 1;
}

int32_t orc_mixed_plan(orc_ctx *c, int32_t nev, int32_t mixed_nev, int32_t *partners,
                       double *angles) {
    // the draws of orc_process_buffer's mixed-event loop, in its order: per
    // event the partner ids (:197-205), then one angle per partner (:495)
    const int nmix = orc_mixed_partners(c, mixed_nev);
    for (int iev = 0; iev < nev; iev++) {
        for (int k = 0; k < nmix; k++) {
            int id = c->uint_dist(c->gen) % mixed_nev;
            while (iev == id && mixed_nev != 1) id = c->uint_dist(c->gen) % mixed_nev;
            partners[(int64_t)iev * nmix + k] = id;
        }
        for (int k = 0; k < nmix; k++) angles[(int64_t)iev * nmix + k] = c->u01(c->gen) * 2 * M_PI;
    }
    return nmix;
}

int64_t orc_n_bins(const orc_ctx *c) { return c->n_slots * c->q3; }

void orc_get_hist(const orc_ctx *c, double *num_count, double *q_out_sum,
                  double *q_side_sum, double *q_long_sum, double *num, double *den) {
    flush_parts(c);
    const size_t n = c->h.cnt.size() * sizeof(double);
    if (num_count) memcpy(num_count, c->h.cnt.data(), n);
    if (q_out_sum) memcpy(q_out_sum, c->h.qo.data(), n);
    if (q_side_sum) memcpy(q_side_sum, c->h.qs.data(), n);
    if (q_long_sum) memcpy(q_long_sum, c->h.ql.data(), n);
    if (num) memcpy(num, c->h.num.data(), n);
    if (den) memcpy(den, c->h.den.data(), n);
}

void orc_get_abs_num(const orc_ctx *c, double *abs_num) {
    flush_parts(c);
    memcpy(abs_num, c->h.anum.data(), c->h.anum.size() * sizeof(double));
}

void orc_get_qinv(const orc_ctx *c, double *qinv_sum, double *num, double *num_count,
                  double *den) {
    flush_parts(c);
    const size_t n = c->h.qi_sum.size() * sizeof(double);
    if (qinv_sum) memcpy(qinv_sum, c->h.qi_sum.data(), n);
    if (num) memcpy(num, c->h.qi_num.data(), n);
    if (num_count) memcpy(num_count, c->h.qi_cnt.data(), n);
    if (den) memcpy(den, c->h.qi_den.data(), n);
}

void orc_get_counters(const orc_ctx *c, uint64_t *num, uint64_t *den,
                      uint64_t *num_qinv, uint64_t *den_qinv) {
    flush_parts(c);
    for (int s = 0; s < c->n_slots; s++) {
        if (num) num[s] = c->h.c_num[s];
        if (den) den[s] = c->h.c_den[s];
    }
    for (int k = 0; k < c->p.n_KT; k++) {
        if (num_qinv) num_qinv[k] = c->h.c_num_qi[k];
        if (den_qinv) den_qinv[k] = c->h.c_den_qi[k];
    }
}

uint64_t orc_anomalies(const orc_ctx *c) {
    flush_parts(c);
    return c->h.anomalies;
}
uint64_t orc_pairs_same(const orc_ctx *c) { return c->pairs_same; }
uint64_t orc_pairs_mixed(const orc_ctx *c) { return c->pairs_mixed; }

namespace {

void put_row(FILE *f, bool eco, double a, double b, double c3, double num,
             double den) {
    if (eco)
        fprintf(f, "%18.8e    %.8e\n", num, den);
    else
        fprintf(f, "%18.8e    %.8e    %.8e    %.8e    %.8e\n", a, b, c3, num, den);
}

// One 3-D correlation file: src/HBT_correlation.cpp:735-780 (and the
// K_phi variant :798-851).
void write_3d(const orc_ctx &c, FILE *f, int slot, double ratio, bool eco) {
    const int n = c.p.qnpts;
    for (int il = 0; il < n; il++)
        for (int io = 0; io < n; io++)
            for (int is = 0; is < n; is++) {
                const int64_t at = slot * c.q3 + ((int64_t)io * n + is) * n + il;
                const int npart_num = static_cast<int>(c.h.cnt[at]);
                const int npart_den = static_cast<int>(c.h.den[at]);
                if (npart_num < 2 || npart_den < 2) {
                    put_row(f, eco, c.q_grid[io], c.q_grid[is], c.q_grid[il], 0.0,
                            static_cast<double>(npart_den));
                } else {
                    put_row(f, eco, c.h.qo[at] / npart_num, c.h.qs[at] / npart_num,
                            c.h.ql[at] / npart_num, c.h.num[at], ratio * c.h.den[at]);
                }
            }
}

}  // namespace

int orc_write(const orc_ctx *c, const char *path, int32_t eco_output) {
    flush_parts(c);
    const bool eco = eco_output == 1;
    if (c->p.invariant_radius_flag == 1) {
        for (int iK = 0; iK < c->p.n_KT - 1; iK++) {
            const double ratio = static_cast<double>(c->h.c_num_qi[iK]) /
                                 static_cast<double>(c->h.c_den_qi[iK]);
            std::ostringstream fn;
            fn << path << "/HBT_correlation_function_inv_KT_" << c->KT_array[iK] << "_"
               << c->KT_array[iK + 1] << ".dat";
            FILE *f = fopen(fn.str().c_str(), "w");
            if (!f) return -1;
            for (int k = 0; k < c->p.qnpts; k++) {
                const int64_t at = (int64_t)iK * c->p.qnpts + k;
                const double qmean = c->h.qi_sum[at] / c->h.qi_cnt[at];
                const double den = c->h.qi_den[at] * ratio;
                if (eco)
                    fprintf(f, "%18.8e    %.8e\n", c->h.qi_num[at], den);
                else
                    fprintf(f, "%18.8e    %.8e    %.8e\n", qmean, c->h.qi_num[at], den);
            }
            fclose(f);
        }
    }
    for (int iK = 0; iK < c->p.n_KT - 1; iK++) {
        const int nphi = c->p.azimuthal_flag ? c->p.n_Kphi : 1;
        for (int ip = 0; ip < nphi; ip++) {
            const int s = slot_of(*c, iK, ip);
            const double ratio = static_cast<double>(c->h.c_num[s]) /
                                 static_cast<double>(c->h.c_den[s]);
            std::ostringstream fn;
            fn << path << "/HBT_correlation_function_KT_" << c->KT_array[iK] << "_"
               << c->KT_array[iK + 1];
            if (c->p.azimuthal_flag) fn << "_Kphi_" << c->Kphi_array[ip];
            fn << ".dat";
            FILE *f = fopen(fn.str().c_str(), "w");
            if (!f) return -1;
            write_3d(*c, f, s, ratio, eco);
            fclose(f);
        }
    }
    return 0;
}

}  // extern "C"
