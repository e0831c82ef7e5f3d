// Balance-function oracle (bf_oracle.h) - test infrastructure only.
//
// Restates src/BalanceFunction.cpp of the reference: four same-event and
// four mixed-event pair histograms over (Delta y, Delta phi), then the
// three output files.  Built with -ffp-contract=off like the reference.
#include "bf_oracle.h"

#include <climits>
#include <cmath>
#include <fstream>
#include <iomanip>
#include <random>
#include <sstream>
#include <string>
#include <vector>

namespace {

const int kBnphi = 20;

struct Particle {
    double pT, phi, y, eta;
};

typedef std::vector<std::vector<Particle>> Events;

}  // namespace

struct orc_bf {
    orc_bf_params p;
    double drap, Brap_min, dphi, Bphi_min;
    std::vector<double> hist[8];  // [Bnpts][Bnphi] each
    long long N_b = 0, N_bbar = 0;
    std::mt19937 gen;
    std::uniform_real_distribution<double> u01{0.0, 1.0};
    std::uniform_int_distribution<int> uint_{0, INT_MAX};
};

extern "C" {

orc_bf *orc_bf_create(const orc_bf_params *p) {
    orc_bf *c = new orc_bf();
    c->p = *p;
    // BalanceFunction::BalanceFunction (src/BalanceFunction.cpp:14-57)
    c->drap = 2. * std::abs(p->Brap_max) / (p->Bnpts - 1);
    c->Brap_min = -std::abs(p->Brap_max) - 0.5 * c->drap;
    c->dphi = 2. * M_PI / kBnphi;
    c->Bphi_min = -M_PI / 2.;
    for (auto &h : c->hist) h.assign((size_t)p->Bnpts * kBnphi, 0.0);
    c->gen.seed(static_cast<std::mt19937::result_type>(p->seed));
    return c;
}

void orc_bf_destroy(orc_bf *c) { delete c; }

void orc_bf_boost(int64_t n, const double *mass, const double *px, const double *py,
                  const double *pz, const double *E, double rap_shift, double *pT, double *phi,
                  double *rap_y, double *rap_eta) {
    for (int64_t k = 0; k < n; k++) {
        const double pt = sqrt(px[k] * px[k] + py[k] * py[k]);
        const double mT = sqrt(pt * pt + mass[k] * mass[k]);
        const double pz_s = pz[k] * cosh(rap_shift) + E[k] * sinh(rap_shift);
        pT[k] = pt;
        phi[k] = atan2(py[k], px[k]);
        rap_y[k] = asinh(pz_s / mT);
        rap_eta[k] = asinh(pz_s / pt);
    }
}

// combine_and_bin_particle_pairs / combine_and_bin_mixed_particle_pairs
// (src/BalanceFunction.cpp:124-208): the pair loop of one event pair.
void orc_bf_bin(orc_bf *c, int32_t which, int64_t na, const double *pTa, const double *phia,
                const double *ya, int64_t nb, const double *pTb, const double *phib,
                const double *yb, int32_t mixed, double rotation) {
    std::vector<double> &h = c->hist[which];
    const orc_bf_params &p = c->p;
    for (int64_t i = 0; i < na; i++) {
        if (pTa[i] < p.BpT_min || pTa[i] > p.BpT_max) continue;
        for (int64_t j = 0; j < nb; j++) {
            if (pTb[j] < p.BpT_min || pTb[j] > p.BpT_max) continue;
            const double dphi_local = mixed ? (phia[i] - phib[j] + rotation) : phia[i] - phib[j];
            int phi_idx = (static_cast<int>(floor((dphi_local - c->Bphi_min) / c->dphi))) % kBnphi;
            if (phi_idx < 0) phi_idx += kBnphi;
            const double dy = ya[i] - yb[j];
            if (std::abs(dy) < 1e-10) continue;
            if (dy < c->Brap_min) continue;
            const int y_idx = static_cast<int>((dy - c->Brap_min) / c->drap);
            if (y_idx >= 0 && y_idx < p.Bnpts) h[(size_t)y_idx * kBnphi + phi_idx] += 1.;
        }
    }
}

void orc_bf_process_buffer(orc_bf *c, int32_t nev, const int64_t *off, const int32_t *monval,
                           const double *pT, const double *phi, const double *y,
                           const double *eta, int32_t mnev, const int64_t *moff,
                           const int32_t *mmonval, const double *mpT, const double *mphi,
                           const double *my, const double *meta) {
    const orc_bf_params &p = c->p;
    const int mon[4] = {p.particle_alpha, -p.particle_alpha, p.particle_beta, -p.particle_beta};
    // the species lists a, abar, b, bbar of each event (filter_particles)
    auto lists = [&](int32_t n, const int64_t *o, const int32_t *m, const double *pt,
                     const double *ph, const double *yy, const double *ee) {
        std::vector<Events> L(4, Events(n));
        for (int e = 0; e < n; e++)
            for (int64_t k = o[e]; k < o[e + 1]; k++)
                for (int s = 0; s < 4; s++)
                    if (m[k] == mon[s]) L[s][e].push_back(Particle{pt[k], ph[k], yy[k], ee[k]});
        return L;
    };
    const std::vector<Events> S = lists(nev, off, monval, pT, phi, y, eta);
    const std::vector<Events> M = lists(mnev, moff, mmonval, mpT, mphi, my, meta);
    auto count = [&](const Events &ev) {
        long long n = 0;
        for (const auto &e : ev)
            for (const auto &q : e)
                if (!(q.pT < p.BpT_min || q.pT > p.BpT_max)) n++;
        return n;
    };
    c->N_b += count(S[2]);
    c->N_bbar += count(S[3]);
    auto cols = [&](const std::vector<Particle> &v, std::vector<double> &a, std::vector<double> &b,
                    std::vector<double> &r) {
        a.clear();
        b.clear();
        r.clear();
        for (const auto &q : v) {
            a.push_back(q.pT);
            b.push_back(q.phi);
            r.push_back(p.rap_type == 0 ? q.eta : q.y);
        }
    };
    std::vector<double> a0, a1, a2, b0, b1, b2;
    // same-event histograms: (a, b), (abar, bbar), (a, bbar), (abar, b)
    const int pairs_of[4][2] = {{0, 2}, {1, 3}, {0, 3}, {1, 2}};
    for (int hgt = 0; hgt < 4; hgt++)
        for (int e = 0; e < nev; e++) {
            cols(S[pairs_of[hgt][0]][e], a0, a1, a2);
            cols(S[pairs_of[hgt][1]][e], b0, b1, b2);
            orc_bf_bin(c, hgt, (int64_t)a0.size(), a0.data(), a1.data(), a2.data(),
                       (int64_t)b0.size(), b0.data(), b1.data(), b2.data(), 0, 0.0);
        }
    // mixed-event histograms: each event against a drawn pool event, with
    // a drawn global rotation
    for (int hgt = 0; hgt < 4; hgt++)
        for (int e = 0; e < nev; e++) {
            const int m = c->uint_(c->gen) % mnev;
            const double rot = c->u01(c->gen) * 2. * M_PI;
            cols(S[pairs_of[hgt][0]][e], a0, a1, a2);
            cols(M[pairs_of[hgt][1]][m], b0, b1, b2);
            orc_bf_bin(c, 4 + hgt, (int64_t)a0.size(), a0.data(), a1.data(), a2.data(),
                       (int64_t)b0.size(), b0.data(), b1.data(), b2.data(), 1, rot);
        }
}

void orc_bf_get_hist(const orc_bf *c, int32_t which, double *out) {
    const std::vector<double> &h = c->hist[which];
    for (size_t k = 0; k < h.size(); k++) out[k] = h[k];
}

void orc_bf_get_norm(const orc_bf *c, int64_t *N_b, int64_t *N_bbar) {
    if (N_b) *N_b = c->N_b;
    if (N_bbar) *N_bbar = c->N_bbar;
}

// output_balance_function (src/BalanceFunction.cpp:211-319).
int orc_bf_write(const orc_bf *c, const char *path) {
    const int n = c->p.Bnpts;
    auto H = [&](int w, int i, int j) { return c->hist[w][(size_t)i * kBnphi + j]; };
    std::vector<double> os_y(n, 0.), ss_y(n, 0.), os_y_m(n, 0.), ss_y_m(n, 0.);
    double N_OS = 0., N_SS = 0., N_OS_m = 0., N_SS_m = 0.;
    for (int i = 0; i < n; i++) {
        for (int j = 0; j < kBnphi; j++) {
            os_y[i] += H(0, i, j) + H(1, i, j);
            ss_y[i] += H(2, i, j) + H(3, i, j);
            os_y_m[i] += H(4, i, j) + H(5, i, j);
            ss_y_m[i] += H(6, i, j) + H(7, i, j);
        }
        N_OS += os_y[i];
        N_SS += ss_y[i];
        N_OS_m += os_y_m[i];
        N_SS_m += ss_y_m[i];
    }
    std::vector<double> os_p(kBnphi, 0.), ss_p(kBnphi, 0.), os_p_m(kBnphi, 0.), ss_p_m(kBnphi, 0.);
    for (int j = 0; j < kBnphi; j++)
        for (int i = 0; i < n; i++) {
            os_p[j] += H(0, i, j) + H(1, i, j);
            ss_p[j] += H(2, i, j) + H(3, i, j);
            os_p_m[j] += H(4, i, j) + H(5, i, j);
            ss_p_m[j] += H(6, i, j) + H(7, i, j);
        }
    std::vector<double> dy(n), dphi(kBnphi);
    for (int i = 0; i < n; i++) dy[i] = c->Brap_min + (i + 0.5) * c->drap;
    for (int j = 0; j < kBnphi; j++) dphi[j] = c->Bphi_min + (j + 0.5) * c->dphi;
    const std::string base = std::string(path) + "/";
    std::ostringstream tag;
    tag << c->p.particle_alpha << "_" << c->p.particle_beta;
    {
        std::ofstream f((base + "Balance_function_" + tag.str() + "_Delta_y.dat").c_str());
        if (!f) return -1;
        f << "# DeltaY  Delta_C2  C2(OS)  rho2(OS)  rho1^2(OS)  "
          << "C2(SS) rho2(SS)  rho1^2(SS)" << std::endl;
        for (int i = 0; i < n; i++) {
            const double os = os_y[i] / os_y_m[i] * N_OS_m / N_OS;
            const double ss = ss_y[i] / ss_y_m[i] * N_SS_m / N_SS;
            f << std::scientific << std::setw(18) << std::setprecision(8) << dy[i] << "   "
              << os - ss << "  " << os << "  " << os_y[i] << "  " << os_y_m[i] << "  " << ss
              << "  " << ss_y[i] << "  " << ss_y_m[i] << std::endl;
        }
    }
    {
        std::ofstream f((base + "Balance_function_" + tag.str() + "_Delta_phi.dat").c_str());
        if (!f) return -1;
        f << "# Delta_phi  Delta_C2  C2(OS)  rho2(OS)  rho1^2(OS)  "
          << "C2(SS) rho2(SS)  rho1^2(SS)" << std::endl;
        for (int j = 0; j < kBnphi; j++) {
            const double os = (os_p[j] / os_p_m[j] * N_OS_m / N_OS);
            const double ss = (ss_p[j] / ss_p_m[j] * N_SS_m / N_SS);
            f << std::scientific << std::setw(18) << std::setprecision(8) << dphi[j] << "   "
              << os - ss << "  " << os << "  " << os_p[j] << "  " << os_p_m[j] << "  " << ss
              << "  " << ss_p[j] << "  " << ss_p_m[j] << std::endl;
        }
    }
    {
        std::ofstream f((base + "Correlation_function_" + tag.str() + "_2D.dat").c_str());
        if (!f) return -1;
        f << "# DY  Dphi  C2(OS)  rho2(OS)  rho1^2(OS)  "
          << "C2(SS)  rho2(SS)  rho1^2(SS)" << std::endl;
        for (int i = 0; i < n; i++)
            for (int j = 0; j < kBnphi; j++) {
                const double os = ((H(0, i, j) + H(1, i, j)) / (H(4, i, j) + H(5, i, j) + 1e-15));
                const double ss = ((H(2, i, j) + H(3, i, j)) / (H(6, i, j) + H(7, i, j) + 1e-15));
                f << std::scientific << std::setw(18) << std::setprecision(8) << dy[i] << "  "
                  << dphi[j] << "  " << os * N_OS_m / N_OS << "  " << H(0, i, j) + H(1, i, j)
                  << "  " << H(4, i, j) + H(5, i, j) << "  " << ss * N_SS_m / N_SS << "  "
                  << H(2, i, j) + H(3, i, j) << "  " << H(6, i, j) + H(7, i, j) << std::endl;
            }
    }
    return 0;
}

}  // extern "C"
