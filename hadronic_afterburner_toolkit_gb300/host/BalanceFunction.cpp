#include "BalanceFunction.h"

#include <charconv>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <stdexcept>

BalanceFunction::BalanceFunction(const ParameterReader &paraRdr, const std::string path,
                                 std::shared_ptr<RandomUtil::Random> ran_gen)
    : paraRdr_(paraRdr), path_(path), ran_gen_ptr(ran_gen) {
    // src/BalanceFunction.cpp:14-57
    particle_monval_a = static_cast<int>(paraRdr_.getVal("particle_alpha"));
    particle_monval_b = static_cast<int>(paraRdr_.getVal("particle_beta"));
    BpT_min = paraRdr_.getVal("BpT_min");
    BpT_max = paraRdr_.getVal("BpT_max");
    Bnpts = static_cast<int>(paraRdr_.getVal("Bnpts"));
    Brap_max = paraRdr_.getVal("Brap_max");
    drap = 2. * std::abs(Brap_max) / (Bnpts - 1);
    Brap_min = -std::abs(Brap_max) - 0.5 * drap;
    dphi = 2. * M_PI / HBT_BF_NPHI;
    Bphi_min = -M_PI / 2.;
    rap_type_ = static_cast<int>(paraRdr_.getVal("rap_type"));
    const int device =
        paraRdr_.exist("hbt_device") ? static_cast<int>(paraRdr_.getVal("hbt_device")) : 0;
    const hbt_bf_params p = {Bnpts, Brap_max};
    check(hbt_bf_create(&p, device, &ctx_), "hbt_bf_create");
}

BalanceFunction::~BalanceFunction() { hbt_bf_destroy(ctx_); }

void BalanceFunction::check(hbt_status s, const char *what) {
    if (s != HBT_OK)
        throw std::runtime_error(std::string("BalanceFunction: ") + what + ": " +
                                 (ctx_ ? hbt_bf_last_error(ctx_) : "engine not created"));
}

namespace {

// A species list of the buffer as the engine takes it: per event the
// particles inside the pT window (the reference skips the others in both
// pair loops, src/BalanceFunction.cpp:130-133), their phi_p and rapidity
// variable.
struct List {
    std::vector<int64_t> off;
    std::vector<double> phi, y;
    long counted = 0;
};

List make_list(const hbt::EventList &events, double pt_min, double pt_max, bool eta) {
    List L;
    L.off.push_back(0);
    for (const auto &ev : events) {
        for (const particle_info &p : ev) {
            if (p.pT < pt_min || p.pT > pt_max) continue;
            L.phi.push_back(p.phi_p);
            L.y.push_back(eta ? p.rap_eta : p.rap_y);
        }
        L.off.push_back(static_cast<int64_t>(L.phi.size()));
    }
    L.counted = static_cast<long>(L.phi.size());
    return L;
}

}  // namespace

void BalanceFunction::calculate_balance_function(
    std::shared_ptr<particleSamples> particle_list_in) {
    set_particle_list(particle_list_in);
    const bool eta = rap_type_ == 0;
    std::vector<List> lists;
    for (int s = 0; s < 4; s++)
        lists.push_back(make_list(particle_list->balance_function_list(s), BpT_min, BpT_max, eta));
    for (int s = 0; s < 4; s++)
        lists.push_back(make_list(particle_list->balance_function_list_mixed_event(s), BpT_min,
                                  BpT_max, eta));
    // get_number_of_particles (:210-220) of the b and bbar lists
    N_b += lists[2].counted;
    N_bbar += lists[3].counted;

    const int nev = particle_list->get_number_of_events();
    const int nev_mixed = static_cast<int>(particle_list->balance_function_list_mixed_event(2).size());
    // (a, b) list pairs of C_ab, C_abarbbar, C_abbar, C_abarb
    const int pairs_of[4][2] = {{0, 2}, {1, 3}, {0, 3}, {1, 2}};
    std::vector<hbt_bf_job> jobs;
    for (int h = 0; h < 4; h++)
        for (int e = 0; e < nev; e++)
            jobs.push_back(hbt_bf_job{h, pairs_of[h][0], e, pairs_of[h][1], e, 0, 0.0});
    // combine_and_bin_mixed_particle_pairs (:163-208): per event a drawn
    // pool event and a drawn global rotation, histograms in the reference's
    // call order
    std::shared_ptr<RandomUtil::Random> rng = ran_gen_ptr.lock();
    for (int h = 0; h < 4; h++)
        for (int e = 0; e < nev; e++) {
            if (nev_mixed < 1)
                throw std::runtime_error("BalanceFunction: the mixed-event pool is empty");
            const int m = rng->rand_int_uniform() % nev_mixed;
            const double rot = rng->rand_uniform() * 2. * M_PI;
            jobs.push_back(hbt_bf_job{4 + h, pairs_of[h][0], e, 4 + pairs_of[h][1], m, 1, rot});
        }
    std::vector<hbt_bf_list> L;
    for (const List &l : lists)
        L.push_back(hbt_bf_list{static_cast<int32_t>(l.off.size() - 1), l.off.data(),
                                l.phi.data(), l.y.data()});
    check(hbt_bf_bin(ctx_, static_cast<int32_t>(L.size()), L.data(),
                     static_cast<int32_t>(jobs.size()), jobs.data()),
          "hbt_bf_bin");
}

std::vector<double> BalanceFunction::histogram(int which) {
    std::vector<double> h(static_cast<size_t>(Bnpts) * HBT_BF_NPHI);
    check(hbt_bf_read(ctx_, which, h.data()), "hbt_bf_read");
    return h;
}

namespace {

// std::scientific with precision 8: printf's "%.8e" (to_chars is specified
// to give the same characters), in a field of `width`.
void put(std::string &o, double v, int width = 0) {
    char tmp[48];
    const std::to_chars_result r =
        std::to_chars(tmp, tmp + sizeof(tmp), v, std::chars_format::scientific, 8);
    const int len = static_cast<int>(r.ptr - tmp);
    for (int k = len; k < width; k++) o.push_back(' ');
    o.append(tmp, len);
}

bool write_text(const std::string &fn, const std::string &text) {
    FILE *f = fopen(fn.c_str(), "w");
    if (!f) return false;
    const bool ok = fwrite(text.data(), 1, text.size(), f) == text.size();
    return fclose(f) == 0 && ok;
}

}  // namespace

void BalanceFunction::output_balance_function() {
    const int n = Bnpts, np = HBT_BF_NPHI;
    std::vector<std::vector<double>> C(8);
    for (int w = 0; w < 8; w++) C[w] = histogram(w);
    auto H = [&](int w, int i, int j) { return C[w][(size_t)i * np + j]; };
    // src/BalanceFunction.cpp:211-244, same summation order
    std::vector<double> os_y(n, 0.), ss_y(n, 0.), os_ym(n, 0.), ss_ym(n, 0.);
    double N_OS = 0., N_OS_m = 0., N_SS = 0., N_SS_m = 0.;
    for (int i = 0; i < n; i++) {
        for (int j = 0; j < np; j++) {
            os_y[i] += H(0, i, j) + H(1, i, j);
            ss_y[i] += H(2, i, j) + H(3, i, j);
            os_ym[i] += H(4, i, j) + H(5, i, j);
            ss_ym[i] += H(6, i, j) + H(7, i, j);
        }
        N_OS += os_y[i];
        N_SS += ss_y[i];
        N_OS_m += os_ym[i];
        N_SS_m += ss_ym[i];
    }
    std::vector<double> os_p(np, 0.), ss_p(np, 0.), os_pm(np, 0.), ss_pm(np, 0.);
    for (int j = 0; j < np; j++)
        for (int i = 0; i < n; i++) {
            os_p[j] += H(0, i, j) + H(1, i, j);
            ss_p[j] += H(2, i, j) + H(3, i, j);
            os_pm[j] += H(4, i, j) + H(5, i, j);
            ss_pm[j] += H(6, i, j) + H(7, i, j);
        }
    std::vector<double> dy(n), dp(np);
    for (int i = 0; i < n; i++) dy[i] = Brap_min + (i + 0.5) * drap;
    for (int j = 0; j < np; j++) dp[j] = Bphi_min + (j + 0.5) * dphi;
    const std::string tag = std::to_string(particle_monval_a) + "_" +
                            std::to_string(particle_monval_b);
    auto row8 = [&](std::string &o, double first, const char *sep1, const double *v) {
        put(o, first, 18);
        o += sep1;
        for (int k = 0; k < 7; k++) {
            if (k > 0) o += "  ";
            put(o, v[k]);
        }
        o += "\n";
    };
    std::string t = "# DeltaY  Delta_C2  C2(OS)  rho2(OS)  rho1^2(OS)  C2(SS) rho2(SS)  rho1^2(SS)\n";
    for (int i = 0; i < n; i++) {
        const double os = os_y[i] / os_ym[i] * N_OS_m / N_OS;
        const double ss = ss_y[i] / ss_ym[i] * N_SS_m / N_SS;
        const double v[7] = {os - ss, os, os_y[i], os_ym[i], ss, ss_y[i], ss_ym[i]};
        row8(t, dy[i], "   ", v);
    }
    bool ok = write_text(path_ + "/Balance_function_" + tag + "_Delta_y.dat", t);
    t = "# Delta_phi  Delta_C2  C2(OS)  rho2(OS)  rho1^2(OS)  C2(SS) rho2(SS)  rho1^2(SS)\n";
    for (int j = 0; j < np; j++) {
        const double os = (os_p[j] / os_pm[j] * N_OS_m / N_OS);
        const double ss = (ss_p[j] / ss_pm[j] * N_SS_m / N_SS);
        const double v[7] = {os - ss, os, os_p[j], os_pm[j], ss, ss_p[j], ss_pm[j]};
        row8(t, dp[j], "   ", v);
    }
    ok = write_text(path_ + "/Balance_function_" + tag + "_Delta_phi.dat", t) && ok;
    t = "# DY  Dphi  C2(OS)  rho2(OS)  rho1^2(OS)  C2(SS)  rho2(SS)  rho1^2(SS)\n";
    for (int i = 0; i < n; i++)
        for (int j = 0; j < np; j++) {
            const double os = ((H(0, i, j) + H(1, i, j)) / (H(4, i, j) + H(5, i, j) + 1e-15));
            const double ss = ((H(2, i, j) + H(3, i, j)) / (H(6, i, j) + H(7, i, j) + 1e-15));
            const double v[7] = {dp[j], os * N_OS_m / N_OS, H(0, i, j) + H(1, i, j),
                                 H(4, i, j) + H(5, i, j), ss * N_SS_m / N_SS,
                                 H(2, i, j) + H(3, i, j), H(6, i, j) + H(7, i, j)};
            row8(t, dy[i], "  ", v);
        }
    ok = write_text(path_ + "/Correlation_function_" + tag + "_2D.dat", t) && ok;
    if (!ok) throw std::runtime_error("BalanceFunction: cannot write the output files under " + path_);
}
