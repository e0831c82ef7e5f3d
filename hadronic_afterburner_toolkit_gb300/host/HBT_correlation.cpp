#include "HBT_correlation.h"

#include <atomic>

#include <charconv>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <iostream>
#include <sstream>
#include <stdexcept>

namespace {

std::string fmt_edge(double v) {
    std::ostringstream s;
    s << v;  // default ostream formatting, as in the reference's file names
    return s.str();
}

}  // namespace

struct HBT_correlation::HostHist {
    std::vector<double> cnt, qo, qs, ql, num, den, qi_sum, qi_num, qi_cnt, qi_den;
    std::vector<uint64_t> c_num, c_den, c_num_qi, c_den_qi;
};

HBT_correlation::HBT_correlation(ParameterReader &paraRdr, std::string path,
                                 std::shared_ptr<RandomUtil::Random> ran_gen)
    : paraRdr_(paraRdr), path_(path), ran_gen_ptr_(ran_gen), ctx_(nullptr) {
    // keys and derived constants of src/HBT_correlation.cpp:22-61
    long_comoving_boost = paraRdr_.getVal("long_comoving_boost") == 1;
    qnpts = static_cast<int>(paraRdr_.getVal("qnpts"));
    q_min = paraRdr_.getVal("q_min");
    q_max = paraRdr_.getVal("q_max");
    delta_q = (q_max - q_min) / (qnpts - 1);
    for (int i = 0; i < qnpts; i++) {
        q_out.push_back(q_min + i * delta_q);
        q_side.push_back(q_min + i * delta_q);
        q_long.push_back(q_min + i * delta_q);
    }
    needed_number_of_pairs_ = paraRdr_.getVal("needed_number_of_pairs");
    azimuthal_flag_ = static_cast<int>(paraRdr_.getVal("azimuthal_flag"));
    invariant_radius_flag_ = static_cast<int>(paraRdr_.getVal("invariant_radius_flag"));
    n_KT = static_cast<int>(paraRdr_.getVal("n_KT"));
    n_Kphi = static_cast<int>(paraRdr_.getVal("n_Kphi"));
    KT_min = paraRdr_.getVal("KT_min");
    KT_max = paraRdr_.getVal("KT_max");
    Krap_min_ = paraRdr_.getVal("HBTrap_min");
    Krap_max_ = paraRdr_.getVal("HBTrap_max");
    dKT = (KT_max - KT_min) / (n_KT - 1);
    dKphi = 2 * M_PI / n_Kphi;
    for (int i = 0; i < n_KT; i++) KT_array_.push_back(KT_min + i * dKT);
    for (int i = 0; i < n_Kphi; i++) Kphi_array_.push_back(i * dKphi);
    psi_ref = 0.;
    number_of_mixed_events_ = 0;
    number_of_oversample_events_ = 0;
    fixed_mixed_partners_ = paraRdr_.exist("hbt_mixed_partners")
                                ? static_cast<int>(paraRdr_.getVal("hbt_mixed_partners"))
                                : 0;
    echo_level_ = paraRdr_.exist("echo_level") ? static_cast<int>(paraRdr_.getVal("echo_level")) : 0;

    hbt_params p;
    p.qnpts = qnpts;
    p.q_min = q_min;
    p.q_max = q_max;
    p.n_KT = n_KT;
    p.KT_min = KT_min;
    p.KT_max = KT_max;
    p.n_Kphi = n_Kphi;
    p.azimuthal_flag = azimuthal_flag_;
    p.invariant_radius_flag = invariant_radius_flag_;
    p.long_comoving_boost = long_comoving_boost ? 1 : 0;
    p.needed_number_of_pairs = needed_number_of_pairs_;
    p.precision = paraRdr_.exist("hbt_precision")
                      ? static_cast<int>(paraRdr_.getVal("hbt_precision"))
                      : HBT_PRECISION_FP64;
    p.kphi_defer_tol = 0.0;
    p.kernel = paraRdr_.exist("hbt_kernel") ? static_cast<int>(paraRdr_.getVal("hbt_kernel"))
                                            : HBT_KERNEL_SCREENED;
    const int device =
        paraRdr_.exist("hbt_device") ? static_cast<int>(paraRdr_.getVal("hbt_device")) : 0;
    const hbt_status s = hbt_create(&p, device, &ctx_);
    if (s != HBT_OK)
        throw std::runtime_error("HBT_correlation: hbt_create failed (status " +
                                 std::to_string(static_cast<int>(s)) + ")");
}

HBT_correlation::~HBT_correlation() { hbt_destroy(ctx_); }

void HBT_correlation::check(hbt_status s, const char *what) {
    if (s != HBT_OK)
        throw std::runtime_error(std::string("HBT_correlation: ") + what + ": " +
                                 hbt_last_error(ctx_));
}

hbt_stats HBT_correlation::engine_stats() {
    hbt_stats st;
    check(hbt_get_stats(ctx_, &st), "hbt_get_stats");
    return st;
}

// src/HBT_correlation.cpp:177-218
void HBT_correlation::calculate_HBT_correlation_function(
    std::shared_ptr<particleSamples> particle_list_in) {
    set_particle_list(particle_list_in);
    fetched_.reset();
    const int nev = particle_list->get_number_of_events();
    if (azimuthal_flag_ == 1) calculate_flow_event_plane_angle(2);
    check(hbt_set_psi_ref(ctx_, psi_ref), "hbt_set_psi_ref");

    number_of_oversample_events_ = nev;
    std::vector<int> event_list(nev);
    for (int k = 0; k < nev; k++) event_list[k] = k;
    // the buffer's same-event list and every event's mixed-event lists are
    // gathered in the reference's order (same RNG draws) and binned in one
    // batched launch; hbt_bin_batch keeps the reference's job order when a
    // pair cap can bind
    batch_begin();
    gather_same(event_list);

    const int mixed_nev = particle_list->get_number_of_mixed_events();
    number_of_mixed_events_ =
        fixed_mixed_partners_ > 0 ? fixed_mixed_partners_ : mixed_nev / 2 + 1;
    if (nev > 0 && mixed_nev == 0)
        throw std::runtime_error("HBT_correlation: the mixed-event pool of this buffer is empty");
    for (int iev = 0; iev < nev; iev++) {
        std::vector<int> partners(number_of_mixed_events_, 0);
        for (int k = 0; k < number_of_mixed_events_; k++) {
            int id = ran_gen_ptr_->rand_int_uniform() % mixed_nev;
            while (iev == id && mixed_nev != 1) id = ran_gen_ptr_->rand_int_uniform() % mixed_nev;
            partners[k] = id;
        }
        gather_mixed(iev, partners);
    }
    batch_flush();
}

// src/HBT_correlation.cpp:233-249
void HBT_correlation::calculate_flow_event_plane_angle(int n_order) {
    const int nev = particle_list->get_number_of_events();
    EventPlaneSums sums;
    for (int iev = 0; iev < nev; iev++)
        for (const particle_info &p : particle_list->event(iev)) sums.add(p.px, p.py, n_order);
    psi_ref = sums.angle(n_order);
}

// Host lists of a batch: every column occupies a multiple of 32 doubles of
// one packed array, the layout the engine's staging copies to the device,
// so the whole batch goes over in one copy.
void HBT_correlation::batch_begin() {
    pack_.clear();
    pending_.clear();
}

size_t HBT_correlation::pack_column(long long n) {
    const size_t at = pack_.size();
    pack_.resize(at + static_cast<size_t>((n + 31) / 32 * 32), 0.0);
    return at;
}

void HBT_correlation::batch_flush() {
    std::vector<hbt_job> jobs;
    jobs.reserve(pending_.size());
    const double *base = pack_.data();
    for (const PendingJob &pj : pending_) {
        hbt_job j = {};
        j.kind = pj.kind;
        j.na = pj.na;
        j.nb = pj.nb;
        const double **a[8] = {&j.a.px, &j.a.py, &j.a.pz, &j.a.E,
                               &j.a.x,  &j.a.y,  &j.a.z,  &j.a.t};
        const double **b[4] = {&j.b.px, &j.b.py, &j.b.pz, &j.b.E};
        for (int f = 0; f < (pj.kind == 0 ? 8 : 4); f++) *a[f] = base + pj.a[f];
        if (pj.kind == 1)
            for (int f = 0; f < 4; f++) *b[f] = base + pj.b[f];
        jobs.push_back(j);
    }
    if (!jobs.empty())
        check(hbt_bin_batch(ctx_, static_cast<int32_t>(jobs.size()), jobs.data()),
              "hbt_bin_batch");
    batch_begin();
}

// Gather of src/HBT_correlation.cpp:254-285 into the batch.
void HBT_correlation::gather_same(const std::vector<int> &event_list) {
    const double ycut_max = tanh(Krap_max_);
    const double ycut_min = tanh(Krap_min_);
    long long n = 0;
    for (int j = 0; j < number_of_oversample_events_; j++)
        for (const particle_info &p : particle_list->event(event_list[j])) {
            const double ratio = p.pz / p.E;
            if (ratio > ycut_min && ratio < ycut_max) n++;
        }
    PendingJob pj = {};
    pj.kind = 0;
    pj.na = n;
    for (int f = 0; f < 8; f++) pj.a[f] = pack_column(n);
    long long k = 0;
    for (int j = 0; j < number_of_oversample_events_; j++)
        for (const particle_info &p : particle_list->event(event_list[j])) {
            const double ratio = p.pz / p.E;
            if (ratio > ycut_min && ratio < ycut_max) {
                const double v[8] = {p.px, p.py, p.pz, p.E, p.x, p.y, p.z, p.t};
                for (int f = 0; f < 8; f++) pack_[pj.a[f] + k] = v[f];
                k++;
            }
        }
    if (echo_level_ > 5)
        std::cout << "[Info] number of pairs: " << (unsigned long long)(n * (n - 1) / 2)
                  << std::endl;
    pending_.push_back(pj);
}

// Gather and random rotation of src/HBT_correlation.cpp:466-552 into the
// batch: one rotation angle drawn per partner event, in partner order.
void HBT_correlation::gather_mixed(int event_id1, const std::vector<int> &mixed_event_list) {
    const double ycut_max = tanh(Krap_max_);
    const double ycut_min = tanh(Krap_min_);
    PendingJob pj = {};
    pj.kind = 1;
    for (const particle_info &p : particle_list->event(event_id1)) {
        const double ratio = p.pz / p.E;
        if (ratio > ycut_min && ratio < ycut_max) pj.na++;
    }
    for (int f = 0; f < 4; f++) pj.a[f] = pack_column(pj.na);
    long long k = 0;
    for (const particle_info &p : particle_list->event(event_id1)) {
        const double ratio = p.pz / p.E;
        if (ratio > ycut_min && ratio < ycut_max) {
            pack_[pj.a[0] + k] = p.px;
            pack_[pj.a[1] + k] = p.py;
            pack_[pj.a[2] + k] = p.pz;
            pack_[pj.a[3] + k] = p.E;
            k++;
        }
    }
    for (int iev = 0; iev < number_of_mixed_events_; iev++)
        for (const particle_info &p : particle_list->mixed_event(mixed_event_list[iev])) {
            const double ratio = p.pz / p.E;
            if (ratio > ycut_min && ratio < ycut_max) pj.nb++;
        }
    for (int f = 0; f < 4; f++) pj.b[f] = pack_column(pj.nb);
    k = 0;
    for (int iev = 0; iev < number_of_mixed_events_; iev++) {
        const double random_rotation = ran_gen_ptr_->rand_uniform() * 2 * M_PI;
        const double cos_phi = cos(random_rotation);
        const double sin_phi = sin(random_rotation);
        for (const particle_info &p : particle_list->mixed_event(mixed_event_list[iev])) {
            const double ratio = p.pz / p.E;
            if (ratio > ycut_min && ratio < ycut_max) {
                pack_[pj.b[0] + k] = p.px * cos_phi - p.py * sin_phi;
                pack_[pj.b[1] + k] = p.px * sin_phi + p.py * cos_phi;
                pack_[pj.b[2] + k] = p.pz;
                pack_[pj.b[3] + k] = p.E;
                k++;
            }
        }
    }
    if (echo_level_ > 5)
        std::cout << "[Info] number of mixed pairs: " << (unsigned long long)(pj.na * pj.nb)
                  << std::endl;
    pending_.push_back(pj);
}

// Pair loop of src/HBT_correlation.cpp:282-461 on the GPU.
void HBT_correlation::combine_and_bin_particle_pairs(std::vector<int> event_list) {
    batch_begin();
    gather_same(event_list);
    batch_flush();
}

// Pair loop of src/HBT_correlation.cpp:554-689 on the GPU.
void HBT_correlation::combine_and_bin_particle_pairs_mixed_events(
    int event_id1, std::vector<int> mixed_event_list) {
    batch_begin();
    gather_mixed(event_id1, mixed_event_list);
    batch_flush();
}

const HBT_correlation::HostHist &HBT_correlation::fetch() {
    if (fetched_) return *fetched_;
    std::unique_ptr<HostHist> h(new HostHist());
    const size_t nb = static_cast<size_t>(hbt_n_bins(ctx_));
    const size_t nq = static_cast<size_t>(n_KT) * qnpts;
    const size_t ns = static_cast<size_t>(azimuthal_flag_ == 1 ? n_KT * n_Kphi : n_KT);
    for (auto *v : {&h->cnt, &h->qo, &h->qs, &h->ql, &h->num, &h->den}) v->assign(nb, 0.0);
    for (auto *v : {&h->qi_sum, &h->qi_num, &h->qi_cnt, &h->qi_den}) v->assign(nq, 0.0);
    h->c_num.assign(ns, 0);
    h->c_den.assign(ns, 0);
    h->c_num_qi.assign(n_KT, 0);
    h->c_den_qi.assign(n_KT, 0);
    check(hbt_read_hist(ctx_, h->cnt.data(), h->qo.data(), h->qs.data(), h->ql.data(),
                        h->num.data(), h->den.data()),
          "hbt_read_hist");
    check(hbt_read_qinv(ctx_, h->qi_sum.data(), h->qi_num.data(), h->qi_cnt.data(),
                        h->qi_den.data()),
          "hbt_read_qinv");
    check(hbt_read_counters(ctx_, h->c_num.data(), h->c_den.data(), h->c_num_qi.data(),
                            h->c_den_qi.data()),
          "hbt_read_counters");
    fetched_ = std::move(h);
    return *fetched_;
}

namespace {

hbt_params params_of(int qnpts, double q_min, double q_max, int n_KT, double KT_min,
                     double KT_max, int n_Kphi, int az, int qinv) {
    hbt_params p = {};
    p.qnpts = qnpts;
    p.q_min = q_min;
    p.q_max = q_max;
    p.n_KT = n_KT;
    p.KT_min = KT_min;
    p.KT_max = KT_max;
    p.n_Kphi = n_Kphi;
    p.azimuthal_flag = az;
    p.invariant_radius_flag = qinv;
    return p;
}

}  // namespace

void HBT_correlation::output_HBTcorrelation() {
    const HostHist &h = fetch();
    const hbt_params p = params_of(qnpts, q_min, q_max, n_KT, KT_min, KT_max, n_Kphi,
                                   azimuthal_flag_, invariant_radius_flag_);
    const hbt_host_hist_view v = {h.cnt.data(),    h.qo.data(),     h.qs.data(),
                                  h.ql.data(),     h.num.data(),    h.den.data(),
                                  h.qi_sum.data(), h.qi_num.data(), h.qi_cnt.data(),
                                  h.qi_den.data(), h.c_num.data(),  h.c_den.data(),
                                  h.c_num_qi.data(), h.c_den_qi.data()};
    const int eco = static_cast<int>(paraRdr_.getVal("ecoOutput", 0));
    if (hbt_write_outputs(p, path_, eco, v) != 0)
        throw std::runtime_error("HBT_correlation: cannot write output files under " + path_);
}

void HBT_correlation::output_correlation_function_inv() {
    if (invariant_radius_flag_ == 1) output_HBTcorrelation();
}
void HBT_correlation::output_correlation_function() { output_HBTcorrelation(); }
void HBT_correlation::output_correlation_function_Kphi_differential() { output_HBTcorrelation(); }

// ------------------------------------------------------------------ writer

namespace {

// "%W.8e" of printf: std::to_chars in scientific form with precision 8 is
// specified to give printf's characters (exact decimal conversion, at least
// two exponent digits, "inf" / "nan" with their sign), right-aligned in a
// field of `width`.
char *put_e(char *p, double v, int width) {
    char tmp[48];
    const std::to_chars_result r =
        std::to_chars(tmp, tmp + sizeof(tmp), v, std::chars_format::scientific, 8);
    const int len = static_cast<int>(r.ptr - tmp);
    for (int k = len; k < width; k++) *p++ = ' ';
    memcpy(p, tmp, len);
    return p + len;
}

// One row: std::scientific, setprecision(8), setw(18) on the first field
// only, four blanks between fields (the reference's writer).
char *row(char *p, int nfield, const double *v) {
    for (int k = 0; k < nfield; k++) {
        if (k > 0) {
            memcpy(p, "    ", 4);
            p += 4;
        }
        p = put_e(p, v[k], k == 0 ? 18 : 0);
    }
    *p++ = '\n';
    return p;
}

bool write_file(const std::string &fn, const std::string &text) {
    FILE *f = fopen(fn.c_str(), "w");
    if (!f) return false;
    const bool ok = fwrite(text.data(), 1, text.size(), f) == text.size();
    return fclose(f) == 0 && ok;
}

}  // namespace

// The files are formatted in memory and written on all host threads, one
// file per task.
int hbt_write_outputs(const hbt_params &p, const std::string &path, int eco_output,
                      const hbt_host_hist_view &h) {
    const bool eco = eco_output == 1;
    const int n = p.qnpts;
    const double delta_q = (p.q_max - p.q_min) / (n - 1);
    const double dKT = (p.KT_max - p.KT_min) / (p.n_KT - 1);
    const double dKphi = 2 * M_PI / p.n_Kphi;
    std::vector<double> grid(n), KT(p.n_KT), Kphi(p.n_Kphi);
    for (int i = 0; i < n; i++) grid[i] = p.q_min + i * delta_q;
    for (int i = 0; i < p.n_KT; i++) KT[i] = p.KT_min + i * dKT;
    for (int i = 0; i < p.n_Kphi; i++) Kphi[i] = i * dKphi;
    const long long q3 = (long long)n * n * n;
    std::atomic<bool> failed(false);

    // q_inv files (src/HBT_correlation.cpp:694-724)
    if (p.invariant_radius_flag == 1) {
        hbt::parallel_ranges(p.n_KT - 1, 0, 1, [&](long lo, long hi) {
            std::string text;
            for (long iK = lo; iK < hi; iK++) {
                const double ratio = static_cast<double>(h.ctr_num_qinv[iK]) /
                                     static_cast<double>(h.ctr_den_qinv[iK]);
                const std::string fn = path + "/HBT_correlation_function_inv_KT_" +
                                       fmt_edge(KT[iK]) + "_" + fmt_edge(KT[iK + 1]) + ".dat";
                text.assign(static_cast<size_t>(n) * 64, '\0');
                char *o = &text[0];
                for (int k = 0; k < n; k++) {
                    const long long at = (long long)iK * n + k;
                    const double v[3] = {h.qinv_sum[at] / h.qinv_count[at], h.qinv_num[at],
                                         h.qinv_den[at] * ratio};
                    o = eco ? row(o, 2, v + 1) : row(o, 3, v);
                }
                text.resize(o - text.data());
                if (!write_file(fn, text)) failed = true;
            }
        });
    }
    // 3-D files (src/HBT_correlation.cpp:726-855)
    const int nphi = p.azimuthal_flag == 1 ? p.n_Kphi : 1;
    hbt::parallel_ranges(static_cast<long>(p.n_KT - 1) * nphi, 0, 1, [&](long lo, long hi) {
        std::string text;
        for (long task = lo; task < hi; task++) {
            const int iK = static_cast<int>(task / nphi), ip = static_cast<int>(task % nphi);
            const int s = p.azimuthal_flag == 1 ? iK * p.n_Kphi + ip : iK;
            const double ratio =
                static_cast<double>(h.ctr_num[s]) / static_cast<double>(h.ctr_den[s]);
            std::string fn = path + "/HBT_correlation_function_KT_" + fmt_edge(KT[iK]) + "_" +
                             fmt_edge(KT[iK + 1]);
            if (p.azimuthal_flag == 1) fn += "_Kphi_" + fmt_edge(Kphi[ip]);
            fn += ".dat";
            text.assign(static_cast<size_t>(q3) * 96, '\0');
            char *o = &text[0];
            for (int il = 0; il < n; il++)
                for (int io = 0; io < n; io++)
                    for (int is = 0; is < n; is++) {
                        const long long at = s * q3 + ((long long)io * n + is) * n + il;
                        const int npart_num = static_cast<int>(h.num_count[at]);
                        const int npart_den = static_cast<int>(h.den[at]);
                        double v[5];
                        if (npart_num < 2 || npart_den < 2) {
                            v[0] = grid[io];
                            v[1] = grid[is];
                            v[2] = grid[il];
                            v[3] = 0.0;
                            v[4] = static_cast<double>(npart_den);
                        } else {
                            v[0] = h.q_out_sum[at] / npart_num;
                            v[1] = h.q_side_sum[at] / npart_num;
                            v[2] = h.q_long_sum[at] / npart_num;
                            v[3] = h.num[at];
                            v[4] = ratio * h.den[at];
                        }
                        o = eco ? row(o, 2, v + 3) : row(o, 5, v);
                    }
            text.resize(o - text.data());
            if (!write_file(fn, text)) failed = true;
        }
    });
    return failed ? -1 : 0;
}
