// C ABI of the drop-in host side (include/hbt_host.h).
#include <chrono>
#include <cmath>
#include <cstring>
#include <iostream>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "Analysis.h"
#include "HBT_correlation.h"
#include "hbt_host.h"

extern "C" {

int hbt_host_run(int argc, char **argv, const char *param_file, const char *results_path) {
    try {
        Analysis analysis(results_path ? results_path : "results");
        analysis.UpdateParameterDict(param_file ? param_file : "parameters.dat", argc, argv);
        analysis.PerformAnalysis();
    } catch (const hbt::ParameterError &e) {
        std::cout << e.what() << std::endl;
        return 255;
    } catch (const std::exception &e) {
        std::cerr << "error: " << e.what() << std::endl;
        return 1;
    }
    return 0;
}

int hbt_host_write(const hbt_params *params, const char *path, int32_t eco_output,
                   const double *num_count, const double *q_out_sum, const double *q_side_sum,
                   const double *q_long_sum, const double *num, const double *den,
                   const double *qinv_sum, const double *qinv_num, const double *qinv_count,
                   const double *qinv_den, const uint64_t *ctr_num, const uint64_t *ctr_den,
                   const uint64_t *ctr_num_qinv, const uint64_t *ctr_den_qinv) {
    if (!params || !path) return -1;
    const hbt_host_hist_view v = {num_count, q_out_sum,  q_side_sum, q_long_sum, num,
                                  den,       qinv_sum,   qinv_num,   qinv_count, qinv_den,
                                  ctr_num,   ctr_den,    ctr_num_qinv, ctr_den_qinv};
    return hbt_write_outputs(*params, path, eco_output, v);
}

double hbt_host_event_plane_angle(int64_t n, const double *px, const double *py,
                                  int32_t n_order) {
    if (n < 0 || (n > 0 && (!px || !py)) || n_order == 0) return NAN;
    EventPlaneSums sums;
    for (int64_t i = 0; i < n; i++) sums.add(px[i], py[i], n_order);
    return sums.angle(n_order);
}

int64_t hbt_host_mixed_plan(int32_t seed, int32_t n_buffers, const int32_t *nev,
                            const int32_t *mixed_nev, int32_t n_partners, int64_t cap,
                            int32_t *partners, double *angles) {
    if (n_buffers < 0 || cap < 0 || (n_buffers > 0 && (!nev || !mixed_nev))) return -1;
    int64_t total = 0;
    for (int b = 0; b < n_buffers; b++) {
        if (nev[b] < 0 || mixed_nev[b] < 0 || (nev[b] > 0 && mixed_nev[b] == 0)) return -1;
        const int nmix = n_partners > 0 ? n_partners : mixed_nev[b] / 2 + 1;
        total += (int64_t)nev[b] * nmix;
    }
    if (total > cap || (total > 0 && (!partners || !angles))) return -1;
    RandomUtil::Random rng(seed);
    int64_t at = 0;
    for (int b = 0; b < n_buffers; b++) {
        const int nmix = n_partners > 0 ? n_partners : mixed_nev[b] / 2 + 1;
        for (int iev = 0; iev < nev[b]; iev++) {
            for (int k = 0; k < nmix; k++) {
                int id = rng.rand_int_uniform() % mixed_nev[b];
                while (iev == id && mixed_nev[b] != 1) id = rng.rand_int_uniform() % mixed_nev[b];
                partners[at + k] = id;
            }
            for (int k = 0; k < nmix; k++) angles[at + k] = rng.rand_uniform() * 2 * M_PI;
            at += nmix;
        }
    }
    return at;
}

int hbt_host_scan_buffers(const char *param_file, const char *results_path, int32_t cap,
                          int32_t *nev, int64_t *n_particles, int32_t *mixed_nev,
                          int64_t *n_mixed_particles) {
    try {
        ParameterReader prm;
        prm.readFromFile(param_file);
        auto rng = std::make_shared<RandomUtil::Random>(1);
        particleSamples ps(prm, results_path, rng);
        int b = 0;
        while (!ps.end_of_file()) {
            ps.read_in_particle_samples_and_filter();
            ps.read_in_particle_samples_mixed_event_and_filter();
            if (b < cap) {
                const int ne = ps.get_number_of_events(), nm = ps.get_number_of_mixed_events();
                int64_t np = 0, nmp = 0;
                for (int e = 0; e < ne; e++) np += ps.get_number_of_particles(e);
                for (int e = 0; e < nm; e++) nmp += ps.get_number_of_particles_mixed_event(e);
                nev[b] = ne;
                n_particles[b] = np;
                mixed_nev[b] = nm;
                n_mixed_particles[b] = nmp;
            }
            b++;
        }
        return b;
    } catch (const std::exception &e) {
        std::cerr << "error: " << e.what() << std::endl;
        return -1;
    }
}

}  // extern "C"

namespace {

struct Fnv {
    uint64_t h = 1469598103934665603ull;
    void add(const void *p, size_t n) {
        const unsigned char *c = static_cast<const unsigned char *>(p);
        for (size_t k = 0; k < n; k++) {
            h ^= c[k];
            h *= 1099511628211ull;
        }
    }
    template <class T>
    void add(const T &v) {
        add(&v, sizeof(v));
    }
};

void hash_events(Fnv &f, const particleSamples &ps, bool mixed) {
    const int ne = mixed ? ps.get_number_of_mixed_events() : ps.get_number_of_events();
    f.add(ne);
    for (int e = 0; e < ne; e++) {
        const std::vector<particle_info> &ev = mixed ? ps.mixed_event(e) : ps.event(e);
        f.add(static_cast<int64_t>(ev.size()));
        for (const particle_info &p : ev) {
            f.add(p.monval);
            const double v[] = {p.mass, p.px, p.py, p.pz, p.E, p.x, p.y, p.z, p.t,
                                p.rap_y, p.rap_eta, p.pT, p.phi_p};
            f.add(v, sizeof(v));
        }
    }
}

void load_params(ParameterReader &prm, const char *param_file, int32_t n_args, char **args) {
    prm.readFromFile(param_file);
    if (n_args > 0) {
        // readFromArguments skips argv[0]
        std::vector<char *> argv(n_args + 1);
        argv[0] = const_cast<char *>("hbt");
        for (int k = 0; k < n_args; k++) argv[k + 1] = args[k];
        prm.readFromArguments(n_args + 1, argv.data());
    }
}

}  // namespace

extern "C" {

int hbt_host_digest_buffers(const char *param_file, const char *results_path, int32_t n_args,
                            char **args, int32_t cap, uint64_t *digest) {
    try {
        ParameterReader prm;
        load_params(prm, param_file, n_args, args);
        auto rng = std::make_shared<RandomUtil::Random>(1);
        particleSamples ps(prm, results_path, rng);
        int b = 0;
        while (!ps.end_of_file()) {
            ps.read_in_particle_samples_and_filter();
            ps.read_in_particle_samples_mixed_event_and_filter();
            if (b < cap) {
                Fnv f;
                hash_events(f, ps, false);
                hash_events(f, ps, true);
                digest[b] = f.h;
            }
            b++;
        }
        return b;
    } catch (const std::exception &e) {
        std::cerr << "error: " << e.what() << std::endl;
        return -1;
    }
}

int hbt_host_time_reader(const char *param_file, const char *results_path, int32_t n_args,
                         char **args, double *seconds, int64_t *particles, int64_t *text_bytes) {
    try {
        ParameterReader prm;
        load_params(prm, param_file, n_args, args);
        auto rng = std::make_shared<RandomUtil::Random>(1);
        const auto t0 = std::chrono::steady_clock::now();
        particleSamples ps(prm, results_path, rng);
        int64_t np = 0;
        while (!ps.end_of_file()) {
            ps.read_in_particle_samples_and_filter();
            ps.read_in_particle_samples_mixed_event_and_filter();
            np += ps.last_buffer_particles();
        }
        const auto t1 = std::chrono::steady_clock::now();
        if (seconds) *seconds = std::chrono::duration<double>(t1 - t0).count();
        if (particles) *particles = np;
        if (text_bytes) *text_bytes = ps.text_bytes();
        return 0;
    } catch (const std::exception &e) {
        std::cerr << "error: " << e.what() << std::endl;
        return -1;
    }
}

}  // extern "C"
