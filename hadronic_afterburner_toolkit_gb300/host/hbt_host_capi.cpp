// C ABI of the drop-in host side (include/hbt_host.h).
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
