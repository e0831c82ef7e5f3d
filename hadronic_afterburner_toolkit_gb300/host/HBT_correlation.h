// HBT two-particle correlation analysis on the GB300 engine.
//
// Source-compatible with the reference's HBT_correlation
// (src/HBT_correlation.h:14-104): same constructor, same public methods,
// same parameters.dat keys and the same output files.  The histograms live
// on the GPU (libhbt_gpu.so, include/hbt_gpu.h); this class keeps the host
// side of the algorithm: psi_ref, the rapidity gather, the mixed-event
// partner draws and rotations from the shared RandomUtil::Random (in the
// reference's order), and the writers.
//
// One addition: the optional key `hbt_mixed_partners` (> 0) replaces the
// reference's partner count nev/2 + 1 (src/HBT_correlation.cpp:200) with a
// fixed count.  Without the key the reference rule applies.
#pragma once

#include <cstdint>
#include <cmath>
#include <memory>
#include <string>
#include <vector>

#include "ParameterReader.h"
#include "Random.h"
#include "hbt_gpu.h"
#include "particleSamples.h"

// The event-plane sums of src/HBT_correlation.cpp:233-249: over the
// particles in order, phi = atan2(py, px), sum cos(n phi) and sin(n phi);
// psi_ref = atan2(sum sin, sum cos) / n.
struct EventPlaneSums {
    double re = 0.0, im = 0.0;
    void add(double px, double py, int n_order) {
        const double phi = atan2(py, px);
        re += cos(n_order * phi);
        im += sin(n_order * phi);
    }
    double angle(int n_order) const { return atan2(im, re) / n_order; }
};

class HBT_correlation {
  public:
    HBT_correlation(ParameterReader &paraRdr, std::string path,
                    std::shared_ptr<RandomUtil::Random> ran_gen);
    ~HBT_correlation();
    HBT_correlation(const HBT_correlation &) = delete;
    HBT_correlation &operator=(const HBT_correlation &) = delete;

    double get_psi_ref() { return psi_ref; }
    void set_particle_list(std::shared_ptr<particleSamples> particle_list_in) {
        particle_list = particle_list_in;
    }

    void calculate_flow_event_plane_angle(int n_order);
    void calculate_HBT_correlation_function(std::shared_ptr<particleSamples> particle_list_in);
    void combine_and_bin_particle_pairs(std::vector<int> event_list);
    void combine_and_bin_particle_pairs_mixed_events(int event_id,
                                                     std::vector<int> mixed_event_list);

    void output_HBTcorrelation();
    void output_correlation_function_inv();
    void output_correlation_function();
    void output_correlation_function_Kphi_differential();

    // Engine statistics (pairs, launches, deferred K_phi edges, anomalies).
    hbt_stats engine_stats();

  private:
    const ParameterReader paraRdr_;
    const std::string path_;
    std::shared_ptr<particleSamples> particle_list;
    std::shared_ptr<RandomUtil::Random> ran_gen_ptr_;

    bool long_comoving_boost;
    int qnpts;
    double q_min, q_max, delta_q;
    int azimuthal_flag_, invariant_radius_flag_;
    double psi_ref;
    int n_KT, n_Kphi;
    double dKT, dKphi, KT_min, KT_max, Krap_min_, Krap_max_;
    std::vector<double> KT_array_, Kphi_array_, q_out, q_side, q_long;
    int number_of_mixed_events_;
    int number_of_oversample_events_;
    int fixed_mixed_partners_;
    double needed_number_of_pairs_;
    int echo_level_;

    hbt_ctx *ctx_;
    // Gathered lists of the jobs of one batch: columns packed in one host
    // array (each a multiple of 32 doubles, the engine's staging layout, so
    // a batch is staged in one copy); jobs refer to columns by offset.
    struct PendingJob {
        int kind;          // 0 same-event (a, 8 columns), 1 mixed (a x b, 4 + 4)
        long long na, nb;  // particles of a and b
        size_t a[8], b[4]; // column offsets in pack_
    };
    std::vector<double> pack_;
    std::vector<PendingJob> pending_;
    void batch_begin();
    size_t pack_column(long long n);
    void batch_flush();
    void gather_same(const std::vector<int> &event_list);
    void gather_mixed(int event_id1, const std::vector<int> &mixed_event_list);

    // histograms copied back from the device for the writers
    struct HostHist;
    std::unique_ptr<HostHist> fetched_;
    const HostHist &fetch();
    void check(hbt_status s, const char *what);
};

// Reference-format writer shared by the drop-in class and the C API
// (src/HBT_correlation.cpp:694-855).  Arrays as hbt_read_hist /
// hbt_read_qinv / hbt_read_counters return them.
struct hbt_host_hist_view {
    const double *num_count, *q_out_sum, *q_side_sum, *q_long_sum, *num, *den;
    const double *qinv_sum, *qinv_num, *qinv_count, *qinv_den;
    const uint64_t *ctr_num, *ctr_den, *ctr_num_qinv, *ctr_den_qinv;
};
int hbt_write_outputs(const hbt_params &p, const std::string &path, int eco_output,
                      const hbt_host_hist_view &h);
