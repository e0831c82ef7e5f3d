// Balance functions of two species: the reference's BalanceFunction class
// (src/BalanceFunction.{h,cpp}) with its pair loops on the GPU
// (include/hbt_bf.h).  Same parameter keys (particle_alpha, particle_beta,
// BpT_min, BpT_max, Bnpts, Brap_max, rap_type), the same draws of the
// mixed-event partners and rotations from the shared Random, and the same
// three output files.
#pragma once

#include <memory>
#include <string>
#include <vector>

#include "../../include/hbt_bf.h"
#include "ParameterReader.h"
#include "Random.h"
#include "particleSamples.h"

class BalanceFunction {
  public:
    BalanceFunction(const ParameterReader &paraRdr, const std::string path,
                    std::shared_ptr<RandomUtil::Random> ran_gen);
    ~BalanceFunction();
    BalanceFunction(const BalanceFunction &) = delete;
    BalanceFunction &operator=(const BalanceFunction &) = delete;

    void set_particle_list(std::shared_ptr<particleSamples> particle_list_in) {
        particle_list = particle_list_in;
    }
    // One buffer: the four same-event and four mixed-event histograms
    // (src/BalanceFunction.cpp:60-97).
    void calculate_balance_function(std::shared_ptr<particleSamples> particle_list_in);
    // The three files (src/BalanceFunction.cpp:211-319).
    void output_balance_function();

    // The counts of histogram `which` (0..7: ab, abar bbar, a bbar, abar b,
    // then the mixed-event four), [y bin][phi bin].
    std::vector<double> histogram(int which);

  private:
    const ParameterReader paraRdr_;
    const std::string path_;
    std::shared_ptr<particleSamples> particle_list;
    std::weak_ptr<RandomUtil::Random> ran_gen_ptr;

    int particle_monval_a, particle_monval_b;
    int rap_type_, Bnpts;
    double Brap_max, BpT_min, BpT_max, drap, Brap_min, dphi, Bphi_min;
    long N_b = 0, N_bbar = 0;
    hbt_bf_ctx *ctx_ = nullptr;

    void check(hbt_status s, const char *what);
};
