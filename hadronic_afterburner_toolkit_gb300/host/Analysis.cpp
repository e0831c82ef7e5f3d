#include "Analysis.h"

#include <fstream>
#include <iostream>

#include "BalanceFunction.h"
#include "HBT_correlation.h"

Analysis::Analysis(std::string path) : path_(path) {}

void Analysis::UpdateParameterDict(std::string param_filename) {
    paraRdr_.readFromFile(param_filename);
    paraRdr_.echo();
}

// src/Analysis.cpp:24-34
void Analysis::UpdateParameterDict(std::string param_filename, int argc, char *argv[]) {
    paraRdr_.readFromFile(param_filename);
    paraRdr_.readFromArguments(argc, argv);
    if (paraRdr_.getVal("readRapidityShiftFromFile", 0) == 1) setRapidityShiftFromFile();
    paraRdr_.echo();
}

// src/Analysis.cpp:36-47: "dummy dummy shift" from rapidity_shift.dat
void Analysis::setRapidityShiftFromFile() {
    std::ifstream in("rapidity_shift.dat");
    if (!in) {
        std::cout << "[Warning] Failed to open the file 'rapidity_shift.dat'." << std::endl;
        return;
    }
    double dummy, shift;
    in >> dummy >> dummy >> shift;
    paraRdr_.setVal("rapidity_shift", shift);
}

void Analysis::InitializeAnalysis() {
    const int seed = static_cast<int>(paraRdr_.getVal("randomSeed", -1));
    ran_gen_ptr_ = std::make_shared<RandomUtil::Random>(seed);
}

void Analysis::PerformAnalysis() {
    InitializeAnalysis();
    if (paraRdr_.getVal("analyze_flow") != 0)
        std::cout << "[Warning] analyze_flow: the flow analysis is not part of this library; "
                     "skipped" << std::endl;
    if (paraRdr_.getVal("analyze_HBT") == 1) {
        std::cout << "[Info] Analyze HBT ..." << std::endl;
        particle_list_ = std::make_shared<particleSamples>(paraRdr_, path_, ran_gen_ptr_);
        HBTAnalysis();
        particle_list_.reset();
    }
    if (paraRdr_.getVal("analyze_balance_function") == 1) {
        std::cout << "[Info] Analyze balance functions ..." << std::endl;
        particle_list_ = std::make_shared<particleSamples>(paraRdr_, path_, ran_gen_ptr_);
        BalanceFunctionAnalysis();
        particle_list_.reset();
    }
    if (paraRdr_.getVal("analyze_ebe_yield") == 1)
        std::cout << "[Warning] analyze_ebe_yield: not part of this library; skipped" << std::endl;
}

// src/Analysis.cpp:817-835
void Analysis::HBTAnalysis() {
    HBT_correlation hbt(paraRdr_, path_, ran_gen_ptr_);
    int event_id = 0;
    while (!particle_list_->end_of_file()) {
        particle_list_->read_in_particle_samples_and_filter();
        particle_list_->read_in_particle_samples_mixed_event_and_filter();
        const int nev = particle_list_->get_number_of_events();
        std::cout << "[Info] Reading event: " << event_id + 1 << " ... nev = " << nev
                  << std::endl;
        hbt.calculate_HBT_correlation_function(particle_list_);
        event_id += nev;
    }
    hbt.output_HBTcorrelation();
    const hbt_stats st = hbt.engine_stats();
    std::cout << "[Info] HBT pairs: " << st.pairs_same << " same-event, " << st.pairs_mixed
              << " mixed-event; " << st.launches << " GPU launches, " << st.deferred_kphi
              << " K_phi edge pairs decided on the host" << std::endl;
}

// src/Analysis.cpp:856-874
void Analysis::BalanceFunctionAnalysis() {
    BalanceFunction bf(paraRdr_, path_, ran_gen_ptr_);
    int event_id = 0;
    while (!particle_list_->end_of_file()) {
        particle_list_->read_in_particle_samples_and_filter();
        particle_list_->read_in_particle_samples_mixed_event_and_filter();
        const int nev = particle_list_->get_number_of_events();
        std::cout << "[Info] Reading event: " << event_id + 1 << " ... nev = " << nev
                  << std::endl;
        bf.calculate_balance_function(particle_list_);
        event_id += nev;
    }
    bf.output_balance_function();
}
