#include "particleSamples.h"

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <sstream>
#include <stdexcept>

particleSamples::particleSamples(ParameterReader &paraRdr, std::string path,
                                 std::shared_ptr<RandomUtil::Random> ran_gen)
    : paraRdr_(paraRdr), path_(path) {
    (void)ran_gen;  // resonance decays (the reference's only use) are not built
    echo_level_ = static_cast<int>(paraRdr_.getVal("echo_level"));
    event_buffer_size_ = static_cast<int>(paraRdr_.getVal("event_buffer_size"));
    read_in_mode_ = static_cast<int>(paraRdr_.getVal("read_in_mode"));
    rap_shift_ = paraRdr_.getVal("rapidity_shift", 0);
    read_mixed_events_ = paraRdr_.getVal("read_in_real_mixed_events") == 1;
    particle_monval_ = static_cast<int>(paraRdr_.getVal("particle_monval"));
    analyze_bf_ = paraRdr_.exist("analyze_balance_function") &&
                  paraRdr_.getVal("analyze_balance_function") == 1;
    if (analyze_bf_) {
        // src/particleSamples.cpp:66-71
        const int a = static_cast<int>(paraRdr_.getVal("particle_alpha"));
        const int b = static_cast<int>(paraRdr_.getVal("particle_beta"));
        bf_monval_[0] = a;
        bf_monval_[1] = -a;
        bf_monval_[2] = b;
        bf_monval_[3] = -b;
    }
    if (paraRdr_.getVal("resonance_feed_down_flag") == 1 ||
        paraRdr_.getVal("resonance_weak_feed_down_flag") == 1)
        throw std::runtime_error("particleSamples: resonance decays are not part of this library");

    std::string file, file_mixed;
    bool gz = false;
    if (read_in_mode_ == 0) {
        file = path_ + "/OSCAR.DAT";
        file_mixed = path_ + "/OSCAR_mixed_event.DAT";
    } else if (read_in_mode_ == 10) {
        file = path_ + "/particle_samples.gz";
        file_mixed = path_ + "/particle_samples_mixed_event.gz";
        gz = true;
    } else {
        throw std::runtime_error("particleSamples: read_in_mode " +
                                 std::to_string(read_in_mode_) +
                                 " is not supported by this library (0 and 10 are)");
    }
    const bool fast =
        !paraRdr_.exist("hbt_fast_reader") || paraRdr_.getVal("hbt_fast_reader") != 0;
    reader_threads_ = paraRdr_.exist("hbt_reader_threads")
                          ? static_cast<int>(paraRdr_.getVal("hbt_reader_threads"))
                          : 0;
    const int threads = reader_threads_;
    const bool cache =
        paraRdr_.exist("hbt_binary_cache") && paraRdr_.getVal("hbt_binary_cache") != 0;
    auto open = [&](const std::string &f) {
        if (!fast) return hbt::make_line_source(f, gz, read_in_mode_);
        return cache ? hbt::make_cached_source(f, gz, read_in_mode_, threads)
                     : hbt::make_block_source(f, gz, read_in_mode_, threads);
    };
    in_ = open(file);
    if (!in_->ok())
        throw std::runtime_error("particleSamples:: Error: input file: " + file + " can not open!");
    if (read_mixed_events_) {
        in_mixed_ = open(file_mixed);
        if (!in_mixed_->ok())
            throw std::runtime_error("particleSamples:: Error: input file: " + file_mixed +
                                     " can not open!");
    }
    list_ = &filtered_;
    mixed_list_ = read_mixed_events_ ? &filtered_mixed_ : &filtered_;
}

particleSamples::~particleSamples() = default;

bool particleSamples::end_of_file() const { return in_->eof(); }

long long particleSamples::last_buffer_particles() const {
    long long n = 0;
    for (const auto &ev : full_) n += static_cast<long long>(ev.size());
    if (read_mixed_events_)
        for (const auto &ev : full_mixed_) n += static_cast<long long>(ev.size());
    return n;
}

long long particleSamples::text_bytes() const {
    return in_->text_bytes() + (in_mixed_ ? in_mixed_->text_bytes() : 0);
}
bool particleSamples::end_of_file_mixed_event() const {
    return in_mixed_ ? in_mixed_->eof() : in_->eof();
}

// particleSamples::boostParticles (src/particleSamples.cpp:442-468).
void particleSamples::boost(EventList &evs) const {
    const double ch = cosh(rap_shift_), sh = sinh(rap_shift_);
    hbt::parallel_ranges(static_cast<long>(evs.size()), reader_threads_, 8, [&](long lo, long hi) {
        for (long e = lo; e < hi; e++)
            for (auto &p : evs[e]) {
            p.pT = sqrt(p.px * p.px + p.py * p.py);
            const double mT = sqrt(p.pT * p.pT + p.mass * p.mass);
            p.phi_p = atan2(p.py, p.px);
            const double E = p.E * ch + p.pz * sh;
            const double pz = p.pz * ch + p.E * sh;
            p.E = E;
            p.pz = pz;
                p.rap_y = asinh(p.pz / mT);
                p.rap_eta = asinh(p.pz / p.pT);
            }
    });
}

int particleSamples::read_in_particle_samples() {
    in_->read_buffer(event_buffer_size_, full_);
    boost(full_);
    return static_cast<int>(full_.size());
}

int particleSamples::read_in_particle_samples_mixed_event() {
    in_mixed_->read_buffer(event_buffer_size_, full_mixed_);
    boost(full_mixed_);
    return static_cast<int>(full_mixed_.size());
}

void particleSamples::read_in_particle_samples_and_filter() {
    read_in_particle_samples();
    filter(full_, filtered_);
    if (analyze_bf_)
        for (int s = 0; s < 4; s++) filter_code(bf_monval_[s], full_, bf_[s]);
}

void particleSamples::read_in_particle_samples_mixed_event_and_filter() {
    if (!read_mixed_events_) {
        mixed_list_ = &filtered_;
        return;
    }
    read_in_particle_samples_mixed_event();
    filter(full_mixed_, filtered_mixed_);
    mixed_list_ = &filtered_mixed_;
    if (analyze_bf_)
        for (int s = 0; s < 4; s++) filter_code(bf_monval_[s], full_mixed_, bf_mixed_[s]);
}

void particleSamples::filter(const EventList &full, EventList &out) {
    out.clear();
    out.resize(full.size());
    for (size_t e = 0; e < full.size(); e++)
        for (const auto &p : full[e])
            if (pick(p.monval)) out[e].push_back(p);
}

void particleSamples::filter_code(int poi, const EventList &full, EventList &out) {
    out.clear();
    out.resize(full.size());
    for (size_t e = 0; e < full.size(); e++)
        for (const auto &p : full[e])
            if (pick_code(poi, p.monval)) out[e].push_back(p);
}

// decide_to_pick_OSCAR (src/particleSamples.cpp:625-678).
bool particleSamples::pick_code(int poi, int monval) {
    if (poi == 99999) return true;
    const bool klass = poi == 9999 || poi == 9998 || poi == -9998 || poi == 9997 ||
                       poi == -9997 || poi == 9996 || poi == -9996;
    if (!klass) return monval == poi;
    load_pdg();
    auto get = [&](const std::map<int, int> &m) {
        auto it = m.find(monval);
        if (it == m.end())
            throw std::runtime_error("particleSamples: Monte-Carlo number " +
                                     std::to_string(monval) + " not in EOS/pdg.dat");
        return it->second;
    };
    switch (poi) {
        case 9999: return get(charge_) != 0;
        case 9998: return get(charge_) > 0;
        case -9998: return get(charge_) < 0;
        case 9997: return get(baryon_) > 0;
        case -9997: return get(baryon_) < 0;
        case 9996: return get(strange_) > 0;
        default: return get(strange_) < 0;
    }
}

// Quantum numbers of EOS/pdg.dat (the reference's particle_decay table,
// src/particle_decay.cpp:24-110): per species a header line
// "monval name mass width gspin baryon strange charm bottom gisospin charge
// decays" followed by `decays` channel lines of 8 numbers; baryons also get
// an anti-particle entry with opposite quantum numbers.
void particleSamples::load_pdg() {
    if (pdg_loaded_) return;
    std::ifstream f("EOS/pdg.dat");
    if (!f) throw std::runtime_error("can not find the file EOS/pdg.dat!");
    int monval;
    while (f >> monval) {
        std::string name;
        double mass, width;
        int gspin, baryon, strange, charm, bottom, giso, charge, decays;
        f >> name >> mass >> width >> gspin >> baryon >> strange >> charm >> bottom >> giso >>
            charge >> decays;
        for (int d = 0; d < decays; d++) {
            double skip;
            for (int k = 0; k < 8; k++) f >> skip;
        }
        charge_[monval] = charge;
        baryon_[monval] = baryon;
        strange_[monval] = strange;
        if (baryon == 1) {
            charge_[-monval] = -charge;
            baryon_[-monval] = -baryon;
            strange_[-monval] = -strange;
        }
    }
    pdg_loaded_ = true;
}
