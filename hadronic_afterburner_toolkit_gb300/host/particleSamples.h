// Event buffers of the particle-of-interest for the HBT analysis.
//
// Source-compatible subset of the reference's particleSamples
// (src/particleSamples.{h,cpp}) for the HBT path:
//  - read_in_mode 10 (iSS gzip text, results/particle_samples.gz) and
//    read_in_mode 0 (OSCAR text, results/OSCAR.DAT), plus the
//    *_mixed_event files when read_in_real_mixed_events = 1;
//  - buffering: whole events are read until the particle count reaches
//    event_buffer_size (particleSamples.cpp:1256-1283, :689-712);
//  - rapidity_shift boost of E and pz (:442-468), on all host threads;
//  - particle_monval filter (:1329-1346): a Monte-Carlo number, or the
//    class codes 9999 / +-9998 / +-9997 / +-9996 (charged, charge sign,
//    baryon sign, strangeness sign) looked up in EOS/pdg.dat;
//  - the balance-function species lists (:1300-1330, :1370-1460, :538-551).
// Other reader modes (UrQMD, JAM, SMASH, iSS binary) and resonance decays
// are not part of this library; asking for them throws.
#pragma once

#include <cstdio>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "ParameterReader.h"
#include "Random.h"
#include "SampleSource.h"
#include "particle_info.h"

class particleSamples {
  public:
    particleSamples(ParameterReader &paraRdr, std::string path,
                    std::shared_ptr<RandomUtil::Random> ran_gen);
    ~particleSamples();

    void read_in_particle_samples_and_filter();
    void read_in_particle_samples_mixed_event_and_filter();
    int read_in_particle_samples();
    int read_in_particle_samples_mixed_event();

    bool end_of_file() const;
    bool end_of_file_mixed_event() const;
    // Particles of the last buffer read, before the species filter (same
    // events plus a separate mixed pool), and text bytes read so far.
    long long last_buffer_particles() const;
    long long text_bytes() const;
    int get_event_buffer_size() const { return event_buffer_size_; }

    int get_number_of_events() const { return static_cast<int>(list_->size()); }
    int get_number_of_mixed_events() const { return static_cast<int>(mixed_list_->size()); }
    int get_number_of_particles(int event_id) const {
        return static_cast<int>((*list_)[event_id].size());
    }
    int get_number_of_particles_mixed_event(int event_id) const {
        return static_cast<int>((*mixed_list_)[event_id].size());
    }
    particle_info get_particle(int event_id, int part_id) const {
        return (*list_)[event_id][part_id];
    }
    particle_info get_particle_from_mixed_event(int event_id, int part_id) const {
        return (*mixed_list_)[event_id][part_id];
    }
    // Direct, copy-free access used by the HBT gather.
    const std::vector<particle_info> &event(int event_id) const { return (*list_)[event_id]; }
    const std::vector<particle_info> &mixed_event(int event_id) const {
        return (*mixed_list_)[event_id];
    }

    // Balance-function species lists (analyze_balance_function = 1; the
    // reference's get_balance_function_particle_list_*): s = 0 a, 1 abar,
    // 2 b, 3 bbar with a = particle_alpha, b = particle_beta, abar = -a,
    // bbar = -b; the mixed-event lists come from the mixed-event pool (the
    // buffer itself when read_in_real_mixed_events = 0).
    const hbt::EventList &balance_function_list(int s) const { return bf_[s]; }
    const hbt::EventList &balance_function_list_mixed_event(int s) const {
        return read_mixed_events_ ? bf_mixed_[s] : bf_[s];
    }

  private:
    typedef hbt::EventList EventList;

    const ParameterReader paraRdr_;
    const std::string path_;
    int echo_level_;
    int event_buffer_size_;
    int read_in_mode_;
    double rap_shift_;
    bool read_mixed_events_;
    int particle_monval_;

    // text sources: the block reader (parallel parse, key hbt_fast_reader =
    // 1, the default; with hbt_binary_cache = 1 it writes and later replays
    // a binary sidecar of the file) or the line-by-line reader
    // (hbt_fast_reader = 0)
    std::unique_ptr<hbt::SampleSource> in_, in_mixed_;
    EventList full_, full_mixed_, filtered_, filtered_mixed_;
    EventList *list_, *mixed_list_;

    // Monte-Carlo number -> (charge, baryon, strange) from EOS/pdg.dat,
    // loaded on first use by a class code.
    std::map<int, int> charge_, baryon_, strange_;
    bool pdg_loaded_ = false;
    int reader_threads_ = 0;  // host threads of the reader and boost (0: all)
    bool analyze_bf_ = false;
    int bf_monval_[4] = {0, 0, 0, 0};
    EventList bf_[4], bf_mixed_[4];

    void boost(EventList &evs) const;
    void filter(const EventList &full, EventList &out);
    void filter_code(int poi, const EventList &full, EventList &out);
    bool pick(int monval) { return pick_code(particle_monval_, monval); }
    bool pick_code(int poi, int monval);
    void load_pdg();
};
