#include "particleSamples.h"

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <sstream>
#include <stdexcept>

#ifdef HBT_HAVE_ZLIB
#include <zlib.h>
#endif

namespace hbt {

// Line reader over a plain or gzip-compressed text file.  next() returns the
// line without its '\n'; eof() is true once a read ran into the end of the
// file, which is the condition the reference's readers test after reading an
// event header (gzeof / ifstream::eof).
class LineSource {
  public:
    LineSource(const std::string &path, bool gz) : gz_(gz) {
        if (gz_) {
#ifdef HBT_HAVE_ZLIB
            gzf_ = gzopen(path.c_str(), "rb");
            ok_ = gzf_ != nullptr;
            if (ok_) gzbuffer(static_cast<gzFile>(gzf_), 1 << 20);
#else
            const std::string cmd = "gzip -dc '" + path + "'";
            pipe_ = popen(cmd.c_str(), "r");
            std::ifstream probe(path.c_str());
            ok_ = pipe_ != nullptr && probe.good();
#endif
        } else {
            fs_.open(path.c_str());
            ok_ = fs_.is_open();
        }
        buf_.resize(1 << 16);
    }
    ~LineSource() {
#ifdef HBT_HAVE_ZLIB
        if (gzf_) gzclose(static_cast<gzFile>(gzf_));
#else
        if (pipe_) pclose(pipe_);
#endif
    }
    bool ok() const { return ok_; }
    bool eof() const { return eof_; }

    std::string next() {
        std::string line;
        if (!gz_) {
            if (!std::getline(fs_, line)) eof_ = true;
            else if (fs_.eof()) eof_ = true;
            return line;
        }
        for (;;) {
            char *got = nullptr;
#ifdef HBT_HAVE_ZLIB
            got = gzgets(static_cast<gzFile>(gzf_), &buf_[0], static_cast<int>(buf_.size()));
#else
            got = fgets(&buf_[0], static_cast<int>(buf_.size()), pipe_);
#endif
            if (!got) {
                eof_ = true;
                return line;
            }
            const size_t len = strlen(got);
            if (len > 0 && got[len - 1] == '\n') {
                line.append(got, len - 1);
                return line;
            }
            line.append(got, len);
            if (len + 1 < buf_.size()) {  // short read without newline: end of file
                eof_ = true;
                return line;
            }
        }
    }

  private:
    bool gz_;
    bool ok_ = false;
    bool eof_ = false;
    std::ifstream fs_;
    void *gzf_ = nullptr;
    FILE *pipe_ = nullptr;
    std::vector<char> buf_;
};

}  // namespace hbt

namespace {

// Parses `count` numbers separated by blanks; returns how many were read.
int parse_numbers(const char *s, double *out, int count) {
    int k = 0;
    char *end = nullptr;
    while (k < count) {
        const double v = strtod(s, &end);
        if (end == s) break;
        out[k++] = v;
        s = end;
    }
    return k;
}

}  // namespace

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
    if (paraRdr_.getVal("resonance_feed_down_flag") == 1 ||
        paraRdr_.getVal("resonance_weak_feed_down_flag") == 1)
        throw std::runtime_error("particleSamples: resonance decays are not part of this build");

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
                                 " is not supported by this build (0 and 10 are)");
    }
    in_.reset(new hbt::LineSource(file, gz));
    if (!in_->ok())
        throw std::runtime_error("particleSamples:: Error: input file: " + file + " can not open!");
    if (read_mixed_events_) {
        in_mixed_.reset(new hbt::LineSource(file_mixed, gz));
        if (!in_mixed_->ok())
            throw std::runtime_error("particleSamples:: Error: input file: " + file_mixed +
                                     " can not open!");
    }
    if (read_in_mode_ == 0) {  // OSCAR header
        for (int k = 0; k < 3; k++) {
            in_->next();
            if (in_mixed_) in_mixed_->next();
        }
    }
    list_ = &filtered_;
    mixed_list_ = read_mixed_events_ ? &filtered_mixed_ : &filtered_;
}

particleSamples::~particleSamples() = default;

bool particleSamples::end_of_file() const { return in_->eof(); }
bool particleSamples::end_of_file_mixed_event() const {
    return in_mixed_ ? in_mixed_->eof() : in_->eof();
}

// One buffer: whole events until the particle count reaches the buffer size
// (src/particleSamples.cpp:1247-1286 for mode 10, :680-714 for mode 0).
int particleSamples::read_buffer(hbt::LineSource &src, EventList &out) {
    out.clear();
    long num_particles = 0;
    double v[11];
    while (num_particles < event_buffer_size_) {
        const std::string head = src.next();
        if (src.eof()) break;
        int n_particle = 0;
        if (read_in_mode_ == 10) {
            n_particle = std::atoi(head.c_str());
        } else {
            std::istringstream hs(head);
            int event_id = 0;
            hs >> event_id >> n_particle;
        }
        out.emplace_back();
        std::vector<particle_info> &ev = out.back();
        ev.reserve(n_particle);
        for (int k = 0; k < n_particle; k++) {
            const std::string line = src.next();
            particle_info p;
            std::memset(&p, 0, sizeof(p));
            if (read_in_mode_ == 10) {
                // monval mass t x y z E px py pz
                if (parse_numbers(line.c_str(), v, 10) != 10)
                    throw std::runtime_error("particleSamples: truncated or malformed particle line");
                p.monval = static_cast<int>(v[0]);
                p.mass = v[1];
                p.t = v[2];
                p.x = v[3];
                p.y = v[4];
                p.z = v[5];
                p.E = v[6];
                p.px = v[7];
                p.py = v[8];
                p.pz = v[9];
            } else {
                // index monval px py pz E mass x y z t
                if (parse_numbers(line.c_str(), v, 11) != 11)
                    throw std::runtime_error("particleSamples: truncated or malformed OSCAR line");
                p.monval = static_cast<int>(v[1]);
                p.px = v[2];
                p.py = v[3];
                p.pz = v[4];
                p.E = v[5];
                p.mass = v[6];
                p.x = v[7];
                p.y = v[8];
                p.z = v[9];
                p.t = v[10];
            }
            ev.push_back(p);
        }
        num_particles += n_particle;
    }
    return static_cast<int>(out.size());
}

// particleSamples::boostParticles (src/particleSamples.cpp:442-468).
void particleSamples::boost(EventList &evs) const {
    const double ch = cosh(rap_shift_), sh = sinh(rap_shift_);
    for (auto &ev : evs)
        for (auto &p : ev) {
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
}

int particleSamples::read_in_particle_samples() {
    read_buffer(*in_, full_);
    boost(full_);
    return static_cast<int>(full_.size());
}

int particleSamples::read_in_particle_samples_mixed_event() {
    read_buffer(*in_mixed_, full_mixed_);
    boost(full_mixed_);
    return static_cast<int>(full_mixed_.size());
}

void particleSamples::read_in_particle_samples_and_filter() {
    read_in_particle_samples();
    filter(full_, filtered_);
}

void particleSamples::read_in_particle_samples_mixed_event_and_filter() {
    if (!read_mixed_events_) {
        mixed_list_ = &filtered_;
        return;
    }
    read_in_particle_samples_mixed_event();
    filter(full_mixed_, filtered_mixed_);
    mixed_list_ = &filtered_mixed_;
}

void particleSamples::filter(const EventList &full, EventList &out) {
    out.clear();
    out.resize(full.size());
    for (size_t e = 0; e < full.size(); e++)
        for (const auto &p : full[e])
            if (pick(p.monval)) out[e].push_back(p);
}

// decide_to_pick_OSCAR (src/particleSamples.cpp:625-678).
bool particleSamples::pick(int monval) {
    const int poi = particle_monval_;
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
