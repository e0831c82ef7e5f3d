#include "SampleSource.h"
#include "TextNumbers.h"

#include <sys/stat.h>

#include <algorithm>
#include <atomic>
#include <charconv>
#include <condition_variable>
#include <cstdio>
#include <deque>
#include <mutex>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <stdexcept>
#include <thread>

#ifdef HBT_HAVE_ZLIB
#include <zlib.h>
#endif

namespace hbt {

namespace {

const char *kBadParticle = "particleSamples: truncated or malformed particle line";
const char *kBadOscar = "particleSamples: truncated or malformed OSCAR line";
// zlib reports a gzip stream that ends before its trailer as Z_BUF_ERROR once
// the data it could inflate is used up; the reference reads on as if the
// file ended there.  Here that is an error.
const char *kTruncatedGz = "particleSamples: gzip stream ends early (truncated file)";

#ifdef HBT_HAVE_ZLIB
void check_gz_end(void *gzf) {
    int errnum = Z_OK;
    gzerror(static_cast<gzFile>(gzf), &errnum);
    if (errnum == Z_BUF_ERROR) throw std::runtime_error(kTruncatedGz);
}
#endif

// Parses `count` numbers separated by blanks from a NUL-terminated line;
// returns how many were read (the reference's readers parse line by line).
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

// Fills one particle from the numbers of its line (reference column order).
void set_particle(int mode, const double *v, particle_info &p) {
    std::memset(&p, 0, sizeof(p));
    if (mode == 10) {
        // monval mass t x y z E px py pz
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
}

int header_count(int mode, const std::string &head) {
    if (mode == 10) return std::atoi(head.c_str());
    std::istringstream hs(head);
    int event_id = 0, n_particle = 0;
    hs >> event_id >> n_particle;
    return n_particle;
}

// ---------------------------------------------------------------- line source

// Line reader over a plain or gzip-compressed text file.  next() returns the
// line without its '\n'; eof() is true once a read ran into the end of the
// file, which is the condition the reference's readers test after reading an
// event header (gzeof / ifstream::eof).
class LineSampleSource : public SampleSource {
  public:
    LineSampleSource(const std::string &path, bool gz, int mode) : gz_(gz), mode_(mode) {
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
        if (ok_ && mode_ == 0)
            for (int k = 0; k < 3; k++) next();  // OSCAR file header
    }
    ~LineSampleSource() override {
#ifdef HBT_HAVE_ZLIB
        if (gzf_) gzclose(static_cast<gzFile>(gzf_));
#else
        if (pipe_) pclose(pipe_);
#endif
    }
    bool ok() const override { return ok_; }
    bool eof() const override { return eof_; }
    long long text_bytes() const override { return bytes_; }

    int read_buffer(long event_buffer_size, EventList &out) override {
        out.clear();
        long num_particles = 0;
        double v[11];
        const int ncol = mode_ == 10 ? 10 : 11;
        while (num_particles < event_buffer_size) {
            const std::string head = next();
            if (eof()) break;
            const int n_particle = header_count(mode_, head);
            out.emplace_back();
            std::vector<particle_info> &ev = out.back();
            ev.reserve(n_particle);
            for (int k = 0; k < n_particle; k++) {
                const std::string line = next();
                if (parse_numbers(line.c_str(), v, ncol) != ncol)
                    throw std::runtime_error(mode_ == 10 ? kBadParticle : kBadOscar);
                particle_info p;
                set_particle(mode_, v, p);
                ev.push_back(p);
            }
            num_particles += n_particle;
        }
        return static_cast<int>(out.size());
    }

  private:
    std::string next() {
        std::string line = next_raw();
        bytes_ += static_cast<long long>(line.size()) + 1;
        return line;
    }

    std::string next_raw() {
        std::string line;
        if (!gz_) {
            if (!std::getline(fs_, line))
                eof_ = true;
            else if (fs_.eof())
                eof_ = true;
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
#ifdef HBT_HAVE_ZLIB
                check_gz_end(gzf_);
#endif
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
#ifdef HBT_HAVE_ZLIB
                check_gz_end(gzf_);
#endif
                eof_ = true;
                return line;
            }
        }
    }

    bool gz_;
    int mode_;
    bool ok_ = false;
    bool eof_ = false;
    long long bytes_ = 0;
    std::ifstream fs_;
    void *gzf_ = nullptr;
    FILE *pipe_ = nullptr;
    std::vector<char> buf_;
};

// --------------------------------------------------------------- block source

// Decompressed bytes of a plain or gzip file, read in large blocks.
class ByteSource {
  public:
    ByteSource(const std::string &path, bool gz) : gz_(gz) {
        if (gz_) {
#ifdef HBT_HAVE_ZLIB
            gzf_ = gzopen(path.c_str(), "rb");
            ok_ = gzf_ != nullptr;
            if (ok_) gzbuffer(static_cast<gzFile>(gzf_), 1 << 22);
#else
            const std::string cmd = "gzip -dc '" + path + "'";
            fp_ = popen(cmd.c_str(), "r");
            std::ifstream probe(path.c_str());
            ok_ = fp_ != nullptr && probe.good();
            piped_ = true;
#endif
        } else {
            fp_ = fopen(path.c_str(), "rb");
            ok_ = fp_ != nullptr;
        }
    }
    ~ByteSource() {
#ifdef HBT_HAVE_ZLIB
        if (gzf_) gzclose(static_cast<gzFile>(gzf_));
#endif
        if (fp_) {
            if (piped_)
                pclose(fp_);
            else
                fclose(fp_);
        }
    }
    bool ok() const { return ok_; }
    // Up to n bytes; 0 at the end of the data.
    size_t read(char *dst, size_t n) {
#ifdef HBT_HAVE_ZLIB
        if (gzf_) {
            const int got = gzread(static_cast<gzFile>(gzf_), dst, static_cast<unsigned>(n));
            if (got < 0) throw std::runtime_error("particleSamples: gzip read error");
            if (got == 0) check_gz_end(gzf_);
            return static_cast<size_t>(got);
        }
#endif
        return fp_ ? fread(dst, 1, n, fp_) : 0;
    }

  private:
    bool gz_;
    bool ok_ = false;
    bool piped_ = false;
    void *gzf_ = nullptr;
    FILE *fp_ = nullptr;
};

// Inflates ahead on a thread of its own: blocks of decompressed bytes wait
// in a short queue, so inflating overlaps with indexing and parsing.
class PrefetchSource {
  public:
    PrefetchSource(const std::string &path, bool gz, size_t block)
        : src_(path, gz), block_(block) {
        if (src_.ok()) worker_ = std::thread([this] { run(); });
    }
    ~PrefetchSource() {
        {
            std::lock_guard<std::mutex> lk(mu_);
            stop_ = true;
        }
        cv_.notify_all();
        if (worker_.joinable()) worker_.join();
    }
    bool ok() const { return src_.ok(); }
    // Next block (empty at the end of the data); rethrows a read error.
    std::vector<char> next() {
        std::unique_lock<std::mutex> lk(mu_);
        cv_.wait(lk, [&] { return !q_.empty() || done_; });
        if (!q_.empty()) {
            std::vector<char> b = std::move(q_.front());
            q_.pop_front();
            cv_.notify_all();
            return b;
        }
        if (!err_.empty()) throw std::runtime_error(err_);
        return std::vector<char>();
    }

  private:
    void run() {
        for (;;) {
            std::vector<char> b(block_);
            size_t got = 0;
            std::string err;
            try {
                got = src_.read(b.data(), block_);
            } catch (const std::exception &e) {
                err = e.what();
            }
            std::unique_lock<std::mutex> lk(mu_);
            if (got == 0 || !err.empty()) {
                err_ = err;
                done_ = true;
                cv_.notify_all();
                return;
            }
            b.resize(got);
            cv_.wait(lk, [&] { return q_.size() < 3 || stop_; });
            if (stop_) return;
            q_.push_back(std::move(b));
            cv_.notify_all();
        }
    }

    ByteSource src_;
    size_t block_;
    std::thread worker_;
    std::mutex mu_;
    std::condition_variable cv_;
    std::deque<std::vector<char>> q_;
    bool done_ = false, stop_ = false;
    std::string err_;
};

// Binary sidecar of a sample file: the events in reading order (the header
// count, then one record per particle), an end marker and whether the text
// ran into the end of the file inside the last event, so that a replay
// reproduces the text reader's buffers and end-of-file exactly.  The header
// records the source file's size and modification time; a cache that does
// not match them is ignored.
struct CacheRecord {
    int32_t monval, pad;
    double mass, t, x, y, z, E, px, py, pz;
};
const char kCacheMagic[8] = {'H', 'B', 'T', 'S', 'M', 'P', '0', '1'};
const int64_t kCacheEnd = INT64_MIN;

struct CacheHeader {
    char magic[8];
    int32_t mode, version;
    int64_t src_size, src_mtime_ns;
};

bool source_stamp(const std::string &path, int64_t &size, int64_t &mtime_ns) {
    struct stat st;
    if (stat(path.c_str(), &st) != 0) return false;
    size = static_cast<int64_t>(st.st_size);
    mtime_ns = static_cast<int64_t>(st.st_mtim.tv_sec) * 1000000000ll + st.st_mtim.tv_nsec;
    return true;
}

// Writes the sidecar while the text is read; renamed into place only once
// the whole file was read without error.
class CacheWriter {
  public:
    CacheWriter(const std::string &src, const std::string &cache, int mode)
        : cache_(cache), tmp_(cache + ".tmp") {
        CacheHeader h = {};
        memcpy(h.magic, kCacheMagic, 8);
        h.mode = mode;
        h.version = 1;
        if (!source_stamp(src, h.src_size, h.src_mtime_ns)) return;
        f_ = fopen(tmp_.c_str(), "wb");
        if (f_ && fwrite(&h, sizeof(h), 1, f_) != 1) fail();
    }
    ~CacheWriter() {
        if (f_) {  // not finished: drop the partial file
            fclose(f_);
            std::remove(tmp_.c_str());
        }
    }
    void add(const EventList &out, const std::vector<int> &counts) {
        if (!f_) return;
        std::vector<CacheRecord> rec;
        for (size_t e = 0; e < out.size(); e++) {
            const int64_t n = counts[e];
            if (fwrite(&n, sizeof(n), 1, f_) != 1) return fail();
            rec.resize(out[e].size());
            for (size_t k = 0; k < out[e].size(); k++) {
                const particle_info &p = out[e][k];
                rec[k] = CacheRecord{p.monval, 0, p.mass, p.t, p.x, p.y, p.z, p.E, p.px, p.py, p.pz};
            }
            if (!rec.empty() && fwrite(rec.data(), sizeof(CacheRecord), rec.size(), f_) != rec.size())
                return fail();
        }
    }
    void finish(bool eof_in_last_event) {
        if (!f_) return;
        const int64_t end = kCacheEnd;
        const int32_t flag = eof_in_last_event ? 1 : 0;
        const bool ok = fwrite(&end, sizeof(end), 1, f_) == 1 && fwrite(&flag, sizeof(flag), 1, f_) == 1;
        fclose(f_);
        f_ = nullptr;
        if (!ok || std::rename(tmp_.c_str(), cache_.c_str()) != 0) std::remove(tmp_.c_str());
    }

  private:
    void fail() {
        fclose(f_);
        f_ = nullptr;
        std::remove(tmp_.c_str());
    }
    std::string cache_, tmp_;
    FILE *f_ = nullptr;
};

class BlockSampleSource : public SampleSource {
  public:
    BlockSampleSource(const std::string &path, bool gz, int mode, int threads,
                      const std::string &cache)
        : src_(path, gz, kBlock), mode_(mode), threads_(threads) {
        if (!cache.empty() && src_.ok()) writer_.reset(new CacheWriter(path, cache, mode));
        win_.assign(kBlock + 1, '\0');
        if (src_.ok() && mode_ == 0)
            for (int k = 0; k < 3; k++) {  // OSCAR file header
                size_t b, e;
                next_line(b, e);
            }
    }
    bool ok() const override { return src_.ok(); }
    bool eof() const override { return eof_; }
    long long text_bytes() const override { return consumed_ + static_cast<long long>(pos_); }

    int read_buffer(long event_buffer_size, EventList &out) override {
        compact();
        out.clear();
        lines_.clear();
        long num_particles = 0;
        const int ncol = mode_ == 10 ? 10 : 11;
        // index the buffer's lines (offsets into the window)
        std::vector<long> first;
        std::vector<int> counts;
        bool eof_in_event = false;
        while (num_particles < event_buffer_size) {
            size_t b, e;
            next_line(b, e);
            if (eof()) break;
            const int n_particle = header_count(mode_, std::string(&win_[b], e - b));
            out.emplace_back();
            out.back().reserve(n_particle);
            first.push_back(static_cast<long>(lines_.size()));
            counts.push_back(n_particle);
            for (int k = 0; k < n_particle; k++) {
                next_line(b, e);
                lines_.push_back({b, e});
            }
            eof_in_event = eof();
            num_particles += n_particle;
        }
        // place every particle, then parse on all threads
        std::vector<particle_info *> dst(lines_.size());
        for (size_t ev = 0; ev < out.size(); ev++) {
            const long n = (ev + 1 < first.size() ? first[ev + 1] : (long)lines_.size()) - first[ev];
            out[ev].resize(static_cast<size_t>(n));
            for (long k = 0; k < n; k++) dst[first[ev] + k] = &out[ev][k];
        }
        std::atomic<bool> bad(false);
        const char *base = win_.data();
        parallel_ranges(static_cast<long>(lines_.size()), threads_, 4096,
                        [&](long lo, long hi) {
                            double v[11];
                            for (long i = lo; i < hi; i++) {
                                const Span &s = lines_[i];
                                if (parse_span(base + s.b, base + s.e, v, ncol) != ncol) {
                                    bad = true;
                                    return;
                                }
                                set_particle(mode_, v, *dst[i]);
                            }
                        });
        if (bad) throw std::runtime_error(mode_ == 10 ? kBadParticle : kBadOscar);
        if (writer_) {
            writer_->add(out, counts);
            if (eof()) {
                writer_->finish(eof_in_event);
                writer_.reset();
            }
        }
        return static_cast<int>(out.size());
    }

  private:
    static const size_t kBlock = 8u << 20;
    struct Span {
        size_t b, e;
    };

    // Appends the next block of decompressed bytes; false at the end.
    bool fill() {
        if (src_eof_) return false;
        const std::vector<char> blk = src_.next();
        if (blk.empty()) {
            src_eof_ = true;
            return false;
        }
        if (win_.size() < end_ + blk.size() + 1)
            win_.resize(std::max(win_.size() * 2, end_ + blk.size() + 1));
        memcpy(&win_[end_], blk.data(), blk.size());
        end_ += blk.size();
        win_[end_] = '\0';
        return true;
    }

    // Drops the bytes already consumed (only between buffers, so that the
    // offsets of a buffer's lines stay valid while it is read).
    void compact() {
        if (pos_ == 0) return;
        consumed_ += static_cast<long long>(pos_);
        memmove(&win_[0], &win_[pos_], end_ - pos_);
        end_ -= pos_;
        pos_ = 0;
        win_[end_] = '\0';
    }

    // The next line [b, e) without its '\n'; a line that runs into the end
    // of the file sets eof (the line reader's rule).
    void next_line(size_t &b, size_t &e) {
        b = pos_;
        size_t scan = pos_;
        for (;;) {
            const void *nl = scan < end_ ? memchr(&win_[scan], '\n', end_ - scan) : nullptr;
            if (nl) {
                e = static_cast<size_t>(static_cast<const char *>(nl) - win_.data());
                pos_ = e + 1;
                return;
            }
            scan = end_;
            if (!fill()) {
                e = end_;
                pos_ = end_;
                eof_ = true;
                return;
            }
        }
    }

    PrefetchSource src_;
    int mode_, threads_;
    std::unique_ptr<CacheWriter> writer_;
    std::vector<char> win_;
    size_t pos_ = 0, end_ = 0;
    long long consumed_ = 0;  // bytes dropped from the window
    bool src_eof_ = false, eof_ = false;
    std::vector<Span> lines_;
};

// Replays a sidecar written by CacheWriter with the buffer rule.
class CacheSampleSource : public SampleSource {
  public:
    explicit CacheSampleSource(FILE *f) : f_(f) {}
    ~CacheSampleSource() override {
        if (f_) fclose(f_);
    }
    bool ok() const override { return f_ != nullptr; }
    bool eof() const override { return eof_; }
    long long text_bytes() const override { return bytes_; }

    int read_buffer(long event_buffer_size, EventList &out) override {
        out.clear();
        long num_particles = 0;
        std::vector<CacheRecord> rec;
        while (num_particles < event_buffer_size) {
            if (!peek()) throw std::runtime_error("particleSamples: truncated sample cache");
            if (next_n_ == kCacheEnd) {
                eof_ = true;
                break;
            }
            const int n_particle = static_cast<int>(next_n_);
            have_n_ = false;
            out.emplace_back();
            std::vector<particle_info> &ev = out.back();
            ev.reserve(n_particle);
            if (n_particle > 0) {
                rec.resize(n_particle);
                if (fread(rec.data(), sizeof(CacheRecord), rec.size(), f_) != rec.size())
                    throw std::runtime_error("particleSamples: truncated sample cache");
                bytes_ += static_cast<long long>(rec.size() * sizeof(CacheRecord));
                ev.resize(n_particle);
                for (int k = 0; k < n_particle; k++) {
                    particle_info &p = ev[k];
                    std::memset(&p, 0, sizeof(p));
                    const CacheRecord &r = rec[k];
                    p.monval = r.monval;
                    p.mass = r.mass;
                    p.t = r.t;
                    p.x = r.x;
                    p.y = r.y;
                    p.z = r.z;
                    p.E = r.E;
                    p.px = r.px;
                    p.py = r.py;
                    p.pz = r.pz;
                }
            }
            num_particles += n_particle;
            // the text ran into its end inside this (last) event
            if (!peek()) throw std::runtime_error("particleSamples: truncated sample cache");
            if (next_n_ == kCacheEnd && eof_in_last_) eof_ = true;
        }
        return static_cast<int>(out.size());
    }

  private:
    // Reads the next event header (or the end marker and its flag).
    bool peek() {
        if (have_n_) return true;
        if (fread(&next_n_, sizeof(next_n_), 1, f_) != 1) return false;
        bytes_ += sizeof(next_n_);
        if (next_n_ == kCacheEnd) {
            int32_t flag = 0;
            if (fread(&flag, sizeof(flag), 1, f_) != 1) return false;
            eof_in_last_ = flag != 0;
        }
        have_n_ = true;
        return true;
    }

    FILE *f_;
    bool eof_ = false, have_n_ = false, eof_in_last_ = false;
    int64_t next_n_ = 0;
    long long bytes_ = 0;
};

}  // namespace

std::unique_ptr<SampleSource> make_cached_source(const std::string &path, bool gz, int mode,
                                                 int threads) {
    const std::string cache = path + ".hbtcache";
    int64_t size = 0, mtime = 0;
    if (source_stamp(path, size, mtime)) {
        FILE *f = fopen(cache.c_str(), "rb");
        if (f) {
            CacheHeader h;
            if (fread(&h, sizeof(h), 1, f) == 1 && memcmp(h.magic, kCacheMagic, 8) == 0 &&
                h.mode == mode && h.version == 1 && h.src_size == size && h.src_mtime_ns == mtime)
                return std::unique_ptr<SampleSource>(new CacheSampleSource(f));
            fclose(f);
        }
    }
    return std::unique_ptr<SampleSource>(new BlockSampleSource(path, gz, mode, threads, cache));
}

void parallel_ranges(long n, int threads, long min_per_thread,
                     const std::function<void(long, long)> &fn) {
    if (n <= 0) return;
    int t = threads > 0 ? threads : static_cast<int>(std::thread::hardware_concurrency());
    if (t < 1) t = 1;
    t = static_cast<int>(std::min<long>(t, std::max<long>(1, n / std::max<long>(1, min_per_thread))));
    if (t == 1) {
        fn(0, n);
        return;
    }
    std::vector<std::thread> pool;
    const long step = (n + t - 1) / t;
    for (int k = 1; k < t; k++) {
        const long lo = k * step, hi = std::min(n, lo + step);
        if (lo < hi) pool.emplace_back(fn, lo, hi);
    }
    fn(0, std::min(n, step));
    for (auto &th : pool) th.join();
}

std::unique_ptr<SampleSource> make_line_source(const std::string &path, bool gz, int mode) {
    return std::unique_ptr<SampleSource>(new LineSampleSource(path, gz, mode));
}

std::unique_ptr<SampleSource> make_block_source(const std::string &path, bool gz, int mode,
                                                int threads) {
    return std::unique_ptr<SampleSource>(new BlockSampleSource(path, gz, mode, threads, ""));
}

}  // namespace hbt
