// Event-buffer sources of particleSamples: the text formats of read_in_mode
// 10 (iSS gzip text, "n" header lines then "monval mass t x y z E px py pz")
// and read_in_mode 0 (OSCAR text, 3 file header lines, "event n" header
// lines then "index monval px py pz E mass x y z t").
//
// Both sources apply the reference's buffer rule (particleSamples.cpp
// :1247-1286 for mode 10, :680-714 for mode 0): whole events are read until
// the particle count reaches the buffer size, and a header line read that
// runs into the end of the file ends the input.
//
//  - LineSampleSource reads line by line and parses with strtod, as the
//    reference's readers do line by line.
//  - BlockSampleSource inflates the file in large blocks on a thread of its
//    own, indexes the lines of a whole buffer, then parses the particle
//    lines on all host threads with std::from_chars (correctly rounded, like
//    strtod: the values are bit-identical) and fills the events in place.
//  - CacheSampleSource replays a binary sidecar (FP64 records) that a block
//    source wrote while reading the text through; a replay gives the same
//    buffers, particles and end-of-file as the text.
#pragma once

#include <functional>
#include <memory>
#include <string>
#include <vector>

#include "particle_info.h"

namespace hbt {

typedef std::vector<std::vector<particle_info>> EventList;

class SampleSource {
  public:
    virtual ~SampleSource() = default;
    virtual bool ok() const = 0;
    // True once a read ran into the end of the file.
    virtual bool eof() const = 0;
    // One buffer of whole events into `out`; returns the number of events.
    virtual int read_buffer(long event_buffer_size, EventList &out) = 0;
    // Bytes of (decompressed) text consumed so far.
    virtual long long text_bytes() const = 0;
};

// mode: 10 or 0; gz: the file is gzip-compressed; threads: parser threads
// of the block source (0: all host threads).
std::unique_ptr<SampleSource> make_line_source(const std::string &path, bool gz, int mode);
std::unique_ptr<SampleSource> make_block_source(const std::string &path, bool gz, int mode,
                                                int threads);
// The binary sidecar `path`.hbtcache when it matches the file (size and
// modification time), else a block source that writes it as the file is
// read through to its end.
std::unique_ptr<SampleSource> make_cached_source(const std::string &path, bool gz, int mode,
                                                 int threads);

// Runs fn(begin, end) over [0, n) split into contiguous ranges on up to
// `threads` host threads (0: all), inline when n is small.
void parallel_ranges(long n, int threads, long min_per_thread,
                     const std::function<void(long, long)> &fn);

}  // namespace hbt
