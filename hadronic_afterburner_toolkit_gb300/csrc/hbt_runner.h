// Host side of the batched, culled, persistent pair binning: builds the
// device tables of a batch (lists, jobs, offsets), owns the scratch it
// needs (sorted particle table, sort buffers, tile boxes, work queues) and
// launches hbt_batch.cu's pipeline.  Used by one engine context
// (hbt_bin_batch*, single fast launches) and by the serving loop, which
// runs jobs of many analyses in one launch.
#pragma once

#include <string>
#include <vector>

#include "hbt_batch.cuh"

namespace hbt {

// One job of a batch, device columns.
struct FastJob {
    int kind;            // 0 same-event (a), 1 mixed-event (a x b)
    long long na, nb;
    const double *a[8];  // px py pz E (x y z t for same-event)
    const double *b[4];  // px py pz E
    int dev;             // index of the analysis (serving), 0 otherwise
    double q_window;     // Q = max(|lo|, |hi|) of the analysis' q window
    int boost;           // long_comoving_boost of the analysis
};

class BatchRunner {
  public:
    BatchRunner() = default;
    ~BatchRunner();
    BatchRunner(const BatchRunner &) = delete;
    BatchRunner &operator=(const BatchRunner &) = delete;

    // Runs the jobs: with devs == nullptr every job uses `d` (one analysis;
    // the FP32-weight partials are merged here); otherwise job.dev indexes
    // the device array devs of n_devs descriptors and the caller merges.
    // Returns false and sets `err` on failure.  Allocates scratch on first
    // use and when a batch outgrows it.
    bool run(const std::vector<FastJob> &jobs, const Device &d, const Device *devs, int n_devs,
             int grid, unsigned chunk, cudaStream_t st, std::string &err);

    // Candidate and kept tile pairs of the last batch (kept read lazily).
    long long last_tile_pairs() const { return last_pairs_; }

  private:
    struct Buf {
        void *p = nullptr;
        size_t bytes = 0;
    };
    bool grow(Buf &b, size_t bytes, std::string &err);
    Buf lists_, jobs_, offs_, table_, keys_, vals_, sort_temp_, boxes_, items_, counters_;
    long long last_pairs_ = 0;
};

}  // namespace hbt
