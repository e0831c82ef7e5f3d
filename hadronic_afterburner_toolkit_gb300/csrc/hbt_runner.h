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

    // Runs the jobs of one analysis: every job bins into `d`.  Returns
    // false and sets `err` on failure.  Allocates scratch on first use and
    // when a batch outgrows it.
    bool run(const std::vector<FastJob> &jobs, const Device &d, int grid, unsigned chunk,
             cudaStream_t st, std::string &err);

    // Runs jobs of several analyses in one launch: job.dev indexes `devs`,
    // whose entries must share azimuthal_flag, long_comoving_boost and
    // precision (they select the kernel).  The FP32-weight partials of
    // every analysis are merged after each chunk of `chunk` same-event
    // items and at the end.
    bool run_multi(const std::vector<FastJob> &jobs, const std::vector<Device> &devs, int grid,
                   unsigned chunk, cudaStream_t st, std::string &err);

    // Candidate and kept tile pairs of the last batch (kept read lazily).
    long long last_tile_pairs() const { return last_pairs_; }

  private:
    struct Buf {
        void *p = nullptr;
        size_t bytes = 0;
    };
    bool grow(Buf &b, size_t bytes, std::string &err);
    bool run_impl(const std::vector<FastJob> &jobs, const Device &d, const Device *devs_dev,
                  const Device *devs_host, int n_devs, int grid, unsigned chunk, cudaStream_t st,
                  std::string &err);
    Buf lists_, jobs_, offs_, table_, keys_, vals_, sort_temp_, boxes_, items_, counters_, devs_;
    long long last_pairs_ = 0;
};

}  // namespace hbt
