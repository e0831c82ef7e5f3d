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
    int qinv;            // 1: the analysis bins q_inv histograms (no cull)
    long long row_base;  // first row in a multi-job ordered admission (Caps::rows_total)
};

// Launch shape of a batch, chosen by hbt_set_tuning / hbt_autotune_batch.
struct Tuning {
    int grid = 0;            // persistent CTAs
    unsigned chunk = 0;      // FP32-weight form: same-event items between merges (0: no chunks)
    double cell_pt = 0.02;   // Morton cell of p_x, p_y (GeV)
    double cell_y = 0.05;    // Morton cell of rapidity
    bool graph = true;       // launch the pipeline as a CUDA graph
    bool time_kernels = false;  // record events around the persistent kernels
    bool order_items = false;   // same-event items in momentum-region order
};

class BatchRunner {
  public:
    BatchRunner() = default;
    ~BatchRunner();
    BatchRunner(const BatchRunner &) = delete;
    BatchRunner &operator=(const BatchRunner &) = delete;

    // Runs the jobs of one analysis: every job bins into `d`.  Returns
    // false and sets `err` on failure.  Allocates scratch on first use and
    // when a batch outgrows it.  mode: MODE_FAST, or one pass (MODE_COUNT,
    // MODE_ORDER) of ordered cap admission with d.caps.
    bool run(const std::vector<FastJob> &jobs, const Device &d, const Tuning &t, cudaStream_t st,
             std::string &err, int mode = MODE_FAST);

    // Runs jobs of several analyses in one launch: job.dev indexes `devs`,
    // whose entries must share azimuthal_flag, long_comoving_boost,
    // precision and invariant_radius_flag (they select the kernel).  The FP32-weight partials of
    // every analysis are merged after each chunk of `chunk` same-event
    // items and at the end.
    bool run_multi(const std::vector<FastJob> &jobs, const std::vector<Device> &devs,
                   const Tuning &t, cudaStream_t st, std::string &err);

    // Candidate tile pairs of the last batch.
    long long last_tile_pairs() const { return last_pairs_; }
    // Candidate and culled (kept) same-event and mixed-event tile pairs of
    // the last batch (reads the kept counts back: waits for the batch).
    bool tile_counts(long long &cand_same, long long &cand_mixed, long long &kept_same,
                     long long &kept_mixed);
    // Graph launches of the last batch: 1 a cached graph was re-launched,
    // 0 captured anew, -1 launched without a graph.
    int last_graph_reuse() const { return last_reuse_; }
    // Device time of the last timed batch's same-event kernels (with their
    // merges) and mixed-event kernel, ms (waits for them); false when the
    // last batch was not timed.
    bool kernel_times(float &same_ms, float &mixed_ms);

  private:
    struct Buf {
        void *p = nullptr;
        size_t bytes = 0;
    };
    bool grow(Buf &b, size_t bytes, std::string &err);
    bool run_impl(const std::vector<FastJob> &jobs, const Device &d, const Device *devs_dev,
                  const Device *devs_host, int n_devs, const Tuning &t, cudaStream_t st,
                  std::string &err, int mode);
    // Runs the device pipeline, through a cached CUDA graph when possible.
    cudaError_t launch(const Device &d, const BatchDev &b, const Device *devs_host, int n_devs,
                       const Tuning &t, cudaStream_t st, int mode);
    Buf lists_, jobs_, offs_, table_, keys_, vals_, sort_temp_, boxes_, items_, counters_, devs_;
    Buf item_order_, item_sort_temp_;
    long long last_pairs_ = 0, last_same_ = 0, last_mixed_ = 0;
    cudaStream_t last_stream_ = nullptr;
    int last_reuse_ = -1;
    // the cached graph and the launch arguments it was captured with; a
    // graph is captured when the same arguments come twice in a row
    cudaGraphExec_t exec_ = nullptr;
    std::vector<unsigned char> key_, last_key_;
    cudaEvent_t marks_[4] = {nullptr, nullptr, nullptr, nullptr};
    bool timed_ = false;
};

}  // namespace hbt
