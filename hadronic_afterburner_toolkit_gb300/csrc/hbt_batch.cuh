// Device tables of the batched, culled, persistent pair binning
// (hbt_batch.cu), filled by the C ABI layer (hbt_capi.cu).
#pragma once

#include "hbt_engine.cuh"

namespace hbt {

// One particle list of a batch, as the caller passed it.
struct BatchList {
    const double *src[8];  // caller columns px py pz E (x y z t for same-event)
    long long n;           // particles
    long long off;         // first row in the sorted table
    long long tiles;       // ceil(n / 128)
    long long tile_off;    // first box of this list
    int ncols;             // 8 (same-event) or 4 (mixed-event)
    int pad;
};

// One job: same-event pairs of list la (kind 0) or la x lb (kind 1).
struct BatchJob {
    int kind, la, lb;
    int dev;             // engine descriptor (BatchDev::devs) when serving many analyses
    long long pair_off;  // first candidate tile pair of this job
    long long n_pairs;   // candidate tile pairs
    // cull thresholds of the job's analysis, Q = max(|lo|, |hi|) of its q
    // window: 2 Q^2 (1 + 1e-6) bounds q_x^2 + q_y^2 and Q (1 + 1e-6) bounds
    // |q_long| of any pair that can be binned
    double qt2_max;
    double ql_max;
    int boost;
    // 1: the job's analysis bins q_inv histograms: a tile pair is also kept
    // when its pairs may fall in the q_inv window (the LCMS q_long bound,
    // for tiles of one particle mass)
    int qinv;
    // ordered cap admission of several jobs at once: the job's first row in
    // the admission's row order (Caps::rows_total)
    long long row_base;
};

// Momentum-space box of a 128-particle tile.
struct Box {
    double x0, x1, y0, y1;  // p_x, p_y ranges
    double Y0, Y1;          // rapidity range
    double m0;              // smallest m_T = sqrt(E^2 - p_z^2)
    double z0, z1;          // p_z range
    double mm0, mm1;        // range of the mass squared E^2 - |p|^2
};

struct Item {
    unsigned job, ti, tj;
};

struct BatchDev {
    const BatchList *lists;
    const BatchJob *jobs;
    const long long *list_off;  // [n_lists] first particle of each list
    const long long *tile_off;  // [n_lists] first tile of each list
    const long long *pair_off;  // [n_jobs] first tile pair of each job
    int n_lists, n_jobs;
    long long total;        // particles in the batch
    long long total_tiles;  // tiles in the batch
    long long total_pairs;  // candidate tile pairs
    long long cap;          // row capacity of the sorted table
    double *table;          // [8][cap] sorted particle table
    unsigned *orig;         // [cap] each row's position in the caller's list
    unsigned long long *keys_in, *keys_out;
    unsigned *vals_in, *vals_out;
    void *sort_temp;
    size_t sort_temp_bytes;
    Box *boxes;
    Item *items;          // same-event queue, then the mixed-event queue
    unsigned same_cap;    // candidate same-event tile pairs
    unsigned mixed_cap;   // candidate mixed-event tile pairs
    unsigned *n_items;    // [2] culled queue lengths (same, mixed)
    unsigned *item_next;  // [2] persistent-kernel cursors
    // Same-event queue order by momentum-space region (order_items): k_cull
    // writes each kept item's region key and position, a radix sort orders
    // the positions by key, and the same-event kernel takes items in that
    // order, so the CTAs running at any time update few histogram slots.
    int order_items;
    unsigned *item_key_in, *item_key_out, *item_pos_in, *item_pos_out;
    void *item_sort_temp;
    size_t item_sort_temp_bytes;
    // cell sizes of the sort key
    double p_extent, inv_cell_pt, y_extent, inv_cell_y;
    // Several analyses in one launch (the serving loop): each job's engine
    // descriptor (grid, screen constants, histograms) is devs[job.dev];
    // nullptr: every job belongs to the launch's own descriptor.
    const Device *devs;
    int n_devs;
};

int persistent_blocks_per_sm();
size_t batch_sort_temp_bytes(long long cap);
// Scratch bytes of the same-event queue's region sort for n items.
size_t item_sort_temp_bytes(long long n);
// Sort, box, cull and bin one batch.  chunk > 0 splits the FP32-weight
// form's same-event queue into chunks of that many items with a merge of
// the FP32 partials after each: of `d` for a one-analysis batch, of every
// host_devs[k] (the host copies of b.devs) for a batch of many analyses.
// marks (optional, 4 events): recorded before and after the same-event
// kernels (with their merges) and before and after the mixed-event kernel.
// mode: MODE_FAST bins every pair; MODE_COUNT / MODE_ORDER run one pass of
// ordered cap admission over the batch (d.caps; rows are positions in the
// callers' lists).
cudaError_t run_batch(const Device &d, const BatchDev &b, int grid, unsigned chunk,
                      const Device *host_devs, int n_host_devs, cudaStream_t st,
                      cudaEvent_t *marks = nullptr, int mode = MODE_FAST);

}  // namespace hbt
