/*
 * hbt_gpu.h - C ABI of the GB300 HBT pair-binning engine (libhbt_gpu.so).
 *
 * The engine owns the device-resident correlation histograms of one HBT
 * analysis and bins particle pairs into them with sm_103a CUDA kernels.  It
 * replaces the pair loops and the histogram storage of the reference's
 * HBT_correlation class (src/HBT_correlation.{h,cpp} of
 * chunshen1987/hadronic_afterburner_toolkit); the host side (parameter
 * reading, event buffering, rapidity gather, random partner selection and
 * rotation, output files) stays in C++ above this boundary.
 *
 * Conventions
 *  - Plain C types only.  Every entry point returns an hbt_status
 *    (HBT_OK == 0); hbt_last_error() describes the last failure.  Nothing
 *    calls exit() or throws across the boundary.
 *  - Host arrays passed in are read during the call only.  Device arrays
 *    (the *_dev entry points) must stay valid until the work is complete
 *    (hbt_sync).
 *  - Work is ordered on the context's CUDA stream.  A context is used by
 *    one host thread at a time.
 *  - Bin indices and pair counts are bit-exact against the reference's CPU
 *    path; the cos(q.dx) numerator and mean-q sums are FP64 sums whose
 *    order differs (relative difference of order 1e-15 per bin).
 */
#ifndef HBT_GPU_H
#define HBT_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum hbt_status {
    HBT_OK = 0,
    HBT_ERR_INVALID = 1,  /* bad argument or parameter */
    HBT_ERR_CUDA = 2,     /* a CUDA call failed */
    HBT_ERR_NOMEM = 3,    /* device or host allocation failed */
    HBT_ERR_TIMEOUT = 4,  /* hbt_sync budget ran out */
    HBT_ERR_DEVICE = 5,   /* a kernel raised its error flag */
    HBT_ERR_STATE = 6     /* call not valid in the context's current state */
} hbt_status;

/* Numerics of the weights and q sums. */
typedef enum hbt_precision {
    HBT_PRECISION_FP64 = 0, /* plain form: everything in FP64 */
    HBT_PRECISION_FP32W = 1, /* cos(q.dx) weight and q sums in FP32 partials,
                                merged into FP64 bins with Kahan compensation;
                                bins and counts stay exact */
    HBT_PRECISION_DF64 = 2   /* same-event weight and q sums computed in
                                double-float arithmetic (value = hi + lo, two
                                FP32 numbers) on the FP32 pipe and added to
                                the FP64 bins; bins and counts stay exact */
} hbt_precision;

/* The HBT keys of parameters.dat that shape the histograms
 * (HBT_correlation::HBT_correlation, src/HBT_correlation.cpp:16-143). */
typedef struct hbt_params {
    int32_t qnpts;                  /* "qnpts" */
    double q_min, q_max;            /* "q_min", "q_max" [GeV] */
    int32_t n_KT;                   /* "n_KT": number of K_T edges */
    double KT_min, KT_max;          /* "KT_min", "KT_max" [GeV] */
    int32_t n_Kphi;                 /* "n_Kphi" */
    int32_t azimuthal_flag;         /* "azimuthal_flag" */
    int32_t invariant_radius_flag;  /* "invariant_radius_flag" */
    int32_t long_comoving_boost;    /* "long_comoving_boost" */
    double needed_number_of_pairs;  /* "needed_number_of_pairs" (pair cap) */
    int32_t precision;              /* hbt_precision */
    /* Half-width (rad) of the zone around a K_phi bin edge inside which the
     * reference chain (the plain kernel, and pairs the screened kernels'
     * FP32 test cannot decide) hands a pair's azimuthal bin to the host's
     * C-library atan2 instead of the device's; 0 selects the default
     * (1e-13).  The screened kernels decide the other pairs' bins in FP32
     * with an error bound.  At most 65536 pairs are handed over per launch,
     * or per count pass of ordered cap admission (which covers all of a
     * batch's mixed-event jobs); more raise HBT_ERR_DEVICE, which only a
     * tolerance many orders above the default can reach. */
    double kphi_defer_tol;
    int32_t kernel; /* hbt_kernel */
} hbt_params;

/* Kernel family for pairs no cap can reject.  Both give the same bins and
 * counts; HBT_KERNEL_REFERENCE_CHAIN evaluates the reference's FP64 chain
 * for every pair and is kept as the plain baseline the screened form is
 * measured against. */
typedef enum hbt_kernel {
    HBT_KERNEL_SCREENED = 0,       /* lists sorted in momentum space, tile pairs
                                      that cannot bin culled, persistent kernel
                                      with FP32 screen + FP64 for binned pairs */
    HBT_KERNEL_REFERENCE_CHAIN = 1, /* FP64 reference chain on every pair */
    HBT_KERNEL_SCREENED_GRID = 2   /* FP32 screen, one CTA per tile pair, no
                                      sorting or culling */
} hbt_kernel;

typedef struct hbt_ctx hbt_ctx;

/* Structure-of-arrays particle lists, FP64. */
typedef struct hbt_soa8 {
    const double *px, *py, *pz, *E, *x, *y, *z, *t;
} hbt_soa8;
typedef struct hbt_soa4 {
    const double *px, *py, *pz, *E;
} hbt_soa4;

/* Totals kept by the engine. */
typedef struct hbt_stats {
    uint64_t pairs_same;      /* candidate same-event pairs, n(n-1)/2 summed */
    uint64_t pairs_mixed;     /* candidate mixed-event pairs, n1*n2 summed */
    uint64_t launches;        /* kernel launches issued */
    uint64_t ordered_passes;  /* launches that needed ordered cap admission */
    uint64_t deferred_kphi;   /* pairs whose K_phi bin was decided on the host */
    uint64_t anomalies;       /* pairs skipped: NaN LCMS component (K_perp == 0)
                                 or a K_T index outside [0, n_KT) */
    uint64_t graph_captures;  /* batched launches captured into a CUDA graph */
    uint64_t graph_replays;   /* batched launches that re-launched a cached graph */
    /* device time of the last batched launch's persistent kernels, ms, when
     * hbt_tuning.time_kernels is set (0 otherwise): the same-event kernels
     * with their FP32 merges, and the mixed-event kernel */
    double same_kernel_ms, mixed_kernel_ms;
    /* the last batched launch's 128 x 128 tile pairs: candidates and those
     * the momentum-space cull kept, same-event and mixed-event */
    uint64_t tiles_same, tiles_mixed, tiles_same_kept, tiles_mixed_kept;
} hbt_stats;

/* Creates a context on `device` and allocates the zeroed histograms
 * (replaces the histogram allocation of HBT_correlation::HBT_correlation,
 * src/HBT_correlation.cpp:16-143). */
hbt_status hbt_create(const hbt_params *params, int device, hbt_ctx **out);
void hbt_destroy(hbt_ctx *ctx);
const char *hbt_last_error(const hbt_ctx *ctx);

/* Uses a caller-owned cudaStream_t (NULL: the context's own stream). */
hbt_status hbt_set_stream(hbt_ctx *ctx, void *cuda_stream);

/* Event-plane reference angle for the K_phi bins of the next launches
 * (the psi_ref member set by calculate_flow_event_plane_angle,
 * src/HBT_correlation.cpp:233-249). */
hbt_status hbt_set_psi_ref(hbt_ctx *ctx, double psi_ref);

/* Zeroes histograms, pair counters and statistics. */
hbt_status hbt_reset(hbt_ctx *ctx);

/* Same-event pairs i < j of one gathered buffer, host arrays
 * (replaces the pair loop of HBT_correlation::combine_and_bin_particle_pairs,
 * src/HBT_correlation.cpp:282-461). */
hbt_status hbt_bin_same(hbt_ctx *ctx, int64_t n, const hbt_soa8 *list);

/* Mixed-event pairs list1 x list2 (list2 = the rotated partners), host
 * arrays (replaces the pair loop of
 * HBT_correlation::combine_and_bin_particle_pairs_mixed_events,
 * src/HBT_correlation.cpp:554-689). */
hbt_status hbt_bin_mixed(hbt_ctx *ctx, int64_t n1, const hbt_soa4 *list1,
                         int64_t n2, const hbt_soa4 *list2);

/* As above with device-resident arrays (inputs already in HBM). */
hbt_status hbt_bin_same_dev(hbt_ctx *ctx, int64_t n, const hbt_soa8 *list);
hbt_status hbt_bin_mixed_dev(hbt_ctx *ctx, int64_t n1, const hbt_soa4 *list1,
                             int64_t n2, const hbt_soa4 *list2);

/* One job of a batch: the same-event pairs of list a (kind 0, eight
 * columns), or the mixed-event pairs a x b (kind 1, columns px py pz E). */
typedef struct hbt_job {
    int32_t kind;
    int64_t na, nb;
    hbt_soa8 a, b;
} hbt_job;

/* Bins a batch of jobs in one persistent launch from a work queue of
 * (job, i-tile, j-tile) items - the pair loops of many
 * combine_and_bin_particle_pairs / _mixed_events calls at once
 * (src/HBT_correlation.cpp:282-461, :554-689).  The result equals calling
 * hbt_bin_same / hbt_bin_mixed for each job in order.  When a pair cap could
 * bind, the reference's admission order is kept: the same-event jobs are
 * admitted one by one, the mixed-event jobs together in their joint order
 * (one count and one order pass over all of them; the numerator and
 * denominator caps are separate, so the two kinds do not interact).
 * hbt_bin_batch takes host arrays, hbt_bin_batch_dev device arrays. */
hbt_status hbt_bin_batch(hbt_ctx *ctx, int32_t n_jobs, const hbt_job *jobs);
hbt_status hbt_bin_batch_dev(hbt_ctx *ctx, int32_t n_jobs, const hbt_job *jobs);

/* Launch shape of the batched path (HBT_KERNEL_SCREENED).  No counterpart
 * in the reference.  Every choice gives the same bins and counts; they
 * differ in speed only (and, for the FP32-weight form, merge_chunk bounds
 * how many pairs an FP32 partial accumulates). */
typedef struct hbt_tuning {
    int32_t blocks_per_sm;  /* persistent CTAs per SM, at most 8 (0: each kernel at
                               its occupancy limit) */
    double cell_pt;         /* sort cell of p_x and p_y in GeV (0: 0.02) */
    double cell_y;          /* sort cell of rapidity (0: 0.05) */
    int32_t merge_chunk;    /* FP32-weight form: same-event tile pairs between two
                               merges of the partials, <= 8192 (0: 8192; the
                               bound keeps the numerator within 1e-6 per pair) */
    int32_t use_graph;      /* 1: launch the sort-cull-bin pipeline as a CUDA graph,
                               captured when a batch of the same shape comes twice in
                               a row and re-launched while it repeats; 0: direct
                               launches */
    int32_t time_kernels;   /* 1: time the persistent kernels with CUDA events
                               (hbt_stats.same_kernel_ms / mixed_kernel_ms) */
    int32_t order_items;    /* 1 (default): take the same-event tile pairs in the
                               order of their momentum-space region (K_T and
                               azimuth of the tiles' mean momentum), so that the
                               CTAs running at any time update few histogram
                               slots (on the central workload 3.3x less DRAM
                               traffic); 0: in the order the cull found them.
                               The FP32-weight form always takes the cull's
                               order (its FP32 partials' bound needs the pairs of
                               a merge chunk spread over many bins) */
} hbt_tuning;

hbt_status hbt_set_tuning(hbt_ctx *ctx, const hbt_tuning *t);
hbt_status hbt_get_tuning(hbt_ctx *ctx, hbt_tuning *t);

/* Autotuner.  No counterpart in the reference.  Times candidate tunings
 * (sort cells, CTAs per SM, item order, merge chunk) on up to `max_pairs`
 * candidate pairs of the batch (device arrays, jobs taken in order; 0: 2e9) with
 * scratch histograms, keeps the fastest for this context and returns it
 * with its time.  The context's histograms are not touched. */
hbt_status hbt_autotune_batch(hbt_ctx *ctx, int32_t n_jobs, const hbt_job *jobs,
                              double max_pairs, hbt_tuning *best, double *best_ms);

/* Waits for the context's stream, polling up to timeout_us microseconds
 * (0: wait without limit).  Returns HBT_ERR_TIMEOUT if work is still
 * running, HBT_ERR_DEVICE if a kernel raised its error flag. */
hbt_status hbt_sync(hbt_ctx *ctx, uint64_t timeout_us);

/* Number of 3-D bins: n_slots * qnpts^3 with n_slots = n_KT, or
 * n_KT * n_Kphi when azimuthal_flag == 1.  Bin order [slot][iqout][iqside]
 * [iqlong], slot = iKT (* n_Kphi + iKphi). */
int64_t hbt_n_bins(const hbt_ctx *ctx);

/* Copies the histograms to host arrays of hbt_n_bins() doubles (any may be
 * NULL): numerator pair count, q_out / q_side / q_long sums, cos(q.dx)
 * numerator, denominator pair count.  These are the arrays the reference's
 * writer reads (correl_3d_num_count, q_out_mean, q_side_mean, q_long_mean,
 * correl_3d_num, correl_3d_denorm and their K_phi twins,
 * src/HBT_correlation.h:55-61). */
hbt_status hbt_read_hist(hbt_ctx *ctx, double *num_count, double *q_out_sum,
                         double *q_side_sum, double *q_long_sum, double *num,
                         double *den);

/* hbt_read_hist without waiting for the copies: the arrays are snapshotted
 * on the device (stream-ordered after everything binned so far) and copied
 * to the caller's arrays on a copy stream, so the next bin calls run while
 * the copies are in flight.  The arrays hold the snapshot once
 * hbt_read_hist_wait returns; with pinned host arrays the copies overlap the
 * binning.  One read is in flight at a time: a second call first waits for
 * the previous one.  The device error flag travels with the snapshot and
 * is reported by hbt_read_hist_wait (HBT_ERR_DEVICE). */
hbt_status hbt_read_hist_async(hbt_ctx *ctx, double *num_count, double *q_out_sum,
                               double *q_side_sum, double *q_long_sum, double *num,
                               double *den);
hbt_status hbt_read_hist_wait(hbt_ctx *ctx);

/* q_inv histograms, n_KT * qnpts doubles each (q_inv_mean,
 * correl_1d_inv_num, correl_1d_inv_num_count, correl_1d_inv_denorm). */
hbt_status hbt_read_qinv(hbt_ctx *ctx, double *qinv_sum, double *num,
                         double *num_count, double *den);

/* Pair counters (number_of_pairs_{numerator,denormenator}_KTdiff or
 * _KTKphidiff: n_slots entries; _qinv_: n_KT entries). */
hbt_status hbt_read_counters(hbt_ctx *ctx, uint64_t *num, uint64_t *den,
                             uint64_t *num_qinv, uint64_t *den_qinv);

hbt_status hbt_get_stats(hbt_ctx *ctx, hbt_stats *out);

/* Fault injection for tests of the error paths; no counterpart in the
 * reference.  After n_ok more device allocations of this context succeed,
 * the next one fails as an out-of-memory would (the call returns
 * HBT_ERR_NOMEM, the histograms are unchanged and the context stays
 * usable); the injection then switches itself off.  n_ok = -1 switches it
 * off. */
hbt_status hbt_inject_alloc_failure(hbt_ctx *ctx, int32_t n_ok);

/* Largest partner pool hbt_bin_mixed_rotated_noalloc accepts (particles). */
#define HBT_NOALLOC_MAX_POOL 65536

/* No counterpart in the reference.  Mixed-event binning for callers that
 * cannot allocate device memory (a host framework that owns the device
 * memory through its own pool, or a loop that cannot afford an
 * allocation's implicit synchronisation).  Everything is caller-owned and
 * device-resident: list1 (n1 particles), the partner pool before rotation
 * (n2 <= HBT_NOALLOC_MAX_POOL particles) and the denominator histogram
 * `den` (hbt_n_bins() u64 counts for these params, not cleared: counts are
 * added).  The pool is rotated by (cos_phi, sin_phi) as the reference
 * rotates a mixed event and binned against list1 on `stream`; the rotated
 * copy lives in a fixed 2 MB __device__ scratch array that every GPU loading
 * the library holds until exit.  Requires azimuthal_flag == 0 and
 * invariant_radius_flag == 0; applies no needed_number_of_pairs cap.  list1
 * and the pool must already carry the rapidity cut the reference applies
 * before rotating (src/HBT_correlation.cpp:474-476, :509-511).  Pairs the
 * reference would index out of bounds (a NaN LCMS component, K_perp == 0)
 * are skipped and not reported by this entry point.  Calls share the
 * scratch and race if they overlap on the GPU.  The first call on a device
 * looks up the scratch address (again after the device's CUDA context is
 * re-created) and should come before any stream capture.  A CUDA error left
 * pending by earlier work is reported as such (HBT_ERR_CUDA) before
 * anything is launched.  On error a message is written to errbuf (may be
 * NULL). */
hbt_status hbt_bin_mixed_rotated_noalloc(const hbt_params *params, int64_t n1,
                                         const hbt_soa4 *list1, int64_t n2,
                                         const hbt_soa4 *pool, double cos_phi,
                                         double sin_phi, uint64_t *den, void *stream,
                                         char *errbuf, size_t errlen);

#ifdef __cplusplus
}
#endif
#endif /* HBT_GPU_H */
