/*
 * hbt_server.h - HBT serving loop of libhbt_gpu.so (C ABI).
 *
 * No counterpart in the reference, whose analysis runs one buffer at a time
 * in a single process (src/main.cpp -> Analysis -> HBT_correlation).  A
 * server owns one GPU and a worker thread.  A request is one HBT analysis of
 * one event buffer with its own parameters (q grid, K_T / K_phi bins,
 * precision); it is what HBT_correlation::calculate_HBT_correlation_function
 * (src/HBT_correlation.cpp:177-218) computes for a buffer, with the pair
 * loops on the GPU:
 *   - the event-plane angle psi_ref of the buffer when azimuthal_flag == 1
 *     (calculate_flow_event_plane_angle(2), src/HBT_correlation.cpp:233-249);
 *   - the same-event pairs of each oversample group (combine_and_bin_particle_
 *     pairs, src/HBT_correlation.cpp:254-461): the buffer's events in groups
 *     of `oversample` consecutive events, each group one pair list;
 *   - for each event, `mixed_partners` partner events drawn from the buffer
 *     with the reference's Random (std::mt19937(seed); a partner id is
 *     redrawn while it equals the event unless the buffer has one event),
 *     each partner rotated by its own random angle, and the mixed pairs of
 *     the event against the rotated partners (combine_and_bin_particle_pairs_
 *     mixed_events, src/HBT_correlation.cpp:466-689);
 *   - the rapidity cut tanh(Krap_min) < pz/E < tanh(Krap_max) of both gathers.
 *
 * Continuous batching: requests wait in a FIFO queue until the device memory
 * their histograms and particle buffers need fits the server's budget and
 * an active slot is free; admitted requests keep their particles and
 * histograms resident in HBM; each round the worker takes pending pair work
 * of several active requests (same kernel class: azimuthal_flag,
 * long_comoving_boost, precision) into ONE sorted, culled, persistent launch
 * (hbt_bin_batch's pipeline), so requests that arrive while others run
 * share the GPU with them.  A finished request's histograms are copied to
 * host memory and its device memory is released at once.
 *
 * Requests whose pair cap (needed_number_of_pairs) could bind, that ask for
 * q_inv histograms or for a kernel other than HBT_KERNEL_SCREENED run alone
 * through the per-analysis entry points (hbt_bin_same_dev / _mixed_dev in
 * the reference's order) on their own stream, concurrently with the rounds.
 *
 * Every result equals the one of the same request run alone: counts and bin
 * indices exactly, FP64 sums to summation order (about 1e-15 relative per
 * bin).
 */
#ifndef HBT_SERVER_H
#define HBT_SERVER_H

#include "hbt_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct hbt_server hbt_server;

typedef struct hbt_server_config {
    int32_t device;            /* CUDA device */
    uint64_t memory_budget;    /* device bytes admitted requests may hold
                                  (0: 80% of the free memory at creation) */
    int32_t max_active;        /* requests resident at once (0: 64) */
    int64_t round_tile_pairs;  /* candidate 128x128 tile pairs per round
                                  (0: 65536, about 1e9 candidate pairs) */
    int32_t max_in_flight;     /* rounds queued on the GPU ahead of the
                                  worker (0: 2) */
} hbt_server_config;

/* One request: an event buffer of one particle species and its analysis.
 * Columns are host arrays of event_offsets[n_events] particles, events
 * stored one after another (event e is rows event_offsets[e] ..
 * event_offsets[e+1]-1).  They are copied during hbt_server_submit. */
typedef struct hbt_request {
    hbt_params params;
    int32_t n_events;
    const int64_t *event_offsets; /* n_events + 1 entries, event_offsets[0] == 0 */
    hbt_soa8 particles;           /* px py pz E x y z t */
    int32_t oversample;           /* events per same-event list (0: the whole buffer) */
    int32_t mixed_partners;       /* partners per event (0: n_events/2 + 1 as the
                                     reference's default) */
    double Krap_min, Krap_max;    /* pair-rapidity window of the gathers */
    int32_t seed;                 /* Random seed (>= 0) */
} hbt_request;

typedef enum hbt_job_state {
    HBT_JOB_QUEUED = 0,  /* waiting for memory or a slot */
    HBT_JOB_ACTIVE = 1,  /* resident, pair work issued or pending */
    HBT_JOB_DONE = 2,    /* results in host memory */
    HBT_JOB_FAILED = 3
} hbt_job_state;

typedef struct hbt_job_info {
    int32_t state;           /* hbt_job_state */
    int32_t status;          /* hbt_status of a failed request */
    int32_t solo;            /* 1: ran through the per-analysis path */
    int32_t rounds;          /* batched rounds that carried its work */
    double queue_ms;         /* submit -> admission */
    double latency_ms;       /* submit -> results in host memory */
    uint64_t pairs_same;     /* candidate same-event pairs */
    uint64_t pairs_mixed;    /* candidate mixed-event pairs */
    uint64_t device_bytes;   /* device memory held while active */
    double psi_ref;          /* event-plane angle used for K_phi */
    int64_t n_bins;          /* hbt_n_bins of its parameters */
    uint64_t anomalies;      /* hbt_stats.anomalies of its pairs */
} hbt_job_info;

typedef struct hbt_server_stats {
    uint64_t submitted, completed, failed;
    uint64_t rounds;             /* batched launches */
    uint64_t pairs;              /* candidate pairs of completed requests */
    uint64_t bytes_in_use, peak_bytes;
    int32_t active, queued, peak_active;
    double p50_ms, p99_ms, mean_ms, max_ms; /* latency of completed requests */
    double gpu_busy_ms;          /* time with at least one round in flight */
} hbt_server_stats;

hbt_status hbt_server_create(const hbt_server_config *cfg, hbt_server **out);
/* Finishes every submitted request, then stops the worker and frees the
 * server (results not read are lost). */
void hbt_server_destroy(hbt_server *s);
const char *hbt_server_last_error(const hbt_server *s);

/* Validates and copies the request, draws its mixed partners and rotation
 * angles, and queues it.  Returns HBT_ERR_INVALID for bad parameters and
 * HBT_ERR_NOMEM when the request could never fit the memory budget. */
hbt_status hbt_server_submit(hbt_server *s, const hbt_request *req, uint64_t *job_id);

/* Waits until the request is done or failed (timeout_us 0: no limit). */
hbt_status hbt_server_wait(hbt_server *s, uint64_t job_id, uint64_t timeout_us);

hbt_status hbt_server_job_info(hbt_server *s, uint64_t job_id, hbt_job_info *out);

/* The mixing the server drew for a request: partners[e * P + k] is the k-th
 * partner of event e and (cos_phi, sin_phi)[e * P + k] its rotation, with
 * P = the request's partner count (any pointer may be NULL). */
hbt_status hbt_server_mixing(hbt_server *s, uint64_t job_id, int32_t *partners_per_event,
                             int32_t *partners, double *cos_phi, double *sin_phi);

/* Results of a done request, in hbt_read_hist / hbt_read_qinv /
 * hbt_read_counters layout (any pointer may be NULL). */
hbt_status hbt_server_read_hist(hbt_server *s, uint64_t job_id, double *num_count,
                                double *q_out_sum, double *q_side_sum, double *q_long_sum,
                                double *num, double *den);
hbt_status hbt_server_read_qinv(hbt_server *s, uint64_t job_id, double *qinv_sum, double *num,
                                double *num_count, double *den);
hbt_status hbt_server_read_counters(hbt_server *s, uint64_t job_id, uint64_t *num,
                                    uint64_t *den, uint64_t *num_qinv, uint64_t *den_qinv);

/* Forgets a done or failed request (frees its host results). */
hbt_status hbt_server_release(hbt_server *s, uint64_t job_id);

hbt_status hbt_server_get_stats(hbt_server *s, hbt_server_stats *out);
/* Clears the latency record and the counters (not the requests). */
hbt_status hbt_server_reset_stats(hbt_server *s);

#ifdef __cplusplus
}
#endif
#endif /* HBT_SERVER_H */
