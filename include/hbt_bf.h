/*
 * hbt_bf.h - balance-function pair binning on the GPU (libhbt_gpu.so).
 *
 * Replaces the pair loops of the reference's BalanceFunction
 * (src/BalanceFunction.cpp:124-208 of chunshen1987/hadronic_afterburner_
 * toolkit): for each event, every particle of species list A against every
 * particle of species list B of the same event (or of a drawn mixed event,
 * with a global rotation added to the azimuthal difference), binned in
 * (Delta y, Delta phi) into one of eight histograms (ab, abar bbar, a bbar,
 * abar b; then the same four with mixed events).  The bins and counts are
 * the reference's exactly: an FP32 screen with rigorous error bounds decides
 * a pair's bin unless it lies near a bin edge or a cut, where the reference's
 * FP64 expressions run in its operation order.
 *
 * The host side (species lists, pT cut, random partner events and
 * rotations, output files) stays in C++ above this boundary.
 */
#ifndef HBT_BF_H
#define HBT_BF_H

#include "hbt_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

#define HBT_BF_NPHI 20 /* Delta phi bins (the reference's Bnphi) */

typedef struct hbt_bf_params {
    int32_t Bnpts;   /* "Bnpts": Delta y bins */
    double Brap_max; /* "Brap_max" */
} hbt_bf_params;

typedef struct hbt_bf_ctx hbt_bf_ctx;

/* One species list of several events, FP64 host arrays: event e holds
 * particles offsets[e] .. offsets[e+1]-1; phi = phi_p; y = the rapidity
 * variable of the analysis (rap_y, or rap_eta when rap_type is 0).
 * Particles outside the pT window must be left out by the caller (the
 * reference skips them in both loops). */
typedef struct hbt_bf_list {
    int32_t n_events;
    const int64_t *offsets;
    const double *phi;
    const double *y;
} hbt_bf_list;

/* One event pair: particles of a's event ea against b's event eb; `rotation`
 * is added to phi_a - phi_b when `mixed` is 1 (the mixed-event loop). */
typedef struct hbt_bf_job {
    int32_t hist;     /* 0..7 */
    int32_t la, ea;   /* list and event of the first particles */
    int32_t lb, eb;   /* list and event of the second particles */
    int32_t mixed;
    double rotation;
} hbt_bf_job;

hbt_status hbt_bf_create(const hbt_bf_params *params, int device, hbt_bf_ctx **out);
void hbt_bf_destroy(hbt_bf_ctx *ctx);
const char *hbt_bf_last_error(const hbt_bf_ctx *ctx);
hbt_status hbt_bf_reset(hbt_bf_ctx *ctx);

/* Bins the jobs over `n_lists` species lists (host arrays, copied during the
 * call) in one launch; counts add to the histograms. */
hbt_status hbt_bf_bin(hbt_bf_ctx *ctx, int32_t n_lists, const hbt_bf_list *lists,
                      int32_t n_jobs, const hbt_bf_job *jobs);

/* Counts of histogram `hist`, Bnpts x HBT_BF_NPHI doubles, [y bin][phi bin]
 * (the reference's C_ab ... C_mixed_abarb arrays). */
hbt_status hbt_bf_read(hbt_bf_ctx *ctx, int32_t hist, double *out);

/* What the last hbt_bf_bin did: candidate pairs, bytes copied to the device
 * (lists passed more than once with the same pointers are copied once), and
 * the device time of the copies and of the binning kernel (CUDA events on
 * the context's stream). */
typedef struct hbt_bf_stats {
    int64_t pairs;
    int64_t bytes_uploaded;
    int64_t fp64_pairs; /* pairs the FP32 screen left to the FP64 path */
    double upload_ms;
    double kernel_ms;
} hbt_bf_stats;

hbt_status hbt_bf_get_stats(const hbt_bf_ctx *ctx, hbt_bf_stats *out);

#ifdef __cplusplus
}
#endif
#endif /* HBT_BF_H */
