/*
 * hbt_fit.h - batched Gaussian HBT radii fits on the GPU (libhbt_gpu.so).
 *
 * Replaces the per-table fit loop of the reference's
 * ebe_scripts/fit_HBT_radii.py (chunshen1987/hadronic_afterburner_toolkit,
 * :60-92): for every correlation table (one K_T bin of one event) and every
 * q_cut, the weighted least-squares fit of
 *
 *   C(q) = lambda exp(-((R_out q_out)^2 + (R_side q_side)^2
 *                       + (R_long q_long)^2 + 2 q_out q_side R_os^2
 *                       + 2 q_out q_long R_ol^2))          (radii / hbar c)
 *
 * to the rows with q_cut_min < |q| < q_cut, weights 1 / (C_err + 1e-15),
 * after NaN -> 0 and +-inf -> +-DBL_MAX on every column (numpy's
 * nan_to_num).  Each fit is a Levenberg-Marquardt minimisation in FP64
 * from the given start point with the analytic Jacobian; the errors are
 * the square roots of the diagonal of (J^T J)^-1 at the minimum (scipy's
 * curve_fit with absolute_sigma=True).  The fits of a batch of tables (up
 * to 256 M input doubles) advance together, pass by pass, with every
 * fit's rows cut into work items spread over the GPU.
 */
#ifndef HBT_FIT_H
#define HBT_FIT_H

#include "hbt_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct hbt_fit_ctx hbt_fit_ctx;

/* One correlation table, host memory: row i of column X is X[i * stride]
 * (stride 1 for separate arrays; 8 with pointers into a row-major
 * eight-column table, q_out = &t[0], q_side = &t[1], q_long = &t[2],
 * C = &t[6], C_err = &t[7]). */
typedef struct hbt_fit_table {
    int64_t n_rows;
    int64_t stride;
    const double *q_out;
    const double *q_side;
    const double *q_long;
    const double *C;
    const double *C_err;
} hbt_fit_table;

typedef struct hbt_fit_options {
    int32_t n_cuts;           /* 1..16 */
    const double *q_cut_max;  /* n_cuts upper |q| bounds (the script's q_cut_max_list) */
    double q_cut_min;         /* lower |q| bound, exclusive (the script's 0) */
    double p0[6];             /* start: lambda, R_out, R_side, R_long, R_os, R_ol (fm) */
    int32_t max_iterations;   /* 0: 500 */
} hbt_fit_options;

/* Fit status */
#define HBT_FIT_CONVERGED 0
#define HBT_FIT_MAX_ITER 1    /* iteration limit reached; p is the best point found */
#define HBT_FIT_SINGULAR 2    /* J^T J not positive definite at the minimum: err = inf */
#define HBT_FIT_TOO_FEW 3     /* fewer rows than parameters: p and err NaN */

typedef struct hbt_fit_result {
    double q_cut;
    double p[6];   /* lambda, R_out, R_side, R_long, R_os, R_ol (fm) */
    double err[6];
    double chi2;   /* sum of squared weighted residuals at p */
    int32_t n_points;
    int32_t iterations;
    int32_t status;
    int32_t reserved;
} hbt_fit_result;

typedef struct hbt_fit_stats {
    int64_t fits;
    int64_t rows;          /* table rows uploaded */
    int64_t points;        /* sum over fits of the rows fitted */
    int64_t passes;        /* sum over fits of the passes over their rows */
    double upload_ms;      /* device time of the copies and row selection */
    double kernel_ms;      /* device time of the fits (passes, steps, errors) */
} hbt_fit_stats;

hbt_status hbt_fit_create(int device, hbt_fit_ctx **out);
void hbt_fit_destroy(hbt_fit_ctx *ctx);
const char *hbt_fit_last_error(const hbt_fit_ctx *ctx);

/* Fits every (table, q_cut): out[t * n_cuts + k]. */
hbt_status hbt_fit_radii(hbt_fit_ctx *ctx, int32_t n_tables, const hbt_fit_table *tables,
                         const hbt_fit_options *options, hbt_fit_result *out);

hbt_status hbt_fit_get_stats(const hbt_fit_ctx *ctx, hbt_fit_stats *out);

#ifdef __cplusplus
}
#endif
#endif /* HBT_FIT_H */
