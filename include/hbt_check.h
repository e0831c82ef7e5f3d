/*
 * hbt_check.h - device checks of the engine's own FP64 elementary functions
 * (libhbt_gpu.so).  The pair kernels and the radii fits evaluate cos and
 * exp with table-driven implementations of their own (csrc/hbt_math.cuh,
 * and the double-float cos of csrc/hbt_tile.cuh);
 * this entry point runs them on the device over caller-given arguments so
 * that tests can compare them with the host's libm.  Not part of the
 * reference's interface.
 */
#ifndef HBT_CHECK_H
#define HBT_CHECK_H

#include "hbt_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

#define HBT_CHECK_COS 0 /* the pair kernels' table_cos at scale 1: cos(x) */
#define HBT_CHECK_EXP 1 /* the radii fits' table_exp */
#define HBT_CHECK_DFCOS 2 /* the double-float form's df_cos, of x split into
                             hi = (float)x and lo = (float)(x - hi) */
#define HBT_CHECK_COS_PHASE 3 /* table_cos with the pair kernels' scale:
                                 cos(x / hbarC), the product never rounded */

/* out[i] = f(x[i]) on `device` for the function `which`; host arrays. */
hbt_status hbt_check_math(int device, int32_t which, int64_t n, const double *x, double *out);

#ifdef __cplusplus
}
#endif
#endif /* HBT_CHECK_H */
