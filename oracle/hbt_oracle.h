/*
 * CPU oracle for the HBT pair-binning path - TEST INFRASTRUCTURE ONLY.
 *
 * A plain, sequential restatement of the reference's HBT correlation
 * algorithm (src/HBT_correlation.cpp in chunshen1987/hadronic_afterburner_toolkit),
 * used by the test-suite as the oracle of the GPU engine and by the
 * benchmark as the timed CPU baseline.  Nothing in the product links or
 * calls this library.
 *
 * Parity pin: driven over the seeded inputs in tests/golden/, the oracle's
 * output files are byte-identical to the reference binary's (built from the
 * reference sources by oracle/Makefile).
 */
#ifndef HBT_ORACLE_H
#define HBT_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_params {
    int32_t qnpts;
    double q_min, q_max;
    int32_t n_KT;
    double KT_min, KT_max;
    int32_t n_Kphi;
    int32_t azimuthal_flag;
    int32_t invariant_radius_flag;
    int32_t long_comoving_boost;
    double needed_number_of_pairs; /* as read from parameters.dat */
    double HBTrap_min, HBTrap_max;
    int32_t number_of_mixed_events; /* <= 0: reference rule nev/2 + 1 */
    int32_t seed;                   /* std::mt19937 seed */
} orc_params;

typedef struct orc_ctx orc_ctx;

orc_ctx *orc_create(const orc_params *p);
void orc_destroy(orc_ctx *c);

/* One buffer (oversample group) through calculate_HBT_correlation_function
 * (src/HBT_correlation.cpp:177-218).  Columns are px, py, pz, E, x, y, z, t;
 * events are CSR (offsets has nev + 1 entries).  The mixed-event pool is a
 * second CSR table (pass the same one when real mixed events are off). */
void orc_process_buffer(orc_ctx *c, int32_t nev, const int64_t *off,
                        const double *const *cols, int32_t mixed_nev,
                        const int64_t *moff, const double *const *mcols);

/* Bare pair loops over already-gathered lists (src/HBT_correlation.cpp
 * :289-461 and :561-689).  cols8 = px, py, pz, E, x, y, z, t; cols4 = px,
 * py, pz, E. */
void orc_bin_same(orc_ctx *c, int64_t n, const double *const *cols8);
void orc_bin_mixed(orc_ctx *c, int64_t n1, const double *const *l1,
                   int64_t n2, const double *const *l2);

/* Multi-threaded variants for the CPU baseline: same counts, summation
 * order differs; only valid while no pair cap can bind. */
void orc_bin_same_mt(orc_ctx *c, int64_t n, const double *const *cols8,
                     int32_t nthreads);
void orc_bin_mixed_mt(orc_ctx *c, int64_t n1, const double *const *l1,
                      int64_t n2, const double *const *l2, int32_t nthreads);

/* particleSamples::boostParticles (src/particleSamples.cpp:442-468) on
 * E and pz, in place: E' = E cosh(s) + pz sinh(s), pz' = pz cosh(s) + E sinh(s). */
void orc_rapidity_shift(int64_t n, double *E, double *pz, double shift);

void orc_set_psi_ref(orc_ctx *c, double psi);
double orc_get_psi_ref(const orc_ctx *c);
/* calculate_flow_event_plane_angle (src/HBT_correlation.cpp:233-249) over
 * the px, py of every particle given. */
double orc_event_plane_angle(int64_t n, const double *px, const double *py,
                             int32_t n_order);

/* Mixed-event partners per event for a pool of mixed_nev events
 * (number_of_mixed_events, or the reference's mixed_nev / 2 + 1). */
int32_t orc_mixed_partners(const orc_ctx *c, int32_t mixed_nev);

/* Draws what orc_process_buffer's mixed-event loop draws for a buffer of
 * nev events and a pool of mixed_nev events (src/HBT_correlation.cpp:197-217,
 * :495-497), advancing the same generator: partners[iev * nmix + k] and the
 * rotation angles[iev * nmix + k] = rand_uniform() * 2 pi.  Returns nmix. */
int32_t orc_mixed_plan(orc_ctx *c, int32_t nev, int32_t mixed_nev, int32_t *partners,
                       double *angles);

/* Histogram geometry: n_slots = n_KT (azimuthal 0) or n_KT * n_Kphi;
 * per slot qnpts^3 bins in [iqout][iqside][iqlong] order. */
int64_t orc_n_bins(const orc_ctx *c);
void orc_get_hist(const orc_ctx *c, double *num_count, double *q_out_sum,
                  double *q_side_sum, double *q_long_sum, double *num,
                  double *den);
/* Sum of |cos(q.dx)| per 3-D bin (the scale against which the numerator's
 * rounding is stated; no counterpart in the reference's output). */
void orc_get_abs_num(const orc_ctx *c, double *abs_num);
/* q_inv histograms, [n_KT][qnpts] each. */
void orc_get_qinv(const orc_ctx *c, double *qinv_sum, double *num,
                  double *num_count, double *den);
/* Pair counters: KT-differential (n_KT each) or KT x Kphi (n_KT*n_Kphi). */
void orc_get_counters(const orc_ctx *c, uint64_t *num, uint64_t *den,
                      uint64_t *num_qinv, uint64_t *den_qinv);
/* Pairs skipped because an LCMS component was NaN (K_perp == 0) or a bin
 * index fell outside the arrays; the reference's behaviour there is
 * undefined (out-of-bounds write). */
uint64_t orc_anomalies(const orc_ctx *c);
uint64_t orc_pairs_same(const orc_ctx *c);
uint64_t orc_pairs_mixed(const orc_ctx *c);

/* output_HBTcorrelation (src/HBT_correlation.cpp:220-228, :694-855). */
int orc_write(const orc_ctx *c, const char *path, int32_t eco_output);

#ifdef __cplusplus
}
#endif
#endif
