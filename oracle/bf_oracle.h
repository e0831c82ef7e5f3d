/*
 * CPU oracle for the balance-function pair binning - TEST INFRASTRUCTURE
 * ONLY.
 *
 * A plain, sequential restatement of the reference's BalanceFunction
 * (src/BalanceFunction.cpp in chunshen1987/hadronic_afterburner_toolkit) and
 * of the reader steps it depends on (particleSamples: the boost fields
 * pT, phi_p, rap_y, rap_eta of boostParticles, src/particleSamples.cpp
 * :442-468, and the per-species lists of filter_particles, :1300-1330 and
 * :1370-1460, plain Monte-Carlo numbers only).  Used by the tests as the
 * oracle of the GPU balance-function kernel and by the benchmark as the
 * timed CPU baseline; nothing in the product links or calls it.
 *
 * Parity pin: driven over tests/golden_bf/, its output files are
 * byte-identical to the reference binary's.
 */
#ifndef BF_ORACLE_H
#define BF_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_bf_params {
    int32_t particle_alpha, particle_beta;
    double BpT_min, BpT_max;
    int32_t Bnpts;
    double Brap_max;
    int32_t rap_type; /* 0: pseudo-rapidity differences, else rapidity */
    int32_t seed;     /* std::mt19937 seed of the mixed-event draws */
} orc_bf_params;

typedef struct orc_bf orc_bf;

orc_bf *orc_bf_create(const orc_bf_params *p);
void orc_bf_destroy(orc_bf *c);

/* The reader's boost of one particle (boostParticles): pT, phi_p, rap_y and
 * rap_eta after the rapidity shift of E and pz. */
void orc_bf_boost(int64_t n, const double *mass, const double *px, const double *py,
                  const double *pz, const double *E, double rap_shift, double *pT,
                  double *phi, double *rap_y, double *rap_eta);

/* One buffer through calculate_balance_function (src/BalanceFunction.cpp
 * :60-97): events as CSR (offsets, nev + 1 entries) with per-particle
 * monval, pT, phi_p, rap_y, rap_eta; the mixed-event pool likewise (the
 * same table when real mixed events are off). */
void orc_bf_process_buffer(orc_bf *c, int32_t nev, const int64_t *off, const int32_t *monval,
                           const double *pT, const double *phi, const double *y,
                           const double *eta, int32_t mnev, const int64_t *moff,
                           const int32_t *mmonval, const double *mpT, const double *mphi,
                           const double *my, const double *meta);

/* Bare pair loop of one histogram over one event pair (combine_and_bin_
 * particle_pairs / _mixed_particle_pairs, :124-208): lists a and b (pT,
 * phi_p, and the rapidity variable), rotation added to the azimuthal
 * difference when `mixed`.  Histogram `which`: 0 ab, 1 abar bbar, 2 a bbar,
 * 3 abar b, 4..7 the same with mixed events. */
void orc_bf_bin(orc_bf *c, int32_t which, int64_t na, const double *pTa, const double *phia,
                const double *ya, int64_t nb, const double *pTb, const double *phib,
                const double *yb, int32_t mixed, double rotation);

/* Bnpts x 20 counts of histogram `which`, [y bin][phi bin]. */
void orc_bf_get_hist(const orc_bf *c, int32_t which, double *out);
/* N_b and N_bbar (particles within the pT cut). */
void orc_bf_get_norm(const orc_bf *c, int64_t *N_b, int64_t *N_bbar);

/* output_balance_function (:211-319): the three files under `path`.
 * Returns 0, or -1 if a file cannot be opened. */
int orc_bf_write(const orc_bf *c, const char *path);

#ifdef __cplusplus
}
#endif
#endif /* BF_ORACLE_H */
