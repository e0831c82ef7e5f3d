/*
 * hbt_host.h - C ABI of the drop-in host side (libhbt_host.so).
 *
 * The C++ classes ParameterReader, RandomUtil::Random, particleSamples,
 * HBT_correlation and Analysis under hadronic_afterburner_toolkit_gb300/host
 * are source-compatible with the reference's (the src/ headers of
 * chunshen1987/hadronic_afterburner_toolkit); C++ callers use them directly.
 * These entry points serve callers through an FFI.
 */
#ifndef HBT_HOST_H
#define HBT_HOST_H

#include <stdint.h>

#include "hbt_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* The reference executable's HBT run (src/main.cpp:21-46 with
 * Analysis::PerformAnalysis, src/Analysis.cpp:54-112): reads `param_file`
 * plus key=value strings argv[1..argc-1], reads the samples under
 * `results_path` and writes the HBT_correlation_function_*.dat files there.
 * Returns 0, 255 for a parameter error, 1 for any other error (message on
 * stderr). */
int hbt_host_run(int argc, char **argv, const char *param_file, const char *results_path);

/* Writes the reference's output files from histogram arrays laid out as
 * hbt_read_hist / hbt_read_qinv / hbt_read_counters return them
 * (HBT_correlation::output_HBTcorrelation, src/HBT_correlation.cpp:220-228,
 * :694-855).  The q_inv arrays are read only when invariant_radius_flag is
 * 1.  Returns 0, or -1 if a file cannot be opened. */
int hbt_host_write(const hbt_params *params, const char *path, int32_t eco_output,
                   const double *num_count, const double *q_out_sum, const double *q_side_sum,
                   const double *q_long_sum, const double *num, const double *den,
                   const double *qinv_sum, const double *qinv_num, const double *qinv_count,
                   const double *qinv_den, const uint64_t *ctr_num, const uint64_t *ctr_den,
                   const uint64_t *ctr_num_qinv, const uint64_t *ctr_den_qinv);

/* psi_ref of the reference's calculate_flow_event_plane_angle(n_order)
 * (src/HBT_correlation.cpp:233-249, what get_psi_ref() returns after it):
 * atan2(sum sin(n phi), sum cos(n phi)) / n over the n particles in order,
 * phi = atan2(py, px).  The drop-in's HBT_correlation computes it with the
 * same sums.  NaN for invalid arguments. */
double hbt_host_event_plane_angle(int64_t n, const double *px, const double *py,
                                  int32_t n_order);

/* The mixed-event partner ids and rotation angles the drop-in draws for a
 * run of n_buffers buffers from one RandomUtil::Random seeded with `seed`
 * (HBT_correlation::calculate_HBT_correlation_function and
 * combine_and_bin_particle_pairs_mixed_events, src/HBT_correlation.cpp
 * :197-217 and :495-497): for buffer b and each of its nev[b] events in
 * order, nmix partner ids (rand_int_uniform() % mixed_nev[b], redrawn while
 * equal to the event when mixed_nev[b] != 1), then nmix angles
 * rand_uniform() * 2 pi, with nmix = n_partners when > 0 (the optional key
 * hbt_mixed_partners), else mixed_nev[b] / 2 + 1.  Entries are written in
 * that order to partners[] and angles[] (sum over b of nev[b] * nmix
 * each, at most `cap`).  The rotation of a partner's particles is
 * px' = px cos(angle) - py sin(angle), py' = px sin(angle) + py cos(angle)
 * with the C library's cos and sin.  For FFI callers that drive the engine
 * themselves with the reference's partners.  Returns the number of entries,
 * or -1 for invalid arguments or a too small `cap`. */
int64_t hbt_host_mixed_plan(int32_t seed, int32_t n_buffers, const int32_t *nev,
                            const int32_t *mixed_nev, int32_t n_partners, int64_t cap,
                            int32_t *partners, double *angles);

/* Reads the samples of a parameter file's HBT setup buffer by buffer with
 * the reference's reader rules (particleSamples, src/particleSamples.cpp),
 * without binning anything: for each buffer, the event count and particle
 * count of the species of interest, same-event list then mixed-event pool.
 * Fills up to `cap` buffers; returns the number of buffers, or -1 on error. */
int hbt_host_scan_buffers(const char *param_file, const char *results_path, int32_t cap,
                          int32_t *nev, int64_t *n_particles, int32_t *mixed_nev,
                          int64_t *n_mixed_particles);

/* The reader's output, buffer by buffer, as a digest: for each buffer a
 * 64-bit FNV-1a hash over the event count, every event's particle count and
 * every field of every particle (bit patterns, after the species filter and
 * the rapidity boost), same-event list then mixed pool.  `args` are extra
 * "key=value" strings applied after the parameter file (e.g.
 * "hbt_fast_reader=0" selects the line-by-line reader).  Fills up to `cap`
 * digests; returns the number of buffers, or -1 on error.  No counterpart in
 * the reference: it lets two readers be compared without moving the
 * particles through the FFI. */
int hbt_host_digest_buffers(const char *param_file, const char *results_path, int32_t n_args,
                            char **args, int32_t cap, uint64_t *digest);

/* Reads every buffer of the samples (same-event list and mixed pool, with
 * the species filter and boost) and returns the wall time in seconds, the
 * particles read (before the filter) and the bytes of decompressed text;
 * `args` as above.  Returns 0, or -1 on error.  For timing the reader. */
int hbt_host_time_reader(const char *param_file, const char *results_path, int32_t n_args,
                         char **args, double *seconds, int64_t *particles, int64_t *text_bytes);

/* Event averaging of the HBT correlation files (the reference's
 * ebe_scripts/average_event_HBT_correlation_function.py): for every HBT*
 * file of the first UrQMD* folder's UrQMD_results under `working_folder`,
 * the element-wise mean over all UrQMD* folders (directory order, as the
 * script's glob) written to `avg_folder` with "%.10e" and two blanks between
 * columns.  Files are averaged on `threads` host threads (0: all).  Returns
 * the number of files written, or -1 on error. */
int hbt_host_average_events(const char *working_folder, const char *avg_folder,
                            int32_t threads);

#ifdef __cplusplus
}
#endif
#endif /* HBT_HOST_H */
