// Shared definitions of the HBT pair-binning engine (device kernels and the
// C ABI layer).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "hbt_math.cuh"

namespace hbt {

typedef unsigned long long u64;

constexpr double kHbarC = 0.197327053;  // GeV fm (src/parameters.h:4)

// Histogram geometry and the constants the reference derives in its
// constructor (src/HBT_correlation.cpp:25-61, :253, :289-290, :342-345),
// computed once on the host with the reference's expressions.
struct Grid {
    int qnpts, n_KT, n_Kphi, n_slots;
    int azimuthal, qinv, boost;
    long long q3;
    double q_lo, q_hi, q_base, delta_q;
    double KT_min, dKT, KT_min_sq, KT_max_sq;
    double dKphi, two_pi, psi_ref, kphi_tol;
    double hbarC_inv;
    CosScale cph;  // table_cos constants for cos(q.dx / hbarC)
};

// Per-bin numerator sums, one 32-byte L2 sector per bin.
struct __align__(32) Sums {
    double qo, qs, ql, w;
};
struct __align__(16) QiSums {
    double q, w;
};

// Device histogram storage.
//  sums  [n_slots*q3] {q_out, q_side, q_long, cos(q.dx)} - one 32-byte sector
//  cnt   [n_slots*q3] numerator pair count
//  den   [n_slots*q3] denominator pair count
//  qi_*  [n_KT*qnpts] q_inv histograms
struct Hist {
    Sums *sums;  // 32-byte aligned {q_out, q_side, q_long, cos}
    u64 *cnt;
    u64 *den;
    QiSums *qi_sums;  // {q_inv, cos(q.dx)}
    u64 *qi_cnt;
    u64 *qi_den;
};

// Pair whose K_phi bin sits within kphi_tol of a bin edge: its azimuthal
// bin is decided on the host with the C library's atan2.  The record holds
// everything needed to bin the pair afterwards.
struct Deferral {
    long long i, j;          // row (list-1 / i) and column (list-2 / j) index
    double Kx, Ky;           // 0.5*(px_i + px_j), 0.5*(py_i + py_j), exact FP64
    double psi;              // psi_ref in force for the launch
    double qo, qs, ql, cosw; // LCMS components and cos(q.dx) (same-event)
    int iK, bin;             // K_T bin and 3-D bin within the slot
    int mixed, pad;          // 1: denominator pair
};

// Resolved deferral, sorted by key = i * cols + j.
struct Resolved {
    long long key;
    int iphi;  // -1: out of range (skip)
    int iK;
};

enum StatIdx {
    STAT_ANOMALY = 0,   // NaN LCMS component or K_T index out of range
    STAT_DEFER = 1,     // deferrals raised
    STAT_ERROR = 2,     // error flags (deferral overflow, missing lookup)
    STAT_N = 4
};

// Ordered cap admission (order-dependent needed_number_of_pairs caps).
// Stream bins: 3-D slots [0, n_slots) then q_inv K_T bins
// [n_slots, n_slots + n_KT).
struct Caps {
    unsigned *rowcnt;          // [n_stream][rows] survivors per row (count pass)
    long long *row_cut;        // [n_stream] rows < cut admitted, == cut straddles
    unsigned long long *quota; // [n_stream] admissions left in the straddle row
    const Resolved *resolved;  // deferred pairs resolved on the host
    int n_resolved;
    // admission of several mixed-event jobs in one pair of passes: a pair's
    // row is its job's row_base plus its position in list 1, rowcnt holds
    // rows_total rows per stream bin and deferral keys are row * cols_key +
    // column (0: one job, its own list sizes)
    long long rows_total, cols_key;
    // the 3-D slots already at their cap in the pass's counter family
    // (n_slots bytes), so that the batched passes skip tile pairs that can
    // reach no other slot; nullptr: none
    const unsigned char *slot_full;
};

// FP32 copies of the constants used by the FP32 pair screen (hbt_fast.cu),
// each with the bound on its rounding (slack) relative to the FP64 value.
struct Screen {
    float kt_lo4, kt_hi4, kt_slack;  // 4 KT_min^2, 4 KT_max^2 (0: no lower cut)
    float lo, hi, win_slack;         // q window bounds
    float base, inv_dq, t_slack;     // bin origin, 1/delta_q, slack in bin units
    float KT_min, inv_dKT, kt_t_slack;
    float psi, psi_slack, two_pi, inv_dKphi;
    int qnpts, n_KT, n_Kphi;
    // prefilter (hbt_tile.cuh prefilter()): Q = max(-lo, hi) + win_slack
    // with margin, Q^2, 2 Q^2 and the coefficient of the input-rounding term
    // of the q_T test
    float pq, pq2, pqt2, pqt_c;
    // 1 / hbarC as a double-float pair (FP32-weight phase)
    float hc_h, hc_l;
    // q_inv prefilter (invariant_radius_flag): square of the upper window
    // bound with its slack and a margin; -1 when no q_inv >= 0 can pass
    float qi_hi2;
    // Grid::kphi_tol rounded up: the K_phi screen leaves pairs this close to
    // an edge (plus its error bound) to the reference chain, which hands
    // them to the host, so that every pass that meets such a pair (the
    // screened kernels and the pair-by-pair cut rows of cap admission)
    // decides it the same way
    float kphi_tol;
};

// Host: the prefilter constants of a screen whose window is filled in.
inline void fill_prefilter(Screen &s) {
    const double U = 5.9604644775390625e-8;  // 2^-24
    const double Q = ((double)(-s.lo > s.hi ? -s.lo : s.hi) + (double)s.win_slack) * (1.0 + 1e-6);
    s.pq = (float)(Q * (1.0 + 1e-5));
    s.pq2 = (float)(Q * Q * (1.0 + 2e-4));
    s.pqt2 = (float)(2.0 * Q * Q * (1.0 + 2e-4));
    // (c + e)^2 <= c^2 + 2 c e (1 + 1e-4), c = sqrt(2) Q, e = 2.01 u L
    s.pqt_c = (float)(2.0 * 1.4142135623730951 * Q * 2.01 * U * (1.0 + 2e-4));
    const double hc = 1.0 / 0.197327053;  // 1 / hbarC [1 / (GeV fm)]
    s.hc_h = (float)hc;
    s.hc_l = (float)(hc - (double)s.hc_h);
    const double qh = ((double)s.hi + (double)s.win_slack) * (1.0 + 1e-6);
    s.qi_hi2 = qh > 0.0 ? (float)(qh * qh * (1.0 + 2e-4)) : -1.0f;
}

struct Device {
    Grid g;
    Screen s;
    Hist h;
    u64 *stats;
    Deferral *defer;
    unsigned *n_defer;
    unsigned defer_cap;
    Caps caps;
    // FP32-weight form: FP32 partial sums per bin {q_out, q_side, q_long,
    // cos}, merged into h.sums with the Kahan compensation terms `comp`.
    // Two arrays: pairs of even warps add to `part`, of odd warps to
    // `part_b`, so each partial bin takes about half of a bin's pairs
    // between two merges (partials_of below).
    int precision;                 // hbt_precision
    float4 *part;
    float4 *part_b;
    Sums *comp;
    long long merge_chunk_blocks;  // same-event CTAs between two merges
    long long block_offset;        // first triangular tile pair of a launch chunk
};

enum Mode { MODE_FAST = 0, MODE_COUNT = 1, MODE_ORDER = 2 };

// The FP32 partial array the calling warp adds to: odd warps of a CTA use
// the second one.  The rounding of an FP32 partial grows with the pairs it
// takes between merges (a busy bin's cos terms are alike, so their
// roundings add up), and two arrays halve that count without merging more
// often.
__device__ __forceinline__ float4 *partials_of(const Device &d) {
    return (threadIdx.x & 32) ? d.part_b : d.part;
}

// Launchers (hbt_kernels.cu).
cudaError_t launch_same(const Device &d, int mode, long long n, const double *const *c8,
                        cudaStream_t st);
cudaError_t launch_mixed(const Device &d, int mode, long long n1, const double *const *l1,
                         long long n2, const double *const *l2, cudaStream_t st);
cudaError_t launch_same_straddle(const Device &d, long long n, const double *const *c8,
                                 int n_stream, cudaStream_t st);
cudaError_t launch_mixed_straddle(const Device &d, long long n1, const double *const *l1,
                                  long long n2, const double *const *l2, int n_stream,
                                  cudaStream_t st);
cudaError_t launch_cut(const Device &d, long long rows, int n_stream,
                       const unsigned long long *remaining, cudaStream_t st);
// Bins n deferred records with their host-resolved K_phi bins (iphi[k]).
cudaError_t launch_apply(const Device &d, const Deferral *rec, const int *iphi, int n,
                         cudaStream_t st);
// The same with the record count in device memory (*count <= cap).
cudaError_t launch_apply_n(const Device &d, const Deferral *rec, const int *iphi, const int *count,
                           int cap, cudaStream_t st);
// A mixed-event job of a multi-job ordered admission, as the straddle
// kernel reads it: its lists in the caller's order and its first row.
struct StraddleJob {
    const double *a[4];
    const double *b[4];
    long long n1, n2, row_base;
};
cudaError_t launch_jobs_straddle(const Device &d, const StraddleJob *jobs, int n_jobs,
                                 long long rows, int n_stream, cudaStream_t st);
cudaError_t launch_defer_count(const Device &d, long long rows, long long cols, int n_res,
                               cudaStream_t st);
cudaError_t launch_counters(const Device &d, unsigned long long *out, cudaStream_t st);
// One output array of hbt_read_hist as FP64 in `out` (nbins doubles):
// field 0..3 = q_out, q_side, q_long, cos sums; 4 = numerator count;
// 5 = denominator count.
cudaError_t launch_export(const Device &d, int field, double *out, long long nbins,
                          cudaStream_t st);

// Merge of the FP32-weight partial sums into the FP64 bins (hbt_fast.cu).
// FP32 partials -> FP64 bins.  With n_items, the merge after a chunk of
// the batched same-event queue starting at chunk_base returns at once when
// the culled queue ended before it.
cudaError_t launch_merge(const Device &d, cudaStream_t st, const unsigned *n_items = nullptr,
                         unsigned chunk_base = 0);

// Screened fast-mode kernels (hbt_fast.cu): same results as MODE_FAST of the
// reference-chain kernels; require invariant_radius_flag == 0, n_KT <= 255
// and qnpts <= 1024.
cudaError_t launch_same_fast(const Device &d, long long n, const double *const *c8,
                             cudaStream_t st);
cudaError_t launch_mixed_fast(const Device &d, long long n1, const double *const *l1,
                              long long n2, const double *const *l2, cudaStream_t st);

}  // namespace hbt
