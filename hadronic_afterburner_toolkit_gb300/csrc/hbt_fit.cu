// Batched Gaussian HBT radii fits (include/hbt_fit.h).
//
// The reference fits each correlation table with scipy's curve_fit, one
// table and one q_cut at a time (ebe_scripts/fit_HBT_radii.py:60-92).  Here
// all fits of a batch of tables advance together:
//
//  * k_fit_select (one CTA per table) applies the script's preprocessing
//    (numpy nan_to_num, C_err + 1e-15, weight 1 / sigma) and keeps the rows
//    with q_cut_min < |q| < the largest cut, ordered by the smallest cut
//    they pass, so the rows of cut k are a prefix of the table's kept rows.
//    Per row it stores the five q products of the exponent (FP64 and FP32),
//    C and the weight.
//  * Each fit's rows are cut into work items of up to 8192 rows.  A pass
//    (k_fit_pass, one CTA per item) sums chi^2, J^T r and J^T J of every
//    active fit's items at its trial point; a step (k_fit_step, one thread
//    per fit) adds its items' sums and makes one Levenberg-Marquardt step:
//    damped 6 x 6 system by Cholesky, accept or reject, next trial point.
//    Passes and steps alternate until no fit has a trial point; work is
//    balanced over the GPU whatever the fits' sizes, and finished fits cost
//    nothing in later passes.
//  * A last pass sums J^T J in FP64 at each minimum; k_fit_finish inverts
//    it for the errors sqrt(diag((J^T J)^-1)) (curve_fit, absolute_sigma).
//
// A pass reads 76 bytes per row against about 35 FP64 operations (exp
// table-driven, hbt_math.cuh): the fits are bound by the FP64 pipe.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <string>
#include <type_traits>
#include <vector>

#include "../../include/hbt_fit.h"
#include "hbt_math.cuh"

namespace {

constexpr double kHbarC = 0.19733;  // fit_HBT_radii.py:10
constexpr double kEps = 1e-15;      // fit_HBT_radii.py:11
constexpr int kMaxCuts = 16;
constexpr int kSelThreads = 512;
constexpr int kFitThreads = 128;
constexpr int kSums = 28;  // chi2, J^T r (6), J^T J (21, packed lower)

// Resident pass CTAs per SM the pass kernel is compiled for.
#ifndef HBT_FIT_MIN_BLOCKS
#define HBT_FIT_MIN_BLOCKS 4
#endif

struct FitConst {
    double cut_sorted[kMaxCuts];  // ascending
    int rank[kMaxCuts];           // position of cut k in cut_sorted
    int by_rank[kMaxCuts];        // the cut at position s of cut_sorted
    int n_cuts;
    double q_cut_min;
    double p0[6];
    int max_iter;
};

// Where a table's columns sit in the batch's input buffer: column k of row
// i at in[base + col[k] + i * stride].  An interleaved host table (all five
// columns in one row-major block) is copied as that block; other tables are
// packed column by column (stride 1).
struct TabDesc {
    long long base, stride, col[5];
};

// Device rows of a batch: the kept rows of table t start at row_off[t];
// cls[t * (n_cuts + 1) + c] = rows of t whose smallest passed cut is c.
// Column k of kept row o: d[k * ld + o] for the doubles (the five q
// products q_out^2, q_side^2, q_long^2, 2 q_out q_side, 2 q_out q_long, then
// C and the weight), f[k * ld + o] for the FP32 copies of the q products.
// One base pointer each keeps the fitting loop's registers for its sums.
struct Rows {
    double *d;
    float *f;
    long long ld;
};
constexpr int kColC = 5, kColW = 6;

__device__ __forceinline__ double nan_to_num(double v) {
    if (isnan(v)) return 0.0;
    if (isinf(v)) return v > 0 ? DBL_MAX : -DBL_MAX;
    return v;
}

// numpy's sqrt(q_out**2. + q_side**2. + q_long**2.), without contraction.
__device__ __forceinline__ double qabs(double qo, double qs, double ql) {
    return sqrt(__dadd_rn(__dadd_rn(__dmul_rn(qo, qo), __dmul_rn(qs, qs)), __dmul_rn(ql, ql)));
}

__device__ __forceinline__ int cut_class(const FitConst &fc, double r) {
    if (!(r > fc.q_cut_min)) return -1;
    for (int c = 0; c < fc.n_cuts; c++)
        if (r < fc.cut_sorted[c]) return c;
    return -1;
}

// Two sweeps over a table's rows: the first counts the rows of each cut
// class (the smallest cut a row passes, or none), the second writes every
// kept row at its class's running position: within a class, rows keep
// their table order (the same arrays and sums on every run).
__global__ void __launch_bounds__(kSelThreads)
    k_fit_select(FitConst fc, const long long *tab_off, const TabDesc *desc, const double *in,
                 Rows out, int *cls) {
    __shared__ int cnt[kSelThreads / 32][kMaxCuts];
    __shared__ int base[kMaxCuts];
    const int t = blockIdx.x;
    const long long r0 = tab_off[t], n = tab_off[t + 1] - r0;
    const TabDesc d = desc[t];
    const double *qo_in = in + d.base + d.col[0], *qs_in = in + d.base + d.col[1],
                 *ql_in = in + d.base + d.col[2], *c_in = in + d.base + d.col[3],
                 *e_in = in + d.base + d.col[4];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nc = fc.n_cuts;
    const unsigned below = (1u << lane) - 1u;
    // sweep 1: rows per class (per-thread counters, then the block's sums)
    int mine[kMaxCuts];
#pragma unroll
    for (int c = 0; c < kMaxCuts; c++) mine[c] = 0;
    for (long long i = threadIdx.x; i < n; i += kSelThreads) {
        const int c = cut_class(fc, qabs(nan_to_num(qo_in[i * d.stride]),
                                         nan_to_num(qs_in[i * d.stride]),
                                         nan_to_num(ql_in[i * d.stride])));
#pragma unroll
        for (int k = 0; k < kMaxCuts; k++) mine[k] += (c == k);
    }
#pragma unroll
    for (int k = 0; k < kMaxCuts; k++) {
        if (k >= nc) break;
        int v = mine[k];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) cnt[warp][k] = v;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int run = 0;
        for (int k = 0; k < nc; k++) {
            int tot = 0;
            for (int w = 0; w < kSelThreads / 32; w++) tot += cnt[w][k];
            base[k] = run;
            cls[t * (nc + 1) + k] = tot;
            run += tot;
        }
        cls[t * (nc + 1) + nc] = run;
    }
    __syncthreads();
    // sweep 2: chunk by chunk, rank each row among its class in row order
    for (long long i0 = 0; i0 < n; i0 += kSelThreads) {
        const long long i = i0 + threadIdx.x;
        double qo = 0, qs = 0, ql = 0;
        int c = -1;
        if (i < n) {
            qo = nan_to_num(qo_in[i * d.stride]);
            qs = nan_to_num(qs_in[i * d.stride]);
            ql = nan_to_num(ql_in[i * d.stride]);
            c = cut_class(fc, qabs(qo, qs, ql));
        }
        // this warp's rows per class: zeroed, then each class group's first
        // lane writes the group's size
        for (int k = lane; k < nc; k += 32) cnt[warp][k] = 0;
        __syncwarp();
        const unsigned same = __match_any_sync(0xffffffffu, c);
        if (c >= 0 && lane == __ffs(same) - 1) cnt[warp][c] = __popc(same);
        __syncthreads();
        if (c >= 0) {
            int off = base[c] + __popc(same & below);
            for (int w = 0; w < warp; w++) off += cnt[w][c];
            const long long o = r0 + off;
            const double cc = nan_to_num(c_in[i * d.stride]);
            const double sigma = nan_to_num(e_in[i * d.stride]) + kEps;
            const double q5[5] = {qo * qo, qs * qs, ql * ql, 2.0 * qo * qs, 2.0 * qo * ql};
            for (int k = 0; k < 5; k++) {
                out.d[k * out.ld + o] = q5[k];
                out.f[k * out.ld + o] = (float)q5[k];
            }
            out.d[kColC * out.ld + o] = cc;
            out.d[kColW * out.ld + o] = 1.0 / sigma;
        }
        __syncthreads();
        if (threadIdx.x < nc) {
            int tot = 0;
            for (int w = 0; w < kSelThreads / 32; w++) tot += cnt[w][threadIdx.x];
            base[threadIdx.x] += tot;
        }
        __syncthreads();
    }
}

// One pass at parameters p: chi^2, J^T r, J^T J of the rows [0, n) of the
// fit, reduced over the block into red[0..27] (valid in thread 0).
// Residual r = w (f - C), J = w df/dp with f = lambda exp(-E),
// E = sum_k a_k^2 Q_k over the five q products Q_k (a_k = R_k / hbar c), so
// J_0 = w e and J_k = -w f (2 a_k / hbar c) Q_k: the constant factors
// 2 a_k / hbar c are applied after the sums.  chi^2 and J^T r, which fix
// where the minimum is, are summed in FP64.  J^T J only shapes the steps
// while iterating (kExact = false: FP32 products and per-thread sums over
// at most a few hundred rows, 1e-5 relative); the pass at the minimum that
// gives the covariance sums it in FP64 (kExact = true).
template <bool kExact>
__device__ void fit_pass(const Rows &rw, long long r0, int n, const double *p, const double *etab,
                         double *red) {
    using AccT = typename std::conditional<kExact, double, float>::type;
    __shared__ double part[kFitThreads / 32][kSums];
    double a2[5], cdf[7];
    cdf[0] = 1.0;
    for (int k = 0; k < 5; k++) {
        const double a = p[k + 1] / kHbarC;
        a2[k] = a * a;
        cdf[k + 1] = -2.0 * a / kHbarC;
    }
    const double lam = p[0];
    double s[7];
    AccT sa[21];
#pragma unroll
    for (int k = 0; k < 7; k++) s[k] = 0.0;
#pragma unroll
    for (int k = 0; k < 21; k++) sa[k] = 0;
    for (int i = threadIdx.x; i < n; i += kFitThreads) {
        const long long o = r0 + i;
        const double *dp = rw.d + o;
        double q[5];
#pragma unroll
        for (int k = 0; k < 5; k++) q[k] = dp[k * rw.ld];
        const double w = dp[kColW * rw.ld];
        double E = 0.0;
#pragma unroll
        for (int k = 0; k < 5; k++) E += a2[k] * q[k];
        const double e = table_exp(etab, -E);
        const double f = lam * e;
        const double r = w * (f - dp[kColC * rw.ld]);
        const double u = w * f;
        double v[6];  // J without its constant factors
        v[0] = w * e;
#pragma unroll
        for (int k = 0; k < 5; k++) v[k + 1] = u * q[k];
        s[0] += r * r;
#pragma unroll
        for (int k = 0; k < 6; k++) s[1 + k] += v[k] * r;
        AccT va[6];
        if (kExact) {
#pragma unroll
            for (int k = 0; k < 6; k++) va[k] = (AccT)v[k];
        } else {
            const float uf = (float)u;
            va[0] = (AccT)v[0];
#pragma unroll
            for (int k = 0; k < 5; k++) va[k + 1] = (AccT)(uf * rw.f[k * rw.ld + o]);
        }
        int m = 0;
#pragma unroll
        for (int j = 0; j < 6; j++)
#pragma unroll
            for (int k = 0; k <= j; k++) sa[m++] += va[j] * va[k];
    }
    double tot[kSums];
    tot[0] = s[0];
#pragma unroll
    for (int k = 0; k < 6; k++) tot[1 + k] = s[1 + k] * cdf[k];
    {
        int m = 0;
#pragma unroll
        for (int j = 0; j < 6; j++)
#pragma unroll
            for (int k = 0; k <= j; k++, m++) tot[7 + m] = (double)sa[m] * (cdf[j] * cdf[k]);
    }
#pragma unroll
    for (int k = 0; k < kSums; k++) {
        double x = tot[k];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        tot[k] = x;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0)
        for (int k = 0; k < kSums; k++) part[warp][k] = tot[k];
    __syncthreads();
    if (threadIdx.x < kSums) {
        double x = 0.0;
        for (int w = 0; w < kFitThreads / 32; w++) x += part[w][threadIdx.x];
        red[threadIdx.x] = x;
    }
    __syncthreads();
}

// Cholesky of the packed symmetric 6 x 6 matrix M (lower, row-major
// packed: M[j(j+1)/2 + k], k <= j) in place; false if not positive definite.
__device__ bool cholesky6(double *M) {
    for (int j = 0; j < 6; j++) {
        for (int k = 0; k <= j; k++) {
            double s = M[j * (j + 1) / 2 + k];
            for (int l = 0; l < k; l++) s -= M[j * (j + 1) / 2 + l] * M[k * (k + 1) / 2 + l];
            if (k == j) {
                if (!(s > 0.0)) return false;
                M[j * (j + 1) / 2 + j] = sqrt(s);
            } else {
                M[j * (j + 1) / 2 + k] = s / M[k * (k + 1) / 2 + k];
            }
        }
    }
    return true;
}

// Solves L L^T x = b with the factor of cholesky6.
__device__ void chol_solve6(const double *L, const double *b, double *x) {
    double y[6];
    for (int j = 0; j < 6; j++) {
        double s = b[j];
        for (int l = 0; l < j; l++) s -= L[j * (j + 1) / 2 + l] * y[l];
        y[j] = s / L[j * (j + 1) / 2 + j];
    }
    for (int j = 5; j >= 0; j--) {
        double s = y[j];
        for (int l = j + 1; l < 6; l++) s -= L[l * (l + 1) / 2 + j] * x[l];
        x[j] = s / L[j * (j + 1) / 2 + j];
    }
}

// Levenberg-Marquardt state of one fit, in device memory, advanced by one
// thread (k_fit_step) between the passes over the fit's rows.
struct LmState {
    double x[6], trial[6];
    double S, g[6], A[21], D[6], mu, nu;
    int iter, status, stop, go;
    int use_x;  // the next pass evaluates x (the start point), not trial
    long long passes;
};

// After the pass at the start point.
__device__ __noinline__ void lm_init(LmState &st, const double *red) {
    st.S = red[0];
    for (int j = 0; j < 6; j++) st.g[j] = red[1 + j];
    for (int j = 0; j < 21; j++) st.A[j] = red[7 + j];
    // Marquardt's scaling: the damping adds mu times the diagonal of J^T J
    // (dimensionless mu), so every parameter is damped on its own scale
    for (int j = 0; j < 6; j++) {
        const double d = st.A[j * (j + 1) / 2 + j];
        st.D[j] = d > 0 ? d : 1.0;
    }
    st.mu = 1e-3;
    st.nu = 2;
    st.iter = 0;
    st.status = HBT_FIT_CONVERGED;
    st.stop = 0;
    st.passes = 1;
}

// The next trial point: solve (A + mu D) delta = -g (D: the largest
// diagonal of J^T J seen, Marquardt's scaling), raising mu while the damped
// matrix is not positive definite.  go = 0 when the step no longer moves
// the point, the damping overflowed or the iterations ran out.
__device__ __noinline__ void lm_propose(LmState &st, int max_iter) {
    st.go = 0;
    while (!st.stop) {
        if (st.iter >= max_iter) {
            st.status = HBT_FIT_MAX_ITER;
            return;
        }
        st.iter++;
        double M[21], delta[6], mg[6];
        for (int j = 0; j < 21; j++) M[j] = st.A[j];
        for (int j = 0; j < 6; j++) {
            M[j * (j + 1) / 2 + j] += st.mu * st.D[j];
            mg[j] = -st.g[j];
        }
        if (!cholesky6(M)) {
            st.mu *= st.nu;
            st.nu *= 2;
            st.stop = !(st.mu < 1e300);
            continue;
        }
        chol_solve6(M, mg, delta);
        bool small = true;
        for (int j = 0; j < 6; j++) {
            st.trial[j] = st.x[j] + delta[j];
            if (fabs(delta[j]) > 1e-12 * (fabs(st.x[j]) + 1e-12)) small = false;
        }
        if (small) {
            st.stop = 1;
            return;
        }
        st.go = 1;
        return;
    }
}

// After the pass at the trial point: accept it when chi^2 fell (gain ratio
// rho > 0, Nielsen's update of mu), else raise mu.  Converged when an
// accepted step changed chi^2 by less than 1e-14 of it, predicted and
// actual.
__device__ __noinline__ void lm_update(LmState &st, const double *red) {
    st.passes++;
    const double Sn = red[0];
    double pred = 0;
    for (int j = 0; j < 6; j++) {
        const double dj = st.trial[j] - st.x[j];
        pred += dj * (st.mu * st.D[j] * dj - st.g[j]);
    }
    const double rho = (isfinite(Sn) && pred > 0) ? (st.S - Sn) / pred : -1.0;
    if (rho > 0) {
        const double drop = st.S - Sn;
        for (int j = 0; j < 6; j++) st.x[j] = st.trial[j];
        st.S = Sn;
        for (int j = 0; j < 6; j++) st.g[j] = red[1 + j];
        for (int j = 0; j < 21; j++) st.A[j] = red[7 + j];
        for (int j = 0; j < 6; j++) st.D[j] = fmax(st.D[j], st.A[j * (j + 1) / 2 + j]);
        const double q = 2 * rho - 1;
        st.mu *= fmax(1.0 / 3.0, 1.0 - q * q * q);
        st.nu = 2;
        st.stop = drop <= 1e-14 * st.S && pred <= 1e-14 * st.S;
    } else {
        st.mu *= st.nu;
        st.nu *= 2;
        st.stop = !(st.mu < 1e300);
    }
}

// A fit of a batch: table t, cut k, its n kept rows and its work items
// [item0, item1).
struct FitInfo {
    int t, k, n, item0, item1;
};

// A work item: up to kItemRows consecutive kept rows of one fit.
struct FitItem {
    int fit, rows;
    long long row0;
};
constexpr int kItemRows = 8192;

__global__ void k_fit_init(FitConst fc, const FitInfo *fits, int n_fits, LmState *st) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= n_fits) return;
    LmState &s = st[f];
    for (int j = 0; j < 6; j++) s.x[j] = s.trial[j] = fc.p0[j];
    s.use_x = 1;
    s.iter = 0;
    s.passes = 0;
    s.stop = 0;
    s.S = NAN;
    const bool enough = fits[f].n >= 6;
    s.go = enough;
    s.status = enough ? HBT_FIT_CONVERGED : HBT_FIT_TOO_FEW;
}

// One pass over every active fit's rows: each item's chi^2, J^T r and
// J^T J (at the fit's trial point, its start point on the first pass, or
// with kExact at its minimum for the covariance) into partial[item].
// Items of finished fits return at once.
template <bool kExact>
__global__ void __launch_bounds__(kFitThreads, HBT_FIT_MIN_BLOCKS)
    k_fit_pass(const FitItem *items, int n_items, Rows rw, const LmState *st, double *partial) {
    __shared__ double etab[EXP_TABLE];
    __shared__ double red[kSums];
    __shared__ double p[6];
    fill_exp_table(etab);
    for (int it = blockIdx.x; it < n_items; it += gridDim.x) {
        const FitItem I = items[it];
        const LmState &s = st[I.fit];
        if (kExact ? s.status == HBT_FIT_TOO_FEW : !s.go) continue;  // uniform in the block
        __syncthreads();  // the previous item's p and red are read
        if (threadIdx.x < 6) p[threadIdx.x] = (kExact || s.use_x) ? s.x[threadIdx.x] : s.trial[threadIdx.x];
        __syncthreads();
        fit_pass<kExact>(rw, I.row0, I.rows, p, etab, red);
        if (threadIdx.x < kSums) partial[(long long)it * kSums + threadIdx.x] = red[threadIdx.x];
    }
}

// The fit's sums: its items' partials added in item order.
__device__ __forceinline__ void fit_sums(const FitInfo &fi, const double *partial, double *red) {
    for (int k = 0; k < kSums; k++) red[k] = 0.0;
    for (int it = fi.item0; it < fi.item1; it++)
        for (int k = 0; k < kSums; k++) red[k] += partial[(long long)it * kSums + k];
}

// One Levenberg-Marquardt step of every active fit (one thread per fit);
// `active` is set while any fit has another trial point.
__global__ void k_fit_step(FitConst fc, const FitInfo *fits, int n_fits, LmState *st,
                           const double *partial, int *active) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= n_fits) return;
    LmState &s = st[f];
    if (!s.go) return;
    double red[kSums];
    fit_sums(fits[f], partial, red);
    if (s.use_x) {
        lm_init(s, red);
        s.use_x = 0;
    } else {
        lm_update(s, red);
    }
    lm_propose(s, fc.max_iter);
    if (s.go) atomicOr(active, 1);
}

// Results: the point, chi^2, the errors sqrt(diag((J^T J)^-1)) from the
// exact pass at the minimum (inf and the singular status when J^T J is not
// positive definite), rows, iterations, status.
__global__ void k_fit_finish(FitConst fc, int first_table, const FitInfo *fits, int n_fits,
                             const LmState *st, const double *partial, hbt_fit_result *res,
                             unsigned long long *n_passes) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= n_fits) return;
    const FitInfo fi = fits[f];
    const LmState &s = st[f];
    hbt_fit_result *out = res + (long long)(first_table + fi.t) * fc.n_cuts + fi.k;
    out->q_cut = fc.cut_sorted[fc.rank[fi.k]];
    out->n_points = fi.n;
    out->iterations = s.iter;
    out->reserved = 0;
    if (s.status == HBT_FIT_TOO_FEW) {
        for (int j = 0; j < 6; j++) out->p[j] = out->err[j] = NAN;
        out->chi2 = NAN;
        out->status = HBT_FIT_TOO_FEW;
        return;
    }
    for (int j = 0; j < 6; j++) out->p[j] = s.x[j];
    out->chi2 = s.S;
    int status = s.status;
    double red[kSums];
    fit_sums(fi, partial, red);
    double L[21];
    for (int j = 0; j < 21; j++) L[j] = red[7 + j];
    if (cholesky6(L)) {
        for (int j = 0; j < 6; j++) {
            double e[6] = {0, 0, 0, 0, 0, 0}, col[6];
            e[j] = 1.0;
            chol_solve6(L, e, col);
            out->err[j] = sqrt(col[j]);
        }
    } else {
        for (int j = 0; j < 6; j++) out->err[j] = INFINITY;
        if (status == HBT_FIT_CONVERGED) status = HBT_FIT_SINGULAR;
    }
    out->status = status;
    atomicAdd(n_passes, (unsigned long long)s.passes + 1);
}

struct Buf {
    void *p = nullptr;
    size_t bytes = 0;
};

bool grow(Buf &b, size_t bytes) {
    if (b.p && b.bytes >= bytes) return true;
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.bytes = 0;
    if (bytes == 0) return true;
    if (cudaMalloc(&b.p, bytes + bytes / 8) != cudaSuccess) {
        b.p = nullptr;
        return false;
    }
    b.bytes = bytes + bytes / 8;
    return true;
}

// Per batch: at most 32 M table rows (7 doubles and 5 floats each once
// kept) and 256 M doubles of input, which bounds the device memory of a
// call to about 4.5 GB; a batch of 41^3-row tables holds 464 of them.
constexpr long long kBatchRows = 32LL << 20;
constexpr long long kBatchIn = 256LL << 20;
// Iterations launched between two reads of the any-fit-active flag.
constexpr int kStepsPerCheck = 4;

// The input doubles of a table and, for an interleaved one, where its
// block starts: the five columns within one row-major block of n rows.
long long table_span(const hbt_fit_table &T, const double **lo_out) {
    const double *col[5] = {T.q_out, T.q_side, T.q_long, T.C, T.C_err};
    const uintptr_t b0 = reinterpret_cast<uintptr_t>(col[0]);
    uintptr_t lo = b0, hi = b0;
    bool aligned = true;
    for (const double *c : col) {
        const uintptr_t a = reinterpret_cast<uintptr_t>(c);
        lo = std::min(lo, a);
        hi = std::max(hi, a);
        aligned = aligned && (a - b0) % sizeof(double) == 0;
    }
    const long long width = (long long)((hi - lo) / sizeof(double)) + 1;
    if (T.stride > 1 && aligned && width <= T.stride && T.n_rows > 0) {
        *lo_out = reinterpret_cast<const double *>(lo);
        return (T.n_rows - 1) * T.stride + width;
    }
    *lo_out = nullptr;
    return 5 * T.n_rows;
}

}  // namespace

struct hbt_fit_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
    Buf in, rows, frows, tab_off, desc, cls, fits, items, state, partial, res, counter, active;
    int *active_host = nullptr;  // pinned
    std::vector<double> packed;
    hbt_fit_stats stats{};
    std::string err;
};

namespace {

hbt_status fit_fail(hbt_fit_ctx *c, hbt_status s, const std::string &m) {
    if (c) c->err = m;
    return s;
}

}  // namespace

extern "C" {

hbt_status hbt_fit_create(int device, hbt_fit_ctx **out) {
    if (!out) return HBT_ERR_INVALID;
    *out = nullptr;
    hbt_fit_ctx *c = new hbt_fit_ctx();
    c->device = device;
    if (cudaSetDevice(device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&c->ev[0]) != cudaSuccess || cudaEventCreate(&c->ev[1]) != cudaSuccess ||
        cudaEventCreate(&c->ev[2]) != cudaSuccess || !grow(c->counter, 8) ||
        !grow(c->active, sizeof(int)) ||
        cudaMallocHost(&c->active_host, sizeof(int)) != cudaSuccess) {
        hbt_fit_destroy(c);
        return HBT_ERR_CUDA;
    }
    *out = c;
    return HBT_OK;
}

void hbt_fit_destroy(hbt_fit_ctx *c) {
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (Buf *b : {&c->in, &c->rows, &c->frows, &c->tab_off, &c->desc, &c->cls, &c->fits,
                   &c->items, &c->state, &c->partial, &c->res, &c->counter, &c->active})
        if (b->p) cudaFree(b->p);
    for (cudaEvent_t e : c->ev)
        if (e) cudaEventDestroy(e);
    if (c->active_host) cudaFreeHost(c->active_host);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

const char *hbt_fit_last_error(const hbt_fit_ctx *c) { return c ? c->err.c_str() : "null context"; }

hbt_status hbt_fit_get_stats(const hbt_fit_ctx *c, hbt_fit_stats *out) {
    if (!c || !out) return HBT_ERR_INVALID;
    *out = c->stats;
    return HBT_OK;
}

hbt_status hbt_fit_radii(hbt_fit_ctx *c, int32_t n_tables, const hbt_fit_table *tables,
                         const hbt_fit_options *opt, hbt_fit_result *out) {
    if (!c || n_tables < 0 || (n_tables > 0 && (!tables || !out)) || !opt)
        return HBT_ERR_INVALID;
    if (opt->n_cuts < 1 || opt->n_cuts > kMaxCuts || !opt->q_cut_max)
        return fit_fail(c, HBT_ERR_INVALID, "n_cuts must be 1..16");
    FitConst fc{};
    fc.n_cuts = opt->n_cuts;
    fc.q_cut_min = opt->q_cut_min;
    fc.max_iter = opt->max_iterations > 0 ? opt->max_iterations : 500;
    for (int j = 0; j < 6; j++) fc.p0[j] = opt->p0[j];
    std::vector<int> order(opt->n_cuts);
    for (int k = 0; k < opt->n_cuts; k++) order[k] = k;
    std::stable_sort(order.begin(), order.end(),
                     [&](int a, int b) { return opt->q_cut_max[a] < opt->q_cut_max[b]; });
    for (int s = 0; s < opt->n_cuts; s++) {
        fc.cut_sorted[s] = opt->q_cut_max[order[s]];
        fc.rank[order[s]] = s;
        fc.by_rank[s] = order[s];
    }
    for (int t = 0; t < n_tables; t++) {
        const hbt_fit_table &T = tables[t];
        if (T.n_rows < 0 || T.stride < 1 ||
            (T.n_rows > 0 && (!T.q_out || !T.q_side || !T.q_long || !T.C || !T.C_err)))
            return fit_fail(c, HBT_ERR_INVALID, "table " + std::to_string(t) + " is invalid");
        const double *lo = nullptr;
        if (T.n_rows > kBatchRows || table_span(T, &lo) > kBatchIn)
            return fit_fail(c, HBT_ERR_INVALID, "table larger than a launch's row budget");
    }
    if (cudaSetDevice(c->device) != cudaSuccess) return fit_fail(c, HBT_ERR_CUDA, "cudaSetDevice");
    c->stats = hbt_fit_stats{};
    c->stats.fits = (int64_t)n_tables * opt->n_cuts;
    if (n_tables == 0) return HBT_OK;
    const int nc = opt->n_cuts;
    if (!grow(c->res, (size_t)n_tables * nc * sizeof(hbt_fit_result)))
        return fit_fail(c, HBT_ERR_NOMEM, "device allocation failed");
    cudaStream_t st = c->stream;
    cudaError_t e = cudaMemsetAsync(c->counter.p, 0, 8, st);
    float up_ms = 0.f, fit_ms = 0.f;
    std::vector<long long> off;
    std::vector<TabDesc> desc;
    std::vector<const double *> block;
    std::vector<long long> packed_at;
    std::vector<int> cls_h;
    std::vector<FitInfo> fits;
    std::vector<FitItem> items;
    for (int t0 = 0; t0 < n_tables && e == cudaSuccess;) {
        // the batch: tables [t0, t1) within the row and input budgets
        int t1 = t0;
        long long rows = 0, in_total = 0, n_packed = 0;
        off.assign(1, 0);
        desc.clear();
        block.clear();
        while (t1 < n_tables) {
            const hbt_fit_table &T = tables[t1];
            const double *lo = nullptr;
            const long long span = table_span(T, &lo);
            if (t1 > t0 && (rows + T.n_rows > kBatchRows || in_total + span > kBatchIn)) break;
            TabDesc d{};
            d.base = in_total;
            if (lo) {
                d.stride = T.stride;
                const double *col[5] = {T.q_out, T.q_side, T.q_long, T.C, T.C_err};
                for (int k = 0; k < 5; k++) d.col[k] = col[k] - lo;
            } else {
                d.stride = 1;
                for (int k = 0; k < 5; k++) d.col[k] = k * T.n_rows;
                n_packed += span;
            }
            desc.push_back(d);
            block.push_back(lo);
            in_total += span;
            rows += T.n_rows;
            off.push_back(rows);
            t1++;
        }
        const int nt = t1 - t0;
        bool ok = grow(c->tab_off, (nt + 1) * sizeof(long long)) &&
                  grow(c->desc, nt * sizeof(TabDesc)) &&
                  grow(c->cls, (size_t)nt * (nc + 1) * sizeof(int)) &&
                  grow(c->in, in_total * sizeof(double)) &&
                  grow(c->rows, 7 * rows * sizeof(double)) &&
                  grow(c->frows, 5 * rows * sizeof(float));
        if (!ok) return fit_fail(c, HBT_ERR_NOMEM, "device allocation failed");
        // tables that are not one interleaved block are packed on the host
        c->packed.resize((size_t)std::max<long long>(n_packed, 1));
        long long pk = 0;
        packed_at.assign(nt, -1);
        for (int t = t0; t < t1; t++) {
            if (block[t - t0]) continue;
            const hbt_fit_table &T = tables[t];
            const double *col[5] = {T.q_out, T.q_side, T.q_long, T.C, T.C_err};
            packed_at[t - t0] = pk;
            for (int k = 0; k < 5; k++)
                for (long long i = 0; i < T.n_rows; i++) c->packed[pk++] = col[k][i * T.stride];
        }
        double *din = static_cast<double *>(c->in.p);
        Rows rw{static_cast<double *>(c->rows.p), static_cast<float *>(c->frows.p), rows};
        const long long *d_off = static_cast<const long long *>(c->tab_off.p);
        if ((e = cudaEventRecord(c->ev[0], st)) != cudaSuccess ||
            (e = cudaMemcpyAsync(c->tab_off.p, off.data(), off.size() * sizeof(long long),
                                 cudaMemcpyHostToDevice, st)) != cudaSuccess ||
            (e = cudaMemcpyAsync(c->desc.p, desc.data(), desc.size() * sizeof(TabDesc),
                                 cudaMemcpyHostToDevice, st)) != cudaSuccess)
            break;
        // all copies first (copies from pageable memory wait for the stream's
        // earlier work, so a kernel between them would serialise them), then
        // the row selection of every table
        for (int t = t0; t < t1 && e == cudaSuccess; t++) {
            const long long span =
                (t + 1 < t1 ? desc[t - t0 + 1].base : in_total) - desc[t - t0].base;
            if (span == 0) continue;
            const double *src = block[t - t0] ? block[t - t0] : c->packed.data() + packed_at[t - t0];
            e = cudaMemcpyAsync(din + desc[t - t0].base, src, span * sizeof(double),
                                cudaMemcpyHostToDevice, st);
        }
        if (e != cudaSuccess) break;
        k_fit_select<<<nt, kSelThreads, 0, st>>>(fc, d_off, static_cast<const TabDesc *>(c->desc.p),
                                                din, rw, static_cast<int *>(c->cls.p));
        if ((e = cudaGetLastError()) != cudaSuccess) break;
        // the fits and their work items, from the selected row counts
        cls_h.resize((size_t)nt * (nc + 1));
        if ((e = cudaMemcpyAsync(cls_h.data(), c->cls.p, cls_h.size() * sizeof(int),
                                 cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
            (e = cudaEventRecord(c->ev[1], st)) != cudaSuccess ||
            (e = cudaStreamSynchronize(st)) != cudaSuccess)
            break;
        fits.clear();
        items.clear();
        for (int t = 0; t < nt; t++)
            for (int k = 0; k < nc; k++) {
                FitInfo fi{t, k, 0, (int)items.size(), 0};
                for (int r = 0; r <= fc.rank[k]; r++) fi.n += cls_h[(size_t)t * (nc + 1) + r];
                if (fi.n >= 6)
                    for (int r = 0; r < fi.n; r += kItemRows)
                        items.push_back(FitItem{(int)fits.size(), std::min(kItemRows, fi.n - r),
                                                off[t] + r});
                fi.item1 = (int)items.size();
                fits.push_back(fi);
            }
        const int nf = (int)fits.size(), ni = (int)items.size();
        ok = grow(c->fits, nf * sizeof(FitInfo)) && grow(c->items, std::max(ni, 1) * sizeof(FitItem)) &&
             grow(c->state, nf * sizeof(LmState)) &&
             grow(c->partial, (size_t)std::max(ni, 1) * kSums * sizeof(double));
        if (!ok) return fit_fail(c, HBT_ERR_NOMEM, "device allocation failed");
        if ((e = cudaMemcpyAsync(c->fits.p, fits.data(), nf * sizeof(FitInfo),
                                 cudaMemcpyHostToDevice, st)) != cudaSuccess ||
            (ni > 0 && (e = cudaMemcpyAsync(c->items.p, items.data(), ni * sizeof(FitItem),
                                            cudaMemcpyHostToDevice, st)) != cudaSuccess))
            break;
        const FitInfo *d_fits = static_cast<const FitInfo *>(c->fits.p);
        const FitItem *d_items = static_cast<const FitItem *>(c->items.p);
        LmState *d_state = static_cast<LmState *>(c->state.p);
        double *d_part = static_cast<double *>(c->partial.p);
        int *d_active = static_cast<int *>(c->active.p);
        const unsigned fb = (unsigned)((nf + 127) / 128);
        const unsigned pg = (unsigned)std::max(1, std::min(ni, 152 * HBT_FIT_MIN_BLOCKS * 8));
        k_fit_init<<<fb, 128, 0, st>>>(fc, d_fits, nf, d_state);
        e = cudaGetLastError();
        // Levenberg-Marquardt: a pass over all active fits' rows, then one
        // step of every active fit; the flag is read every few iterations
        for (int done = 0; e == cudaSuccess && ni > 0 && done <= fc.max_iter + 1;
             done += kStepsPerCheck) {
            for (int r = 0; r < kStepsPerCheck && e == cudaSuccess; r++) {
                if ((e = cudaMemsetAsync(d_active, 0, sizeof(int), st)) != cudaSuccess) break;
                k_fit_pass<false><<<pg, kFitThreads, 0, st>>>(d_items, ni, rw, d_state, d_part);
                k_fit_step<<<fb, 128, 0, st>>>(fc, d_fits, nf, d_state, d_part, d_active);
                e = cudaGetLastError();
            }
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(c->active_host, d_active, sizeof(int), cudaMemcpyDeviceToHost,
                                    st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(st);
            if (e != cudaSuccess || *c->active_host == 0) break;
        }
        if (e != cudaSuccess) break;
        // J^T J in FP64 at each minimum, then the results
        if (ni > 0) k_fit_pass<true><<<pg, kFitThreads, 0, st>>>(d_items, ni, rw, d_state, d_part);
        k_fit_finish<<<fb, 128, 0, st>>>(fc, t0, d_fits, nf, d_state, d_part,
                                          static_cast<hbt_fit_result *>(c->res.p),
                                          static_cast<unsigned long long *>(c->counter.p));
        if ((e = cudaGetLastError()) != cudaSuccess) break;
        if ((e = cudaEventRecord(c->ev[2], st)) != cudaSuccess) break;
        if ((e = cudaStreamSynchronize(st)) != cudaSuccess) break;
        float a = 0.f, b = 0.f;
        cudaEventElapsedTime(&a, c->ev[0], c->ev[1]);
        cudaEventElapsedTime(&b, c->ev[1], c->ev[2]);
        up_ms += a;
        fit_ms += b;
        c->stats.rows += rows;
        t0 = t1;
    }
    if (e != cudaSuccess) {
        cudaStreamSynchronize(st);
        return fit_fail(c, HBT_ERR_CUDA, cudaGetErrorString(e));
    }
    unsigned long long passes = 0;
    if ((e = cudaMemcpyAsync(out, c->res.p, (size_t)n_tables * nc * sizeof(hbt_fit_result),
                             cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
        (e = cudaMemcpyAsync(&passes, c->counter.p, 8, cudaMemcpyDeviceToHost, st)) !=
            cudaSuccess ||
        (e = cudaStreamSynchronize(st)) != cudaSuccess)
        return fit_fail(c, HBT_ERR_CUDA, cudaGetErrorString(e));
    for (long long f = 0; f < (long long)n_tables * nc; f++) c->stats.points += out[f].n_points;
    c->stats.passes = (int64_t)passes;
    c->stats.upload_ms = up_ms;
    c->stats.kernel_ms = fit_ms;
    return HBT_OK;
}

}  // extern "C"
