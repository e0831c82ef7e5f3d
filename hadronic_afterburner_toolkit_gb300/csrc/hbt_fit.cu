// Batched Gaussian HBT radii fits (include/hbt_fit.h).
//
// The reference fits each correlation table with scipy's curve_fit, one
// table and one q_cut at a time (ebe_scripts/fit_HBT_radii.py:60-92).  Here
// every (table, q_cut) of a batch is one CTA of one launch, and two batches
// are in flight on two streams (one copying while the other fits):
//
//  * k_fit_select (one CTA per table) applies the script's preprocessing
//    (numpy nan_to_num, C_err + 1e-15, weight 1 / sigma) and keeps the rows
//    with q_cut_min < |q| < the largest cut, ordered by the smallest cut
//    they pass, so the rows of cut k are a prefix of the table's kept rows.
//    Per row it stores the five q products of the exponent, C and the
//    weight (7 doubles).
//  * k_fit_lm (one CTA per fit) runs Levenberg-Marquardt in FP64: each pass
//    over the rows accumulates chi^2, J^T r and J^T J (28 sums, analytic
//    Jacobian) with a block reduction; one thread solves the damped 6 x 6
//    system by Cholesky and decides the next trial point.  At the minimum
//    the errors are sqrt(diag((J^T J)^-1)) (curve_fit, absolute_sigma).
//
// The rows a fit touches are read once per pass: 76 bytes per row against
// about 35 FP64 operations (exp table-driven, hbt_math.cuh), so the fits
// are bound by the FP64 pipe.
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

// Resident fitting CTAs per SM the iterations' kernel is compiled for.
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

// Levenberg-Marquardt state of one fit, in shared memory, advanced by one
// thread between the block's passes over the rows.
struct LmState {
    double x[6], trial[6];
    double S, g[6], A[21], D[6], mu, nu;
    int iter, status, stop, go;
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

// Results of the iterations: the point and chi^2 (the errors follow in
// k_fit_cov).
__device__ __noinline__ void lm_finish(const LmState &st, double q_cut, int n,
                                       hbt_fit_result *out) {
    out->q_cut = q_cut;
    for (int j = 0; j < 6; j++) {
        out->p[j] = st.x[j];
        out->err[j] = NAN;
    }
    out->chi2 = st.S;
    out->n_points = n;
    out->iterations = st.iter;
    out->reserved = 0;
    out->status = st.status;
}

// The errors: sqrt(diag((J^T J)^-1)) with J^T J summed in FP64 at the
// minimum (inf and the singular status when it is not positive definite).
__device__ __noinline__ void cov_finish(const double *red, hbt_fit_result *out) {
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
        if (out->status == HBT_FIT_CONVERGED) out->status = HBT_FIT_SINGULAR;
    }
}

// The fit of a block: the largest cuts first (they have the most rows), so
// a launch's tail is made of the small fits.
__device__ __forceinline__ void fit_of_block(const FitConst &fc, int &t, int &k) {
    const int nt = gridDim.x / fc.n_cuts;
    t = blockIdx.x % nt;
    k = fc.by_rank[fc.n_cuts - 1 - blockIdx.x / nt];
}

__device__ __forceinline__ int rows_of_fit(const FitConst &fc, const int *cls, int t, int k) {
    int n = 0;
    for (int c = 0; c <= fc.rank[k]; c++) n += cls[t * (fc.n_cuts + 1) + c];
    return n;
}

__global__ void __launch_bounds__(kFitThreads, HBT_FIT_MIN_BLOCKS)
    k_fit_lm(FitConst fc, int first_table, const long long *tab_off, const int *cls, Rows rw,
             hbt_fit_result *res, unsigned long long *n_passes) {
    __shared__ double red[kSums];
    __shared__ LmState st;
    __shared__ double etab[EXP_TABLE];
    int t, k;
    fit_of_block(fc, t, k);
    const long long r0 = tab_off[t];
    const int n = rows_of_fit(fc, cls, t, k);
    hbt_fit_result *out = res + (long long)(first_table + t) * fc.n_cuts + k;
    const double q_cut = fc.cut_sorted[fc.rank[k]];
    if (n < 6) {
        if (threadIdx.x == 0) {
            out->q_cut = q_cut;
            for (int j = 0; j < 6; j++) out->p[j] = out->err[j] = NAN;
            out->chi2 = NAN;
            out->n_points = n;
            out->iterations = 0;
            out->status = HBT_FIT_TOO_FEW;
            out->reserved = 0;
        }
        return;
    }
    if (threadIdx.x < 6) st.x[threadIdx.x] = fc.p0[threadIdx.x];
    fill_exp_table(etab);
    __syncthreads();
    // one pass per trial point: the first at the start point
    for (bool first = true;; first = false) {
        fit_pass<false>(rw, r0, n, first ? st.x : st.trial, etab, red);
        if (threadIdx.x == 0) {
            if (first)
                lm_init(st, red);
            else
                lm_update(st, red);
            lm_propose(st, fc.max_iter);
        }
        __syncthreads();
        if (!st.go) break;
    }
    if (threadIdx.x == 0) {
        lm_finish(st, q_cut, n, out);
        atomicAdd(n_passes, (unsigned long long)st.passes + 1);  // + k_fit_cov's pass
    }
}

// One pass at each fit's minimum with J^T J in FP64, for the errors.  A
// kernel of its own so that the iterations' kernel keeps the FP32 sums'
// register budget.
__global__ void __launch_bounds__(kFitThreads)
    k_fit_cov(FitConst fc, int first_table, const long long *tab_off, const int *cls, Rows rw,
              hbt_fit_result *res) {
    __shared__ double red[kSums];
    __shared__ double x[6];
    __shared__ double etab[EXP_TABLE];
    int t, k;
    fit_of_block(fc, t, k);
    const int n = rows_of_fit(fc, cls, t, k);
    if (n < 6) return;
    hbt_fit_result *out = res + (long long)(first_table + t) * fc.n_cuts + k;
    if (threadIdx.x < 6) x[threadIdx.x] = out->p[threadIdx.x];
    fill_exp_table(etab);
    __syncthreads();
    fit_pass<true>(rw, tab_off[t], n, x, etab, red);
    if (threadIdx.x == 0) cov_finish(red, out);
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

// Per batch: at most 4 M table rows (7 doubles and 5 floats each once
// kept) and 32 M doubles of input; two batches are in flight (one copying
// while the other fits), which bounds the device memory of a call to
// 1.1 GB.  A batch of 41^3-row tables holds 58 of them (290 fits).
constexpr long long kBatchRows = 4LL << 20;
constexpr long long kBatchIn = 32LL << 20;

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

// One of the two batches in flight: its device buffers, its stream (copies,
// row selection, fits, errors in order) and the host arrays its copies read.
struct FitSlot {
    cudaStream_t stream = nullptr;
    cudaEvent_t t0 = nullptr, t1 = nullptr, t2 = nullptr;
    Buf in, rows, frows, tab_off, desc, cls;
    std::vector<double> packed;
    std::vector<long long> off;
    std::vector<TabDesc> desc_h;
    bool busy = false;
};

struct hbt_fit_ctx {
    int device = 0;
    FitSlot slot[2];
    Buf res, counter;
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
    bool ok = cudaSetDevice(device) == cudaSuccess && grow(c->counter, 8);
    for (FitSlot &sl : c->slot)
        ok = ok && cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking) == cudaSuccess &&
             cudaEventCreate(&sl.t0) == cudaSuccess && cudaEventCreate(&sl.t1) == cudaSuccess &&
             cudaEventCreate(&sl.t2) == cudaSuccess;
    if (!ok) {
        hbt_fit_destroy(c);
        return HBT_ERR_CUDA;
    }
    *out = c;
    return HBT_OK;
}

void hbt_fit_destroy(hbt_fit_ctx *c) {
    if (!c) return;
    cudaSetDevice(c->device);
    for (FitSlot &sl : c->slot) {
        if (sl.stream) cudaStreamSynchronize(sl.stream);
        for (Buf *b : {&sl.in, &sl.rows, &sl.frows, &sl.tab_off, &sl.desc, &sl.cls})
            if (b->p) cudaFree(b->p);
        for (cudaEvent_t e : {sl.t0, sl.t1, sl.t2})
            if (e) cudaEventDestroy(e);
        if (sl.stream) cudaStreamDestroy(sl.stream);
    }
    for (Buf *b : {&c->res, &c->counter})
        if (b->p) cudaFree(b->p);
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
    if (!grow(c->res, (size_t)n_tables * opt->n_cuts * sizeof(hbt_fit_result)))
        return fit_fail(c, HBT_ERR_NOMEM, "device allocation failed");
    FitSlot *S = c->slot;
    cudaError_t e = cudaMemsetAsync(c->counter.p, 0, 8, S[0].stream);
    // slot 1 starts after the counter is cleared
    if (e == cudaSuccess) e = cudaEventRecord(S[0].t2, S[0].stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(S[1].stream, S[0].t2, 0);
    float up_ms = 0.f, fit_ms = 0.f;
    // a slot's previous batch must be done before its buffers and host
    // arrays are reused; its times are collected then
    auto retire = [&](FitSlot &sl) -> cudaError_t {
        if (!sl.busy) return cudaSuccess;
        const cudaError_t r = cudaEventSynchronize(sl.t2);
        if (r != cudaSuccess) return r;
        float a = 0.f, b = 0.f;
        cudaEventElapsedTime(&a, sl.t0, sl.t1);
        cudaEventElapsedTime(&b, sl.t1, sl.t2);
        up_ms += a;
        fit_ms += b;
        sl.busy = false;
        return cudaSuccess;
    };
    std::vector<const double *> block;
    std::vector<long long> packed_at;
    int batch = 0;
    for (int t0 = 0; t0 < n_tables && e == cudaSuccess; batch++) {
        FitSlot &sl = S[batch & 1];
        if ((e = retire(sl)) != cudaSuccess) break;
        // the batch: tables [t0, t1) within the row and input budgets
        int t1 = t0;
        long long rows = 0, in_total = 0, n_packed = 0;
        sl.off.assign(1, 0);
        sl.desc_h.clear();
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
            sl.desc_h.push_back(d);
            block.push_back(lo);
            in_total += span;
            rows += T.n_rows;
            sl.off.push_back(rows);
            t1++;
        }
        const int nt = t1 - t0;
        bool ok = grow(sl.tab_off, (nt + 1) * sizeof(long long)) &&
                  grow(sl.desc, nt * sizeof(TabDesc)) &&
                  grow(sl.cls, (size_t)nt * (opt->n_cuts + 1) * sizeof(int)) &&
                  grow(sl.in, in_total * sizeof(double));
        ok = ok && grow(sl.rows, 7 * rows * sizeof(double)) &&
             grow(sl.frows, 5 * rows * sizeof(float));
        if (!ok) {
            for (FitSlot &x : c->slot) cudaStreamSynchronize(x.stream);
            return fit_fail(c, HBT_ERR_NOMEM, "device allocation failed");
        }
        // tables that are not one interleaved block are packed on the host
        sl.packed.resize((size_t)std::max<long long>(n_packed, 1));
        long long pk = 0;
        packed_at.assign(nt, -1);
        for (int t = t0; t < t1; t++) {
            if (block[t - t0]) continue;
            const hbt_fit_table &T = tables[t];
            const double *col[5] = {T.q_out, T.q_side, T.q_long, T.C, T.C_err};
            packed_at[t - t0] = pk;
            for (int k = 0; k < 5; k++)
                for (long long i = 0; i < T.n_rows; i++) sl.packed[pk++] = col[k][i * T.stride];
        }
        double *din = static_cast<double *>(sl.in.p);
        e = cudaEventRecord(sl.t0, sl.stream);
        for (int t = t0; t < t1 && e == cudaSuccess; t++) {
            const long long span =
                (t + 1 < t1 ? sl.desc_h[t - t0 + 1].base : in_total) - sl.desc_h[t - t0].base;
            if (span == 0) continue;
            const double *src = block[t - t0] ? block[t - t0] : sl.packed.data() + packed_at[t - t0];
            e = cudaMemcpyAsync(din + sl.desc_h[t - t0].base, src, span * sizeof(double),
                                cudaMemcpyHostToDevice, sl.stream);
        }
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(sl.tab_off.p, sl.off.data(), sl.off.size() * sizeof(long long),
                                cudaMemcpyHostToDevice, sl.stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(sl.desc.p, sl.desc_h.data(), sl.desc_h.size() * sizeof(TabDesc),
                                cudaMemcpyHostToDevice, sl.stream);
        if (e != cudaSuccess) break;
        Rows rw{static_cast<double *>(sl.rows.p), static_cast<float *>(sl.frows.p), rows};
        const long long *d_off = static_cast<const long long *>(sl.tab_off.p);
        k_fit_select<<<nt, kSelThreads, 0, sl.stream>>>(
            fc, d_off, static_cast<const TabDesc *>(sl.desc.p), din, rw,
            static_cast<int *>(sl.cls.p));
        if ((e = cudaGetLastError()) != cudaSuccess) break;
        if ((e = cudaEventRecord(sl.t1, sl.stream)) != cudaSuccess) break;
        k_fit_lm<<<nt * opt->n_cuts, kFitThreads, 0, sl.stream>>>(
            fc, t0, d_off, static_cast<const int *>(sl.cls.p), rw,
            static_cast<hbt_fit_result *>(c->res.p), static_cast<unsigned long long *>(c->counter.p));
        if ((e = cudaGetLastError()) != cudaSuccess) break;
        k_fit_cov<<<nt * opt->n_cuts, kFitThreads, 0, sl.stream>>>(
            fc, t0, d_off, static_cast<const int *>(sl.cls.p), rw,
            static_cast<hbt_fit_result *>(c->res.p));
        if ((e = cudaGetLastError()) != cudaSuccess) break;
        if ((e = cudaEventRecord(sl.t2, sl.stream)) != cudaSuccess) break;
        sl.busy = true;
        c->stats.rows += rows;
        t0 = t1;
    }
    for (FitSlot &sl : c->slot) {
        const cudaError_t r = retire(sl);
        if (e == cudaSuccess) e = r;
    }
    if (e != cudaSuccess) {
        for (FitSlot &sl : c->slot) cudaStreamSynchronize(sl.stream);
        return fit_fail(c, HBT_ERR_CUDA, cudaGetErrorString(e));
    }
    unsigned long long passes = 0;
    if ((e = cudaMemcpyAsync(out, c->res.p, (size_t)n_tables * opt->n_cuts * sizeof(hbt_fit_result),
                             cudaMemcpyDeviceToHost, S[0].stream)) != cudaSuccess ||
        (e = cudaMemcpyAsync(&passes, c->counter.p, 8, cudaMemcpyDeviceToHost, S[0].stream)) !=
            cudaSuccess ||
        (e = cudaStreamSynchronize(S[0].stream)) != cudaSuccess)
        return fit_fail(c, HBT_ERR_CUDA, cudaGetErrorString(e));
    for (long long f = 0; f < (long long)n_tables * opt->n_cuts; f++)
        c->stats.points += out[f].n_points;
    c->stats.passes = (int64_t)passes;
    c->stats.upload_ms = up_ms;
    c->stats.kernel_ms = fit_ms;
    return HBT_OK;
}

}  // extern "C"
