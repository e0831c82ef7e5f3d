// HBT pair-binning kernels for sm_103a (plain FP64 form).
//
// Every bin-deciding expression follows the reference's operand order
// (src/HBT_correlation.cpp:311-458 same-event, :574-687 mixed-event) and the
// translation unit is compiled with --fmad=false, so each FP64 add, multiply,
// divide and square root is the same IEEE-rounded operation the reference's
// CPU build performs.  Pair counts and bin indices are therefore bit-exact;
// only the order of the FP64 sums differs.
//
// Launch shapes
//  same-event : one CTA per (i-tile <= j-tile) pair of 128-particle tiles;
//               the j-tile is staged in shared memory, each thread owns one i.
//  mixed-event: one CTA per (list-1 tile, list-2 tile).
// Admission modes for the order-dependent pair caps (needed_number_of_pairs):
//  FAST  - no cap can bind in this launch: bin every survivor.
//  COUNT - count survivors per (stream bin, row) for the ordered pass.
//  ORDER - admit rows before each stream bin's cut row; the cut row itself
//          is admitted in pair order by the straddle kernel.
#include "hbt_engine.cuh"
#include <algorithm>

#include "hbt_chain.cuh"

namespace hbt {
namespace {

using namespace chain;

template <int MODE>
__global__ void __launch_bounds__(TILE) k_same(Device d, long long n, Cols8 c) {
    __shared__ double sj[8][TILE];
    long long ti, tj;
    tri_tile(blockIdx.x, ti, tj);
    const int tid = threadIdx.x;
    const long long j0 = tj * TILE;
    for (int f = 0; f < 8; f++) sj[f][tid] = (j0 + tid < n) ? c.p[f][j0 + tid] : 0.0;
    __syncthreads();
    const long long i = ti * TILE + tid;
    if (i >= n) return;
    const double apx = c.p[0][i], apy = c.p[1][i], apz = c.p[2][i], aE = c.p[3][i];
    const double ax[4] = {c.p[4][i], c.p[5][i], c.p[6][i], c.p[7][i]};
    const int jend = (int)min((long long)TILE, n - j0);
    for (int jj = 0; jj < jend; jj++) {
        const long long j = j0 + jj;
        if (j <= i) continue;
        const double bx[4] = {sj[4][jj], sj[5][jj], sj[6][jj], sj[7][jj]};
        const Chain ch = pair_chain<false>(d.g, apx, apy, apz, aE, sj[0][jj], sj[1][jj],
                                           sj[2][jj], sj[3][jj], ax, bx);
        consume<false, MODE>(d, i, j, n, n, ch);
    }
}

template <int MODE>
__global__ void __launch_bounds__(TILE) k_mixed(Device d, long long n1, Cols4 l1,
                                                long long n2, Cols4 l2, long long tiles1) {
    __shared__ double sj[4][TILE];
    const long long ti = blockIdx.x % tiles1;
    const long long tj = blockIdx.x / tiles1;
    const int tid = threadIdx.x;
    const long long j0 = tj * TILE;
    for (int f = 0; f < 4; f++) sj[f][tid] = (j0 + tid < n2) ? l2.p[f][j0 + tid] : 0.0;
    __syncthreads();
    const long long i = ti * TILE + tid;
    if (i >= n1) return;
    const double apx = l1.p[0][i], apy = l1.p[1][i], apz = l1.p[2][i], aE = l1.p[3][i];
    const int jend = (int)min((long long)TILE, n2 - j0);
    for (int jj = 0; jj < jend; jj++) {
        const Chain ch = pair_chain<true>(d.g, apx, apy, apz, aE, sj[0][jj], sj[1][jj],
                                          sj[2][jj], sj[3][jj], nullptr, nullptr);
        consume<true, MODE>(d, i, j0 + jj, n2, n1, ch);
    }
}

// Ordered admission of stream bin b's cut row (row r of the list a8, whose
// pairs run over cols particles: a8 itself after r for same-event lists,
// b4 for mixed-event lists): the first `quota` survivors in pair order, by
// one warp.  A deferred K_phi bin is looked up under key_row * key_cols + j.
template <bool MIXED>
__device__ __forceinline__ void straddle_row(const Device &d, int b, long long r,
                                             long long key_row, long long key_cols,
                                             long long cols, const double *const *a8,
                                             const double *const *b4) {
    const unsigned long long quota = d.caps.quota[b];
    const int lane = threadIdx.x;
    const int ns = d.g.n_slots;
    unsigned long long admitted = 0;
    const double apx = a8[0][r], apy = a8[1][r], apz = a8[2][r], aE = a8[3][r];
    double ax[4] = {0, 0, 0, 0};
    if (!MIXED) {
        ax[0] = a8[4][r];
        ax[1] = a8[5][r];
        ax[2] = a8[6][r];
        ax[3] = a8[7][r];
    }
    const long long jstart = MIXED ? 0 : r + 1;
    for (long long j0 = jstart; j0 < cols && admitted < quota; j0 += 32) {
        const long long j = j0 + lane;
        Chain c;
        c.iK = -1;
        bool has = false;
        int slot = -1;
        if (j < cols) {
            double bx[4] = {0, 0, 0, 0};
            if (!MIXED) {
                bx[0] = a8[4][j];
                bx[1] = a8[5][j];
                bx[2] = a8[6][j];
                bx[3] = a8[7][j];
            }
            const double *const *src = MIXED ? b4 : a8;
            c = pair_chain<MIXED>(d.g, apx, apy, apz, aE, src[0][j], src[1][j], src[2][j],
                                  src[3][j], ax, bx);
            if (c.iK >= 0) {
                if (b >= ns) {
                    has = c.qi_k >= 0 && ns + c.iK == b;
                } else if (c.ev3 == 1) {
                    slot = c.slot;
                    has = slot == b;
                } else if (c.ev3 == 2) {
                    slot = resolved_slot(d, key_row * key_cols + j, c.iK);
                    has = slot == b;
                }
            }
        }
        const unsigned m = __ballot_sync(0xffffffffu, has);
        const unsigned long long rank =
            admitted + __popc(m & ((1u << lane) - 1u));
        if (has && rank < quota) {
            if (b >= ns) {
                if (MIXED)
                    bin_den_qinv(d, c);
                else
                    bin_num_qinv(d, c);
            } else {
                if (MIXED)
                    bin_den3(d, slot, c.bin);
                else
                    bin_num3(d, slot, c.bin, c);
            }
        }
        admitted += __popc(m);
    }
}

// One launch's cut rows, one warp per stream bin.
template <bool MIXED>
__global__ void k_straddle(Device d, long long rows, long long cols, Cols8 a8, Cols4 b4) {
    const int b = blockIdx.x;
    const long long r = d.caps.row_cut[b];
    if (r >= rows) return;
    straddle_row<MIXED>(d, b, r, r, cols, cols, a8.p, b4.p);
}

// The cut rows of several mixed-event jobs admitted together: a stream
// bin's cut row r (in the jobs' joint row order) belongs to the last job
// whose row_base is at most r.
__global__ void k_straddle_jobs(Device d, const StraddleJob *jobs, int n_jobs, long long rows) {
    const int b = blockIdx.x;
    const long long r = d.caps.row_cut[b];
    if (r >= rows) return;
    int lo = 0, hi = n_jobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (jobs[mid].row_base <= r)
            lo = mid;
        else
            hi = mid - 1;
    }
    const StraddleJob &job = jobs[lo];
    straddle_row<true>(d, b, r - job.row_base, r, d.caps.cols_key, job.n2, job.a, job.b);
}

// Per stream bin: first row at which the running survivor count exceeds
// remaining[b]; everything before it is admitted, `quota` more inside it.
__global__ void __launch_bounds__(1024) k_cut(Device d, long long rows,
                                              const unsigned long long *remaining) {
    const int b = blockIdx.x;
    const unsigned long long rem = remaining[b];
    const unsigned *rc = d.caps.rowcnt + (long long)b * rows;
    __shared__ unsigned long long warp_tot[32];
    __shared__ long long found;
    __shared__ unsigned long long found_quota;
    if (threadIdx.x == 0) found = rows;
    unsigned long long running = 0;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (long long base = 0; base < rows; base += 1024) {
        const long long r = base + threadIdx.x;
        const unsigned long long v = r < rows ? rc[r] : 0;
        unsigned long long incl = v;
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        if (lane == 31) warp_tot[w] = incl;
        __syncthreads();
        unsigned long long before = 0;
        for (int k = 0; k < w; k++) before += warp_tot[k];
        incl += before;
        unsigned long long chunk = 0;
        for (int k = 0; k < 32; k++) chunk += warp_tot[k];
        const unsigned long long excl = running + incl - v;
        if (r < rows && running + incl > rem && excl <= rem) {
            // exactly one row satisfies this: the first that crosses rem
            found = r;
            found_quota = rem - excl;
        }
        __syncthreads();
        if (found < rows) break;
        running += chunk;
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        d.caps.row_cut[b] = found;
        d.caps.quota[b] = found < rows ? found_quota : 0ull;
    }
}

// Bins deferred records with their host-resolved K_phi bins (fast mode).
__device__ __forceinline__ void apply_one(const Device &d, const Deferral *rec, const int *iphi,
                                          int k) {
    const int ip = iphi[k];
    if (ip < 0) return;
    const Deferral r = rec[k];
    const long long at = (long long)(r.iK * d.g.n_Kphi + ip) * d.g.q3 + r.bin;
    if (r.mixed) {
        atomicAdd(d.h.den + at, 1ull);
    } else {
        Sums *s = d.h.sums + at;
        atomicAdd(&s->qo, r.qo);
        atomicAdd(&s->qs, r.qs);
        atomicAdd(&s->ql, r.ql);
        atomicAdd(&s->w, r.cosw);
        atomicAdd(d.h.cnt + at, 1ull);
    }
}

__global__ void k_apply(Device d, const Deferral *rec, const int *iphi, int n) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) apply_one(d, rec, iphi, k);
}

// As k_apply, with the number of records read from device memory (decided
// by a host function queued on the same stream).
__global__ void k_apply_n(Device d, const Deferral *rec, const int *iphi, const int *count) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < *count) apply_one(d, rec, iphi, k);
}

// Adds host-resolved deferred pairs to the per-row survivor counts.
__global__ void k_defer_count(Device d, long long rows, long long cols, int n_res) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n_res) return;
    const Resolved rv = d.caps.resolved[k];
    if (rv.iphi < 0) return;
    const long long i = rv.key / cols;
    const int slot = rv.iK * d.g.n_Kphi + rv.iphi;
    atomicAdd(d.caps.rowcnt + (long long)slot * rows + i, 1u);
}

// Pair counters = sums of the count histograms (each counter is
// incremented exactly when a pair is binned).  out: [num slots][den
// slots][num q_inv][den q_inv].
__global__ void __launch_bounds__(256) k_counters(Device d, unsigned long long *out) {
    const int ns = d.g.n_slots, nk = d.g.n_KT;
    const int b = blockIdx.x;
    const u64 *src;
    long long len;
    if (b < ns) {
        src = d.h.cnt + (long long)b * d.g.q3;
        len = d.g.q3;
    } else if (b < 2 * ns) {
        src = d.h.den + (long long)(b - ns) * d.g.q3;
        len = d.g.q3;
    } else if (b < 2 * ns + nk) {
        src = d.h.qi_cnt + (long long)(b - 2 * ns) * d.g.qnpts;
        len = d.g.qnpts;
    } else {
        src = d.h.qi_den + (long long)(b - 2 * ns - nk) * d.g.qnpts;
        len = d.g.qnpts;
    }
    unsigned long long s = 0;
    for (long long k = threadIdx.x; k < len; k += blockDim.x) s += src[k];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    __shared__ unsigned long long ws[8];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long t = 0;
        for (int k = 0; k < 8; k++) t += ws[k];
        out[b] = t;
    }
}

Cols8 cols8(const double *const *c) {
    Cols8 r;
    for (int f = 0; f < 8; f++) r.p[f] = c ? c[f] : nullptr;
    return r;
}
Cols4 cols4(const double *const *c) {
    Cols4 r;
    for (int f = 0; f < 4; f++) r.p[f] = c ? c[f] : nullptr;
    return r;
}

}  // namespace

cudaError_t launch_same(const Device &d, int mode, long long n, const double *const *c8,
                        cudaStream_t st) {
    if (n < 2) return cudaSuccess;
    const long long nt = (n + TILE - 1) / TILE;
    const long long blocks = nt * (nt + 1) / 2;
    if (blocks > 0x7fffffffLL) return cudaErrorInvalidValue;
    const Cols8 c = cols8(c8);
    if (mode == MODE_FAST)
        k_same<MODE_FAST><<<(unsigned)blocks, TILE, 0, st>>>(d, n, c);
    else if (mode == MODE_COUNT)
        k_same<MODE_COUNT><<<(unsigned)blocks, TILE, 0, st>>>(d, n, c);
    else
        k_same<MODE_ORDER><<<(unsigned)blocks, TILE, 0, st>>>(d, n, c);
    return cudaGetLastError();
}

cudaError_t launch_mixed(const Device &d, int mode, long long n1, const double *const *l1,
                         long long n2, const double *const *l2, cudaStream_t st) {
    if (n1 < 1 || n2 < 1) return cudaSuccess;
    const long long t1 = (n1 + TILE - 1) / TILE, t2 = (n2 + TILE - 1) / TILE;
    const long long blocks = t1 * t2;
    if (blocks > 0x7fffffffLL) return cudaErrorInvalidValue;
    const Cols4 a = cols4(l1), b = cols4(l2);
    if (mode == MODE_FAST)
        k_mixed<MODE_FAST><<<(unsigned)blocks, TILE, 0, st>>>(d, n1, a, n2, b, t1);
    else if (mode == MODE_COUNT)
        k_mixed<MODE_COUNT><<<(unsigned)blocks, TILE, 0, st>>>(d, n1, a, n2, b, t1);
    else
        k_mixed<MODE_ORDER><<<(unsigned)blocks, TILE, 0, st>>>(d, n1, a, n2, b, t1);
    return cudaGetLastError();
}

cudaError_t launch_same_straddle(const Device &d, long long n, const double *const *c8,
                                 int n_stream, cudaStream_t st) {
    k_straddle<false><<<n_stream, 32, 0, st>>>(d, n, n, cols8(c8), cols4(nullptr));
    return cudaGetLastError();
}

cudaError_t launch_mixed_straddle(const Device &d, long long n1, const double *const *l1,
                                  long long n2, const double *const *l2, int n_stream,
                                  cudaStream_t st) {
    Cols8 a;
    for (int f = 0; f < 8; f++) a.p[f] = f < 4 ? l1[f] : nullptr;
    k_straddle<true><<<n_stream, 32, 0, st>>>(d, n1, n2, a, cols4(l2));
    return cudaGetLastError();
}

cudaError_t launch_jobs_straddle(const Device &d, const StraddleJob *jobs, int n_jobs,
                                 long long rows, int n_stream, cudaStream_t st) {
    if (n_jobs < 1) return cudaSuccess;
    k_straddle_jobs<<<n_stream, 32, 0, st>>>(d, jobs, n_jobs, rows);
    return cudaGetLastError();
}

cudaError_t launch_cut(const Device &d, long long rows, int n_stream,
                       const unsigned long long *remaining, cudaStream_t st) {
    k_cut<<<n_stream, 1024, 0, st>>>(d, rows, remaining);
    return cudaGetLastError();
}

cudaError_t launch_apply(const Device &d, const Deferral *rec, const int *iphi, int n,
                         cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    k_apply<<<(n + 127) / 128, 128, 0, st>>>(d, rec, iphi, n);
    return cudaGetLastError();
}

cudaError_t launch_apply_n(const Device &d, const Deferral *rec, const int *iphi, const int *count,
                           int cap, cudaStream_t st) {
    k_apply_n<<<(cap + 127) / 128, 128, 0, st>>>(d, rec, iphi, count);
    return cudaGetLastError();
}

cudaError_t launch_defer_count(const Device &d, long long rows, long long cols, int n_res,
                               cudaStream_t st) {
    if (n_res <= 0) return cudaSuccess;
    k_defer_count<<<(n_res + 127) / 128, 128, 0, st>>>(d, rows, cols, n_res);
    return cudaGetLastError();
}

__global__ void __launch_bounds__(256) k_export(Device d, int field, double *out,
                                                long long nbins) {
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < nbins;
         k += (long long)gridDim.x * blockDim.x) {
        double v;
        switch (field) {
            case 0: v = d.h.sums[k].qo; break;
            case 1: v = d.h.sums[k].qs; break;
            case 2: v = d.h.sums[k].ql; break;
            case 3: v = d.h.sums[k].w; break;
            case 4: v = (double)d.h.cnt[k]; break;
            default: v = (double)d.h.den[k]; break;
        }
        out[k] = v;
    }
}

cudaError_t launch_export(const Device &d, int field, double *out, long long nbins,
                          cudaStream_t st) {
    const long long blocks = std::min<long long>((nbins + 255) / 256, 152 * 16);
    k_export<<<(unsigned)std::max<long long>(blocks, 1), 256, 0, st>>>(d, field, out, nbins);
    return cudaGetLastError();
}

cudaError_t launch_counters(const Device &d, unsigned long long *out, cudaStream_t st) {
    k_counters<<<2 * d.g.n_slots + 2 * d.g.n_KT, 256, 0, st>>>(d, out);
    return cudaGetLastError();
}

}  // namespace hbt
