// C ABI of the HBT pair-binning engine (include/hbt_gpu.h).
//
// Owns the device histograms of one analysis, stages host particle lists
// into HBM, chooses per launch between the fast path (no pair cap can bind)
// and ordered cap admission, and decides the few K_phi bins that lie on a
// bin edge with the C library's atan2 (as the reference does,
// src/HBT_correlation.cpp:408-416).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include "../../include/hbt_gpu.h"
#include "hbt_batch.cuh"
#include "hbt_engine.cuh"
#include "hbt_internal.h"
#include "hbt_runner.h"

using hbt::u64;

namespace {

const unsigned kDeferCap = 1u << 16;
const u64 kInf = ~0ull;

struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
};

}  // namespace

// FP32-weight form: same-event tile pairs (at most 128 x 128 pairs each)
// between two merges of the FP32 partials into the FP64 bins, and the
// largest value a tuning may set.  The partials' rounding grows with the
// pairs a partial bin takes between merges (about linearly: the cos terms
// a busy bin takes are alike, so their roundings add up rather than
// cancel).  On the central workload, with one partial array, the worst
// numerator error per pair reached 1.05e-6 with 8192 (the work items' queue
// order, and so each chunk's items, vary from run to run), above the
// form's 1e-6 bound; the two partial arrays (partials_of) halve it.
constexpr int kMergeChunk = 8192;

struct hbt_ctx {
    hbt_params prm;
    int device = 0;
    cudaStream_t own = nullptr, stream = nullptr;
    cudaEvent_t staged = nullptr;
    // stream-ordered allocation from this pool on `own` (serving loop
    // contexts); nullptr: cudaMalloc / cudaFree
    cudaMemPool_t pool = nullptr;
    hbt::Device d;
    u64 cap = 0, cap_qinv = 0;
    int n_stream = 0;  // 3-D slots + q_inv K_T bins
    // histograms
    DevBuf sums, cnt, den, qi_sums, qi_cnt, qi_den, stats, defer, n_defer;
    // FP32-weight form: partial sums and Kahan compensation
    DevBuf part, comp;
    // batched path: tables, sorted particle table, sort scratch, boxes, queue
    hbt::BatchRunner runner;
    int persistent_grid = 152 * 4;
    int sms = 152, max_blocks_per_sm = 5;
    hbt_tuning tune = {0, 0.02, 0.05, kMergeChunk, 1, 0, 1};
    // ordered admission scratch
    DevBuf rowcnt, row_cut, quota, remaining, resolved, counters, apply_iphi, straddle_jobs,
        slot_full;
    // input staging, two buffers in turn: the host-to-device copy of a call
    // runs on `copy_in` while the binning of the previous call still reads
    // the other buffer (in_free: recorded on `stream` after that binning)
    DevBuf in[2];
    int in_next = 0, in_cur = -1;
    bool in_used[2] = {false, false};
    cudaStream_t copy_in = nullptr;
    cudaEvent_t in_free[2] = {nullptr, nullptr};
    // readback: two FP64 arrays of the histogram size, used in turn
    DevBuf exp;
    // overlapped readback (hbt_read_hist_async): a snapshot of the six
    // arrays and the error flag, copied to the host on `copy` while later
    // work runs on `stream`
    DevBuf snap;
    cudaStream_t copy = nullptr;
    cudaEvent_t snap_ev = nullptr, copy_ev = nullptr;
    u64 *flag_host = nullptr;  // pinned
    bool read_pending = false;
    // upper bounds of the four counter families (num 3-D, den 3-D, num
    // q_inv, den q_inv): max counter <= bound
    u64 ub[4] = {0, 0, 0, 0};
    hbt_stats st;
    std::string err;
    // allocation-failure injection (hbt_inject_alloc_failure): allocations
    // left to succeed before one fails; -1 = off
    int fail_after = -1;
    // stream-ordered K_phi deferral drain (drain_deferrals_async): pinned
    // copies of the deferral count and records, the host-decided bins
    // ([0] = records to apply, [4 + k] = bin of record k) and their device
    // copy; pairs decided by queued host functions
    unsigned *count_host = nullptr;
    hbt::Deferral *defer_host = nullptr;
    int *apply_host = nullptr;
    DevBuf apply_dev;
    std::atomic<unsigned long long> deferred_async{0};
};

namespace {

hbt_status fail(hbt_ctx *c, hbt_status s, const std::string &msg) {
    if (c) c->err = msg;
    return s;
}

#define CU(call)                                                                     \
    do {                                                                             \
        cudaError_t e_ = (call);                                                     \
        if (e_ != cudaSuccess)                                                       \
            return fail(c, HBT_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

#define TRY(expr)                          \
    do {                                   \
        hbt_status s_ = (expr);            \
        if (s_ != HBT_OK) return s_;       \
    } while (0)

void dfree(hbt_ctx *c, DevBuf &b) {
    if (b.p) {
        if (c->pool)
            cudaFreeAsync(b.p, c->own);
        else
            cudaFree(b.p);
    }
    b.p = nullptr;
    b.bytes = 0;
}

hbt_status dalloc(hbt_ctx *c, DevBuf &b, size_t bytes) {
    if (b.bytes >= bytes && b.p) return HBT_OK;
    dfree(c, b);
    if (bytes == 0) return HBT_OK;
    if (c->fail_after >= 0 && c->fail_after-- == 0)
        return fail(c, HBT_ERR_NOMEM, "device allocation failed (injected)");
    cudaError_t e = c->pool ? cudaMallocFromPoolAsync(&b.p, bytes, c->pool, c->own)
                            : cudaMalloc(&b.p, bytes);
    if (e != cudaSuccess) {
        b.p = nullptr;
        return fail(c, HBT_ERR_NOMEM, "device allocation failed");
    }
    b.bytes = bytes;
    return HBT_OK;
}

template <class T>
T *ptr(DevBuf &b) {
    return static_cast<T *>(b.p);
}

void refresh_device(hbt_ctx *c) {
    c->d.h.sums = ptr<hbt::Sums>(c->sums);
    c->d.h.cnt = ptr<u64>(c->cnt);
    c->d.h.den = ptr<u64>(c->den);
    c->d.h.qi_sums = ptr<hbt::QiSums>(c->qi_sums);
    c->d.h.qi_cnt = ptr<u64>(c->qi_cnt);
    c->d.h.qi_den = ptr<u64>(c->qi_den);
    c->d.stats = ptr<u64>(c->stats);
    c->d.defer = ptr<hbt::Deferral>(c->defer);
    c->d.n_defer = ptr<unsigned>(c->n_defer);
    c->d.defer_cap = kDeferCap;
    c->d.caps.rowcnt = ptr<unsigned>(c->rowcnt);
    c->d.caps.row_cut = ptr<long long>(c->row_cut);
    c->d.caps.quota = ptr<unsigned long long>(c->quota);
    c->d.caps.resolved = ptr<hbt::Resolved>(c->resolved);
    c->d.part = ptr<float4>(c->part);
    // the second partial array follows the first (same length)
    c->d.part_b = c->d.part ? c->d.part + (size_t)c->d.g.n_slots * c->d.g.q3 : nullptr;
    c->d.comp = ptr<hbt::Sums>(c->comp);
}

// Reference K_phi decision on the host (src/HBT_correlation.cpp:408-416).
int host_kphi(const hbt::Grid &g, double Kx, double Ky, double psi_ref) {
    const double phi = atan2(Ky, Kx);
    double d = phi - psi_ref;
    while (d < 0.) d += 2. * M_PI;
    while (d > 2. * M_PI) d -= 2. * M_PI;
    const int ip = static_cast<int>(d / g.dKphi);
    if (ip < 0 || ip >= g.n_Kphi) return -1;
    return ip;
}

// True when c + P - 1 <= limit (all of P more admissions pass `<= limit`).
bool fits_le(u64 c, u64 P, u64 limit) {
    if (P == 0) return true;
    if (c > limit) return false;
    return P - 1 <= limit - c;
}

hbt_status read_defer_count(hbt_ctx *c, unsigned *n) {
    CU(cudaMemcpyAsync(n, c->n_defer.p, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    return HBT_OK;
}

// Bins the fast-mode deferrals collected so far (each record carries its
// kind and the psi_ref of its launch, so they can wait until the
// histograms or counters are read).
hbt_status drain_deferrals(hbt_ctx *c) {
    if (!c->prm.azimuthal_flag) return HBT_OK;
    unsigned n = 0;
    TRY(read_defer_count(c, &n));
    if (n == 0) return HBT_OK;
    if (n > kDeferCap) return fail(c, HBT_ERR_DEVICE, "K_phi deferral buffer overflow");
    std::vector<hbt::Deferral> rec(n);
    CU(cudaMemcpyAsync(rec.data(), c->defer.p, n * sizeof(hbt::Deferral),
                       cudaMemcpyDeviceToHost, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    std::vector<int> iphi(n);
    for (unsigned k = 0; k < n; k++)
        iphi[k] = host_kphi(c->d.g, rec[k].Kx, rec[k].Ky, rec[k].psi);
    TRY(dalloc(c, c->apply_iphi, n * sizeof(int)));
    CU(cudaMemcpyAsync(c->apply_iphi.p, iphi.data(), n * sizeof(int), cudaMemcpyHostToDevice,
                       c->stream));
    CU(hbt::launch_apply(c->d, ptr<hbt::Deferral>(c->defer), ptr<int>(c->apply_iphi), (int)n,
                         c->stream));
    CU(cudaMemsetAsync(c->n_defer.p, 0, sizeof(unsigned), c->stream));
    CU(cudaStreamSynchronize(c->stream));
    c->st.deferred_kphi += n;
    c->st.launches++;
    return HBT_OK;
}

// Host function queued on the context's stream by drain_deferrals_async:
// decides the copied records' K_phi bins with the C library's atan2.  Makes
// no CUDA call.  An overflowing buffer applies nothing (the kernels raised
// the error flag, which the reads report).
void CUDART_CB decide_deferrals(void *arg) {
    hbt_ctx *c = static_cast<hbt_ctx *>(arg);
    const unsigned n = *c->count_host;
    const unsigned m = n > kDeferCap ? 0u : n;
    for (unsigned k = 0; k < m; k++) {
        const hbt::Deferral &r = c->defer_host[k];
        c->apply_host[4 + k] = host_kphi(c->d.g, r.Kx, r.Ky, r.psi);
    }
    c->apply_host[0] = (int)m;
    c->deferred_async += m;
}

// drain_deferrals without waiting: the count and records are copied to
// pinned host memory, a host function decides the bins, and the apply
// kernel runs after it, all in the context's stream order, so the caller
// returns while the binning before it is still running.  Serving contexts
// (memory from a pool) take the waiting path.
hbt_status drain_deferrals_async(hbt_ctx *c) {
    if (!c->prm.azimuthal_flag) return HBT_OK;
    if (c->pool) return drain_deferrals(c);
    if (!c->count_host) {
        CU(cudaMallocHost(&c->count_host, sizeof(unsigned)));
        CU(cudaMallocHost(&c->defer_host, kDeferCap * sizeof(hbt::Deferral)));
        CU(cudaMallocHost(&c->apply_host, (4 + kDeferCap) * sizeof(int)));
    }
    TRY(dalloc(c, c->apply_dev, (4 + kDeferCap) * sizeof(int)));
    CU(cudaMemcpyAsync(c->count_host, c->n_defer.p, sizeof(unsigned), cudaMemcpyDeviceToHost,
                       c->stream));
    CU(cudaMemcpyAsync(c->defer_host, c->defer.p, kDeferCap * sizeof(hbt::Deferral),
                       cudaMemcpyDeviceToHost, c->stream));
    CU(cudaLaunchHostFunc(c->stream, decide_deferrals, c));
    CU(cudaMemcpyAsync(c->apply_dev.p, c->apply_host, (4 + kDeferCap) * sizeof(int),
                       cudaMemcpyHostToDevice, c->stream));
    const int *dev = ptr<int>(c->apply_dev);
    CU(hbt::launch_apply_n(c->d, ptr<hbt::Deferral>(c->defer), dev + 4, dev, (int)kDeferCap,
                           c->stream));
    CU(cudaMemsetAsync(c->n_defer.p, 0, sizeof(unsigned), c->stream));
    c->st.launches++;
    return HBT_OK;
}

// Exact counters: [num slots][den slots][num q_inv][den q_inv].
hbt_status read_counters(hbt_ctx *c, std::vector<u64> &out) {
    const int ns = c->d.g.n_slots, nk = c->d.g.n_KT;
    const size_t n = 2 * ns + 2 * nk;
    TRY(dalloc(c, c->counters, n * sizeof(u64)));
    CU(hbt::launch_counters(c->d, ptr<unsigned long long>(c->counters), c->stream));
    out.assign(n, 0);
    CU(cudaMemcpyAsync(out.data(), c->counters.p, n * sizeof(u64), cudaMemcpyDeviceToHost,
                       c->stream));
    CU(cudaStreamSynchronize(c->stream));
    c->st.launches++;
    // tighten the upper bounds
    for (int f = 0; f < 4; f++) c->ub[f] = 0;
    for (int s = 0; s < ns; s++) {
        c->ub[0] = std::max(c->ub[0], out[s]);
        c->ub[1] = std::max(c->ub[1], out[ns + s]);
    }
    for (int k = 0; k < nk; k++) {
        c->ub[2] = std::max(c->ub[2], out[2 * ns + k]);
        c->ub[3] = std::max(c->ub[3], out[2 * ns + nk + k]);
    }
    return HBT_OK;
}

// Can any cap reject one of P more pairs of this kind?  `mixed` selects the
// denominator families.
bool caps_may_bind(const hbt_ctx *c, int mixed, u64 P) {
    const u64 ub3 = c->ub[mixed ? 1 : 0], ubq = c->ub[mixed ? 3 : 2];
    if (!fits_le(ub3, P, c->cap)) return true;
    if (c->prm.invariant_radius_flag == 1) {
        if (c->cap_qinv == 0) return true;
        if (!fits_le(ubq, P, c->cap_qinv - 1)) return true;
    }
    return false;
}

hbt_status run_fast_jobs(hbt_ctx *c, std::vector<hbt::FastJob> jobs, int mode = hbt::MODE_FAST);
bool batched_ok(const hbt_ctx *c);

// After a count pass with K_phi bins: the pairs deferred to the host (K_phi
// within kphi_defer_tol of an edge) get their bins from the C library's
// atan2 here, are added to the row counts, and are looked up by the order
// pass and the straddle kernel under key row * cols + column.
hbt_status resolve_count_deferrals(hbt_ctx *c, long long rows, long long cols) {
    if (!c->prm.azimuthal_flag) return HBT_OK;
    unsigned n = 0;
    TRY(read_defer_count(c, &n));
    if (n > kDeferCap) return fail(c, HBT_ERR_DEVICE, "K_phi deferral buffer overflow");
    if (n > 0) {
        std::vector<hbt::Deferral> rec(n);
        CU(cudaMemcpyAsync(rec.data(), c->defer.p, n * sizeof(hbt::Deferral),
                           cudaMemcpyDeviceToHost, c->stream));
        CU(cudaStreamSynchronize(c->stream));
        std::vector<hbt::Resolved> res(n);
        for (unsigned k = 0; k < n; k++) {
            res[k].key = rec[k].i * cols + rec[k].j;
            res[k].iphi = host_kphi(c->d.g, rec[k].Kx, rec[k].Ky, rec[k].psi);
            res[k].iK = rec[k].iK;
        }
        std::sort(res.begin(), res.end(),
                  [](const hbt::Resolved &x, const hbt::Resolved &y) { return x.key < y.key; });
        TRY(dalloc(c, c->resolved, n * sizeof(hbt::Resolved)));
        refresh_device(c);
        CU(cudaMemcpyAsync(c->resolved.p, res.data(), n * sizeof(hbt::Resolved),
                           cudaMemcpyHostToDevice, c->stream));
        c->d.caps.n_resolved = (int)n;
        CU(hbt::launch_defer_count(c->d, rows, cols, (int)n, c->stream));
        c->st.deferred_kphi += n;
        c->st.launches++;
    }
    CU(cudaMemsetAsync(c->n_defer.p, 0, sizeof(unsigned), c->stream));
    return HBT_OK;
}

// Remaining admissions per stream bin of one counter family (mixed = 0:
// numerators, 1: denominators), from the counters read back: cap - count
// + 1 (a counter may pass the cap by one, as the reference's test is
// `count > cap`), 0 for a full bin, unlimited for bins without a cap.
std::vector<u64> remaining_of(const hbt_ctx *c, int mixed, const std::vector<u64> &ctr) {
    const int ns = c->d.g.n_slots, nk = c->d.g.n_KT, nst = c->n_stream;
    std::vector<u64> rem(nst, kInf);
    for (int s = 0; s < ns; s++) {
        const u64 v = ctr[(mixed ? ns : 0) + s];
        if (v > c->cap)
            rem[s] = 0;
        else
            rem[s] = (c->cap - v == kInf) ? kInf : c->cap - v + 1;
    }
    for (int k = 0; k < nk; k++) {
        const u64 v = ctr[2 * ns + (mixed ? nk : 0) + k];
        rem[ns + k] = (c->prm.invariant_radius_flag == 1) ? (v < c->cap_qinv ? c->cap_qinv - v : 0)
                                                          : kInf;
    }
    return rem;
}

// Uploads which 3-D slots have no admission left (rem[s] == 0) for the
// batched passes' cull (Caps::slot_full); the caller clears it afterwards.
hbt_status set_slot_full(hbt_ctx *c, const std::vector<u64> &rem) {
    const int ns = c->d.g.n_slots;
    std::vector<unsigned char> full(ns);
    bool any = false;
    for (int s = 0; s < ns; s++) {
        full[s] = rem[s] == 0 ? 1 : 0;
        any = any || full[s];
    }
    if (!any) return HBT_OK;
    TRY(dalloc(c, c->slot_full, ns));
    CU(cudaMemcpyAsync(c->slot_full.p, full.data(), ns, cudaMemcpyHostToDevice, c->stream));
    // the copy reads the host vector before it goes out of scope
    CU(cudaStreamSynchronize(c->stream));
    c->d.caps.slot_full = ptr<unsigned char>(c->slot_full);
    return HBT_OK;
}

// Clears Caps::slot_full when an ordered pass ends, on every return path.
struct SlotFullScope {
    hbt::Caps &caps;
    ~SlotFullScope() { caps.slot_full = nullptr; }
};

// Ordered admission for one launch (same-event: mixed = 0).  The two
// passes over every pair (COUNT: survivors per stream bin and row; ORDER:
// the rows before each bin's cut) run on the batched screened kernels when
// the context uses them, else on the reference-chain kernels; the cut row
// of each bin is admitted pair by pair in the reference's order
// (k_straddle).
hbt_status ordered_launch(hbt_ctx *c, int mixed, long long rows, long long cols,
                          const double *const *a, const double *const *b) {
    // (the batched kernels' admission passes cover the 3-D histograms; with
    // the q_inv histograms the reference-chain kernels run both passes)
    const bool batched = batched_ok(c) && !c->d.g.qinv;
    hbt::FastJob job = {};
    job.kind = mixed;
    job.na = rows;
    job.nb = mixed ? cols : 0;
    for (int f = 0; f < (mixed ? 4 : 8); f++) job.a[f] = a[f];
    if (mixed)
        for (int f = 0; f < 4; f++) job.b[f] = b[f];
    TRY(drain_deferrals(c));
    std::vector<u64> ctr;
    TRY(read_counters(c, ctr));
    const int nst = c->n_stream;
    const std::vector<u64> rem = remaining_of(c, mixed, ctr);
    TRY(dalloc(c, c->rowcnt, (size_t)nst * rows * sizeof(unsigned)));
    TRY(dalloc(c, c->row_cut, nst * sizeof(long long)));
    TRY(dalloc(c, c->quota, nst * sizeof(u64)));
    TRY(dalloc(c, c->remaining, nst * sizeof(u64)));
    refresh_device(c);
    // the batched passes skip tile pairs that reach only full slots
    SlotFullScope slot_scope{c->d.caps};
    if (batched) TRY(set_slot_full(c, rem));
    c->d.caps.n_resolved = 0;
    CU(cudaMemsetAsync(c->rowcnt.p, 0, (size_t)nst * rows * sizeof(unsigned), c->stream));
    CU(cudaMemsetAsync(c->n_defer.p, 0, sizeof(unsigned), c->stream));
    // pass A: survivors per (stream bin, row)
    if (batched) {
        TRY(run_fast_jobs(c, std::vector<hbt::FastJob>{job}, hbt::MODE_COUNT));
    } else {
        if (mixed)
            CU(hbt::launch_mixed(c->d, hbt::MODE_COUNT, rows, a, cols, b, c->stream));
        else
            CU(hbt::launch_same(c->d, hbt::MODE_COUNT, rows, a, c->stream));
        c->st.launches++;
    }
    TRY(resolve_count_deferrals(c, rows, cols));
    CU(cudaMemcpyAsync(c->remaining.p, rem.data(), nst * sizeof(u64), cudaMemcpyHostToDevice,
                       c->stream));
    CU(hbt::launch_cut(c->d, rows, nst, ptr<unsigned long long>(c->remaining), c->stream));
    // pass B: rows before each cut, then the cut rows in pair order
    if (batched) {
        TRY(run_fast_jobs(c, std::vector<hbt::FastJob>{job}, hbt::MODE_ORDER));
    } else {
        if (mixed)
            CU(hbt::launch_mixed(c->d, hbt::MODE_ORDER, rows, a, cols, b, c->stream));
        else
            CU(hbt::launch_same(c->d, hbt::MODE_ORDER, rows, a, c->stream));
        c->st.launches++;
    }
    if (mixed)
        CU(hbt::launch_mixed_straddle(c->d, rows, a, cols, b, nst, c->stream));
    else
        CU(hbt::launch_same_straddle(c->d, rows, a, nst, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    c->st.launches += 2;
    c->st.ordered_passes++;
    c->d.caps.n_resolved = 0;
    return HBT_OK;
}

// Ordered admission of several mixed-event jobs at once, in the reference's
// order (src/HBT_correlation.cpp:199-216: the events in turn, each against
// its partners; within a job the pairs by list-1 row, then list-2 column).
// The jobs' rows are numbered jointly (a job's first row is the number of
// list-1 particles of the jobs before it), so that one count pass, one cut
// per stream bin and one order pass on the batched kernels admit exactly the
// pairs that job-by-job admission would, and each stream bin's cut row is
// admitted pair by pair inside its own job (k_straddle_jobs).  Batched
// kernels without q_inv histograms only (the callers check).
hbt_status ordered_launch_mixed_jobs(hbt_ctx *c, const std::vector<hbt::FastJob> &in) {
    std::vector<hbt::FastJob> jobs;
    std::vector<hbt::StraddleJob> sj;
    long long rows = 0, cols = 0;
    for (hbt::FastJob j : in) {
        if (j.kind != 1 || j.na < 1 || j.nb < 1) continue;
        j.row_base = rows;
        hbt::StraddleJob t = {};
        for (int f = 0; f < 4; f++) {
            t.a[f] = j.a[f];
            t.b[f] = j.b[f];
        }
        t.n1 = j.na;
        t.n2 = j.nb;
        t.row_base = rows;
        jobs.push_back(j);
        sj.push_back(t);
        rows += j.na;
        cols = std::max(cols, j.nb);
    }
    if (jobs.empty()) return HBT_OK;
    TRY(drain_deferrals(c));
    std::vector<u64> ctr;
    TRY(read_counters(c, ctr));
    const int nst = c->n_stream;
    const std::vector<u64> rem = remaining_of(c, 1, ctr);
    TRY(dalloc(c, c->rowcnt, (size_t)nst * rows * sizeof(unsigned)));
    TRY(dalloc(c, c->row_cut, nst * sizeof(long long)));
    TRY(dalloc(c, c->quota, nst * sizeof(u64)));
    TRY(dalloc(c, c->remaining, nst * sizeof(u64)));
    TRY(dalloc(c, c->straddle_jobs, sj.size() * sizeof(hbt::StraddleJob)));
    refresh_device(c);
    // the joint row numbering holds for the two passes and the straddle only
    struct JointRows {
        hbt::Caps &caps;
        ~JointRows() {
            caps.rows_total = caps.cols_key = 0;
            caps.n_resolved = 0;
        }
    } joint{c->d.caps};
    SlotFullScope slot_scope{c->d.caps};
    TRY(set_slot_full(c, rem));
    c->d.caps.n_resolved = 0;
    c->d.caps.rows_total = rows;
    c->d.caps.cols_key = cols;
    CU(cudaMemsetAsync(c->rowcnt.p, 0, (size_t)nst * rows * sizeof(unsigned), c->stream));
    CU(cudaMemsetAsync(c->n_defer.p, 0, sizeof(unsigned), c->stream));
    CU(cudaMemcpyAsync(c->straddle_jobs.p, sj.data(), sj.size() * sizeof(hbt::StraddleJob),
                       cudaMemcpyHostToDevice, c->stream));
    TRY(run_fast_jobs(c, jobs, hbt::MODE_COUNT));
    TRY(resolve_count_deferrals(c, rows, cols));
    CU(cudaMemcpyAsync(c->remaining.p, rem.data(), nst * sizeof(u64), cudaMemcpyHostToDevice,
                       c->stream));
    CU(hbt::launch_cut(c->d, rows, nst, ptr<unsigned long long>(c->remaining), c->stream));
    TRY(run_fast_jobs(c, jobs, hbt::MODE_ORDER));
    CU(hbt::launch_jobs_straddle(c->d, ptr<hbt::StraddleJob>(c->straddle_jobs), (int)sj.size(),
                                 rows, nst, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    c->st.launches += 2;
    c->st.ordered_passes++;
    return HBT_OK;
}

// FP32 copies of the screen constants with their rounding slack.
void fill_screen(hbt_ctx *c) { hbt::screen_from_grid(c->d.g, c->d.s); }

// The screened kernels decide bins in FP32 with error bounds; the q_inv
// histograms are screened on the batched path only.
bool screened_ok(const hbt_ctx *c) {
    return (c->prm.kernel == HBT_KERNEL_SCREENED ||
            (c->prm.kernel == HBT_KERNEL_SCREENED_GRID && !c->d.g.qinv)) &&
           c->d.g.n_KT <= 255 && c->d.g.qnpts <= 1024 && c->d.g.n_slots < 16384;
}

bool batched_ok(const hbt_ctx *c) {
    return screened_ok(c) && c->prm.kernel == HBT_KERNEL_SCREENED;
}

using hbt::FastJob;

// The batched path's launch shape from the context's tuning.
hbt::Tuning runner_tuning(const hbt_ctx *c, const hbt_tuning &t) {
    hbt::Tuning r;
    // 0: each persistent kernel at its own occupancy
    r.grid = t.blocks_per_sm > 0 ? c->sms * std::min(t.blocks_per_sm, 8) : 0;
    r.chunk = c->d.precision == HBT_PRECISION_FP32W ? (unsigned)t.merge_chunk : 0u;
    r.cell_pt = t.cell_pt;
    r.cell_y = t.cell_y;
    r.graph = t.use_graph != 0;
    r.time_kernels = t.time_kernels != 0;
    // the FP32-weight form keeps the cull's order: in region order a merge
    // chunk's pairs crowd into fewer bins and the FP32 partials' rounding
    // reached 3e-6 per pair on the central workload, above the form's bound
    r.order_items = t.order_items != 0 && c->d.precision != HBT_PRECISION_FP32W;
    return r;
}

// Sort, cull and bin fast jobs of this analysis in one persistent launch
// (mode: MODE_FAST, or a pass of ordered cap admission).
hbt_status run_fast_jobs(hbt_ctx *c, std::vector<FastJob> jobs, int mode) {
    const double Q = std::max(std::fabs(c->d.g.q_lo), std::fabs(c->d.g.q_hi));
    for (FastJob &j : jobs) {
        j.dev = 0;
        j.q_window = Q;
        j.boost = c->d.g.boost;
        j.qinv = c->d.g.qinv;
    }
    std::string err;
    if (!c->runner.run(jobs, c->d, runner_tuning(c, c->tune), c->stream, err, mode))
        return fail(c, HBT_ERR_CUDA, err);
    c->st.launches += 6;
    if (c->runner.last_graph_reuse() == 0) c->st.graph_captures++;
    if (c->runner.last_graph_reuse() == 1) c->st.graph_replays++;
    return HBT_OK;
}

// Device-array jobs of the C ABI as batch jobs.
std::vector<FastJob> fast_jobs_of(int32_t n_jobs, const hbt_job *jobs) {
    std::vector<FastJob> fj;
    for (int k = 0; k < n_jobs; k++) {
        const hbt_job &j = jobs[k];
        FastJob f = {};
        f.kind = j.kind;
        f.na = j.na;
        f.nb = j.nb;
        const double *a[8] = {j.a.px, j.a.py, j.a.pz, j.a.E, j.a.x, j.a.y, j.a.z, j.a.t};
        for (int q = 0; q < 8; q++) f.a[q] = a[q];
        const double *b[4] = {j.b.px, j.b.py, j.b.pz, j.b.E};
        for (int q = 0; q < 4; q++) f.b[q] = b[q];
        fj.push_back(f);
    }
    return fj;
}

bool tuning_valid(const hbt_tuning &t) {
    return t.blocks_per_sm >= 0 && t.cell_pt >= 0.0 && t.cell_y >= 0.0 && t.merge_chunk >= 0 &&
           t.merge_chunk <= kMergeChunk && (t.use_graph == 0 || t.use_graph == 1) &&
           (t.time_kernels == 0 || t.time_kernels == 1) &&
           (t.order_items == 0 || t.order_items == 1);
}

hbt_tuning tuning_defaults(hbt_tuning t) {
    if (t.cell_pt == 0.0) t.cell_pt = 0.02;
    if (t.cell_y == 0.0) t.cell_y = 0.05;
    if (t.merge_chunk == 0) t.merge_chunk = kMergeChunk;
    return t;
}

hbt_status bin_same_device(hbt_ctx *c, long long n, const double *const *c8) {
    if (n < 2) return HBT_OK;
    const u64 P = (u64)n * (u64)(n - 1) / 2;
    c->st.pairs_same += P;
    bool may_bind = caps_may_bind(c, 0, P);
    if (may_bind) {
        TRY(drain_deferrals(c));
        std::vector<u64> ctr;
        TRY(read_counters(c, ctr));
        may_bind = caps_may_bind(c, 0, P);
    }
    if (may_bind) {
        TRY(ordered_launch(c, 0, n, n, c8, nullptr));
        std::vector<u64> ctr;
        TRY(read_counters(c, ctr));
    } else {
        if (batched_ok(c)) {
            FastJob j = {};
            j.kind = 0;
            j.na = n;
            for (int f = 0; f < 8; f++) j.a[f] = c8[f];
            TRY(run_fast_jobs(c, std::vector<FastJob>{j}));
        } else if (screened_ok(c)) {
            CU(hbt::launch_same_fast(c->d, n, c8, c->stream));
        } else {
            CU(hbt::launch_same(c->d, hbt::MODE_FAST, n, c8, c->stream));
        }
        c->st.launches++;
        c->ub[0] += P;
        if (c->prm.invariant_radius_flag == 1) c->ub[2] += P;
    }
    return HBT_OK;
}

hbt_status bin_mixed_device(hbt_ctx *c, long long n1, const double *const *l1, long long n2,
                            const double *const *l2) {
    if (n1 < 1 || n2 < 1) return HBT_OK;
    const u64 P = (u64)n1 * (u64)n2;
    c->st.pairs_mixed += P;
    bool may_bind = caps_may_bind(c, 1, P);
    if (may_bind) {
        TRY(drain_deferrals(c));
        std::vector<u64> ctr;
        TRY(read_counters(c, ctr));
        may_bind = caps_may_bind(c, 1, P);
    }
    if (may_bind) {
        TRY(ordered_launch(c, 1, n1, n2, l1, l2));
        std::vector<u64> ctr;
        TRY(read_counters(c, ctr));
    } else {
        if (batched_ok(c)) {
            FastJob j = {};
            j.kind = 1;
            j.na = n1;
            j.nb = n2;
            for (int f = 0; f < 4; f++) {
                j.a[f] = l1[f];
                j.b[f] = l2[f];
            }
            TRY(run_fast_jobs(c, std::vector<FastJob>{j}));
        } else if (screened_ok(c)) {
            CU(hbt::launch_mixed_fast(c->d, n1, l1, n2, l2, c->stream));
        } else {
            CU(hbt::launch_mixed(c->d, hbt::MODE_FAST, n1, l1, n2, l2, c->stream));
        }
        c->st.launches++;
        c->ub[1] += P;
        if (c->prm.invariant_radius_flag == 1) c->ub[3] += P;
    }
    return HBT_OK;
}

// Copies host columns into a staging buffer; returns device pointers.  The
// copies run on the context's copy stream into the buffer the previous call
// did not use, so they overlap that call's binning; the call returns once
// the copies are done (the caller may then reuse its arrays).  Serving
// contexts, whose memory comes stream-ordered from a pool, copy on their
// own stream.
hbt_status stage(hbt_ctx *c, const double *const *src, const long long *len, int ncols,
                 const double **dst) {
    if (!c->copy_in && !c->pool) {
        CU(cudaStreamCreateWithFlags(&c->copy_in, cudaStreamNonBlocking));
        for (cudaEvent_t &e : c->in_free) CU(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
    cudaStream_t cs = c->pool ? c->stream : c->copy_in;
    const int buf = c->pool ? 0 : c->in_next;
    size_t total = 0;
    for (int f = 0; f < ncols; f++) total += (size_t)((len[f] + 31) / 32 * 32);
    TRY(dalloc(c, c->in[buf], total * sizeof(double)));
    double *base = ptr<double>(c->in[buf]);
    // the binning that read this buffer last must be done with it
    if (!c->pool && c->in_used[buf]) CU(cudaStreamWaitEvent(cs, c->in_free[buf], 0));
    size_t off = 0;
    for (int f = 0; f < ncols; f++) {
        dst[f] = base + off;
        if (len[f] > 0 && !src[f]) return fail(c, HBT_ERR_INVALID, "null particle array");
        off += (size_t)((len[f] + 31) / 32 * 32);
    }
    // columns laid out in host memory as they will be on the device (each a
    // multiple of 32 doubles, back to back) go over in one copy per run
    for (int f = 0; f < ncols;) {
        if (len[f] <= 0) {
            f++;
            continue;
        }
        int g = f;
        while (g + 1 < ncols && len[g + 1] > 0 &&
               src[g] + (len[g] + 31) / 32 * 32 == src[g + 1])
            g++;
        const size_t n = (size_t)(dst[g] - dst[f]) + (size_t)len[g];
        CU(cudaMemcpyAsync(const_cast<double *>(dst[f]), src[f], n * sizeof(double),
                           cudaMemcpyHostToDevice, cs));
        f = g + 1;
    }
    // the caller's arrays may be reused once the copies are done; the
    // binning stream starts after them
    CU(cudaEventRecord(c->staged, cs));
    CU(cudaEventSynchronize(c->staged));
    if (cs != c->stream) CU(cudaStreamWaitEvent(c->stream, c->staged, 0));
    if (!c->pool) {
        c->in_cur = buf;
        c->in_next ^= 1;
    }
    return HBT_OK;
}

// After the binning of the staged lists is queued on the context's stream:
// the staging buffer is free once that work is done.
hbt_status staged_done(hbt_ctx *c, hbt_status s) {
    if (c->in_cur >= 0) {
        const cudaError_t e = cudaEventRecord(c->in_free[c->in_cur], c->stream);
        c->in_used[c->in_cur] = e == cudaSuccess;
        c->in_cur = -1;
        if (e != cudaSuccess && s == HBT_OK)
            return fail(c, HBT_ERR_CUDA, std::string("cudaEventRecord: ") + cudaGetErrorString(e));
    }
    return s;
}

}  // namespace

namespace hbt {

void grid_from_params(const hbt_params &p, Grid &g) {
    // constants with the reference's expressions (src/HBT_correlation.cpp:25-61)
    g = Grid{};
    g.qnpts = p.qnpts;
    g.n_KT = p.n_KT;
    g.n_Kphi = p.n_Kphi;
    g.azimuthal = p.azimuthal_flag == 1;
    g.qinv = p.invariant_radius_flag == 1;
    g.boost = p.long_comoving_boost == 1;
    g.n_slots = g.azimuthal ? p.n_KT * p.n_Kphi : p.n_KT;
    g.q3 = (long long)p.qnpts * p.qnpts * p.qnpts;
    g.delta_q = (p.q_max - p.q_min) / (p.qnpts - 1);
    g.q_lo = p.q_min - g.delta_q / 2. + 1e-8;
    g.q_hi = p.q_max + g.delta_q / 2. - 1e-8;
    g.q_base = p.q_min - g.delta_q / 2.;
    g.KT_min = p.KT_min;
    g.dKT = (p.KT_max - p.KT_min) / (p.n_KT - 1);
    g.KT_min_sq = p.KT_min * p.KT_min;
    g.KT_max_sq = p.KT_max * p.KT_max;
    g.dKphi = 2 * M_PI / p.n_Kphi;
    g.two_pi = 2. * M_PI;
    g.psi_ref = 0.0;
    g.kphi_tol = p.kphi_defer_tol > 0 ? p.kphi_defer_tol : 1e-13;
    g.hbarC_inv = 1. / hbt::kHbarC;
    g.cph = make_cos_scale(g.hbarC_inv);
}

void screen_from_grid(const Grid &g, Screen &s) {
    auto f = [](double v) { return static_cast<float>(v); };
    auto slack = [](double v, float v32) { return std::fabs(v - static_cast<double>(v32)); };
    const double lo4 = 4.0 * g.KT_min_sq, hi4 = 4.0 * g.KT_max_sq;
    s.kt_lo4 = f(lo4);
    s.kt_hi4 = f(hi4);
    s.kt_slack = f(std::max(slack(lo4, s.kt_lo4), slack(hi4, s.kt_hi4)) + 1e-7 * hi4);
    s.lo = f(g.q_lo);
    s.hi = f(g.q_hi);
    s.win_slack = f(std::max(slack(g.q_lo, s.lo), slack(g.q_hi, s.hi)) + 1e-12);
    s.base = f(g.q_base);
    s.inv_dq = f(1.0 / g.delta_q);
    s.t_slack = f(slack(g.q_base, s.base) / g.delta_q + 4.0 * 5.96e-8 * g.qnpts + 1e-9);
    s.KT_min = f(g.KT_min);
    s.inv_dKT = f(1.0 / g.dKT);
    s.kt_t_slack = f(slack(g.KT_min, s.KT_min) / g.dKT + 4.0 * 5.96e-8 * g.n_KT + 1e-9);
    s.psi = f(g.psi_ref);
    s.psi_slack = f(slack(g.psi_ref, s.psi));
    s.two_pi = f(g.two_pi);
    s.inv_dKphi = f(1.0 / g.dKphi);
    s.kphi_tol = std::nextafter(f(g.kphi_tol), INFINITY);
    s.qnpts = g.qnpts;
    s.n_KT = g.n_KT;
    s.n_Kphi = g.n_Kphi;
    fill_prefilter(s);
}

bool params_valid(const hbt_params &p) {
    if (p.qnpts < 2 || p.n_KT < 2 || p.n_Kphi < 1 || p.qnpts > 1024) return false;
    if (p.precision != HBT_PRECISION_FP64 && p.precision != HBT_PRECISION_FP32W &&
        p.precision != HBT_PRECISION_DF64)
        return false;
    if (p.kernel != HBT_KERNEL_SCREENED && p.kernel != HBT_KERNEL_REFERENCE_CHAIN &&
        p.kernel != HBT_KERNEL_SCREENED_GRID)
        return false;
    return true;
}

}  // namespace hbt

extern "C" {

hbt_status hbt_create(const hbt_params *p, int device, hbt_ctx **out) {
    return hbt::ctx_create(p, device, nullptr, out);
}

}  // extern "C"

namespace hbt {

hbt_status ctx_create(const hbt_params *p, int device, cudaMemPool_t pool, hbt_ctx **out) {
    hbt_ctx *c = nullptr;
    if (!p || !out) return HBT_ERR_INVALID;
    *out = nullptr;
    if (!hbt::params_valid(*p)) return HBT_ERR_INVALID;
    c = new hbt_ctx();
    c->prm = *p;
    c->device = device;
    c->pool = pool;
    // a failure below leaves c to hbt_destroy
    std::unique_ptr<hbt_ctx, void (*)(hbt_ctx *)> guard(c, hbt_destroy);
    if (cudaSetDevice(device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&c->own, cudaStreamNonBlocking) != cudaSuccess)
        return HBT_ERR_CUDA;
    c->stream = c->own;
    CU(cudaEventCreateWithFlags(&c->staged, cudaEventDisableTiming));

    hbt::Grid &g = c->d.g;
    hbt::grid_from_params(*p, g);
    fill_screen(c);
    c->cap = static_cast<u64>(p->needed_number_of_pairs);
    c->cap_qinv = 50 * c->cap;
    c->n_stream = g.n_slots + g.n_KT;
    c->d.precision = p->precision;
    // merge the FP32 partials every kMergeChunk same-event CTAs
    c->d.merge_chunk_blocks = kMergeChunk;
    c->d.block_offset = 0;
    {
        int sms = 0;
        CU(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
        c->sms = sms;
        c->max_blocks_per_sm = hbt::persistent_blocks_per_sm();
        c->persistent_grid = sms * c->max_blocks_per_sm;
    }

    const size_t nb = (size_t)g.n_slots * g.q3, nq = (size_t)g.n_KT * g.qnpts;
    hbt_status s = HBT_OK;
    if ((s = dalloc(c, c->sums, nb * sizeof(hbt::Sums))) != HBT_OK ||
        (s = dalloc(c, c->cnt, nb * sizeof(u64))) != HBT_OK ||
        (s = dalloc(c, c->den, nb * sizeof(u64))) != HBT_OK ||
        (s = dalloc(c, c->qi_sums, nq * sizeof(hbt::QiSums))) != HBT_OK ||
        (s = dalloc(c, c->qi_cnt, nq * sizeof(u64))) != HBT_OK ||
        (s = dalloc(c, c->qi_den, nq * sizeof(u64))) != HBT_OK ||
        (s = dalloc(c, c->stats, hbt::STAT_N * sizeof(u64))) != HBT_OK ||
        (s = dalloc(c, c->defer, kDeferCap * sizeof(hbt::Deferral))) != HBT_OK ||
        (s = dalloc(c, c->n_defer, sizeof(unsigned))) != HBT_OK ||
        (p->precision == HBT_PRECISION_FP32W &&
         ((s = dalloc(c, c->part, 2 * nb * sizeof(float4))) != HBT_OK ||
          (s = dalloc(c, c->comp, nb * sizeof(hbt::Sums))) != HBT_OK)))
        return s;
    refresh_device(c);
    if ((s = hbt_reset(c)) != HBT_OK) return s;
    *out = guard.release();
    return HBT_OK;
}

}  // namespace hbt

extern "C" {

void hbt_destroy(hbt_ctx *c) {
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    DevBuf *bufs[] = {&c->sums,   &c->cnt,     &c->den,       &c->qi_sums,  &c->qi_cnt,
                      &c->qi_den, &c->stats,   &c->defer,     &c->n_defer,  &c->rowcnt,
                      &c->row_cut, &c->quota,  &c->remaining, &c->resolved, &c->counters,
                      &c->apply_iphi, &c->straddle_jobs, &c->slot_full, &c->in[0], &c->in[1],
                      &c->part, &c->comp, &c->exp};
    if (c->copy) cudaStreamSynchronize(c->copy);
    for (DevBuf *b : bufs) dfree(c, *b);
    dfree(c, c->snap);
    if (c->snap_ev) cudaEventDestroy(c->snap_ev);
    if (c->copy_ev) cudaEventDestroy(c->copy_ev);
    if (c->copy) cudaStreamDestroy(c->copy);
    if (c->flag_host) cudaFreeHost(c->flag_host);
    if (c->count_host) cudaFreeHost(c->count_host);
    if (c->defer_host) cudaFreeHost(c->defer_host);
    if (c->apply_host) cudaFreeHost(c->apply_host);
    dfree(c, c->apply_dev);
    if (c->staged) cudaEventDestroy(c->staged);
    if (c->copy_in) cudaStreamSynchronize(c->copy_in);
    for (cudaEvent_t e : c->in_free)
        if (e) cudaEventDestroy(e);
    if (c->copy_in) cudaStreamDestroy(c->copy_in);
    if (c->own) cudaStreamDestroy(c->own);
    delete c;
}

const char *hbt_last_error(const hbt_ctx *c) { return c ? c->err.c_str() : "null context"; }

hbt_status hbt_set_stream(hbt_ctx *c, void *s) {
    if (!c) return HBT_ERR_INVALID;
    c->stream = s ? static_cast<cudaStream_t>(s) : c->own;
    return HBT_OK;
}

hbt_status hbt_set_psi_ref(hbt_ctx *c, double psi) {
    if (!c) return HBT_ERR_INVALID;
    c->d.g.psi_ref = psi;
    fill_screen(c);
    return HBT_OK;
}

hbt_status hbt_reset(hbt_ctx *c) {
    if (!c) return HBT_ERR_INVALID;
    CU(cudaSetDevice(c->device));
    CU(cudaMemsetAsync(c->sums.p, 0, c->sums.bytes, c->stream));
    CU(cudaMemsetAsync(c->cnt.p, 0, c->cnt.bytes, c->stream));
    CU(cudaMemsetAsync(c->den.p, 0, c->den.bytes, c->stream));
    CU(cudaMemsetAsync(c->qi_sums.p, 0, c->qi_sums.bytes, c->stream));
    CU(cudaMemsetAsync(c->qi_cnt.p, 0, c->qi_cnt.bytes, c->stream));
    CU(cudaMemsetAsync(c->qi_den.p, 0, c->qi_den.bytes, c->stream));
    CU(cudaMemsetAsync(c->stats.p, 0, c->stats.bytes, c->stream));
    if (c->part.p) CU(cudaMemsetAsync(c->part.p, 0, c->part.bytes, c->stream));
    if (c->comp.p) CU(cudaMemsetAsync(c->comp.p, 0, c->comp.bytes, c->stream));
    CU(cudaMemsetAsync(c->n_defer.p, 0, sizeof(unsigned), c->stream));
    CU(cudaStreamSynchronize(c->stream));
    for (int f = 0; f < 4; f++) c->ub[f] = 0;
    memset(&c->st, 0, sizeof(c->st));
    c->deferred_async = 0;
    return HBT_OK;
}

hbt_status hbt_bin_same_dev(hbt_ctx *c, int64_t n, const hbt_soa8 *l) {
    if (!c || !l || n < 0) return HBT_ERR_INVALID;
    CU(cudaSetDevice(c->device));
    const double *c8[8] = {l->px, l->py, l->pz, l->E, l->x, l->y, l->z, l->t};
    return bin_same_device(c, n, c8);
}

hbt_status hbt_bin_mixed_dev(hbt_ctx *c, int64_t n1, const hbt_soa4 *a, int64_t n2,
                             const hbt_soa4 *b) {
    if (!c || !a || !b || n1 < 0 || n2 < 0) return HBT_ERR_INVALID;
    CU(cudaSetDevice(c->device));
    const double *l1[4] = {a->px, a->py, a->pz, a->E};
    const double *l2[4] = {b->px, b->py, b->pz, b->E};
    return bin_mixed_device(c, n1, l1, n2, l2);
}

hbt_status hbt_bin_same(hbt_ctx *c, int64_t n, const hbt_soa8 *l) {
    if (!c || !l || n < 0) return HBT_ERR_INVALID;
    if (n < 2) {
        if (n >= 0) c->st.pairs_same += 0;
        return HBT_OK;
    }
    CU(cudaSetDevice(c->device));
    const double *src[8] = {l->px, l->py, l->pz, l->E, l->x, l->y, l->z, l->t};
    const long long len[8] = {n, n, n, n, n, n, n, n};
    const double *dv[8];
    TRY(stage(c, src, len, 8, dv));
    return staged_done(c, bin_same_device(c, n, dv));
}

hbt_status hbt_bin_mixed(hbt_ctx *c, int64_t n1, const hbt_soa4 *a, int64_t n2,
                         const hbt_soa4 *b) {
    if (!c || !a || !b || n1 < 0 || n2 < 0) return HBT_ERR_INVALID;
    if (n1 == 0 || n2 == 0) return HBT_OK;
    CU(cudaSetDevice(c->device));
    const double *src[8] = {a->px, a->py, a->pz, a->E, b->px, b->py, b->pz, b->E};
    const long long len[8] = {n1, n1, n1, n1, n2, n2, n2, n2};
    const double *dv[8];
    TRY(stage(c, src, len, 8, dv));
    return staged_done(c, bin_mixed_device(c, n1, dv, n2, dv + 4));
}

hbt_status hbt_bin_batch_dev(hbt_ctx *c, int32_t n_jobs, const hbt_job *jobs) {
    if (!c || n_jobs < 0 || (n_jobs > 0 && !jobs)) return HBT_ERR_INVALID;
    CU(cudaSetDevice(c->device));
    u64 P_same = 0, P_mixed = 0;
    for (int k = 0; k < n_jobs; k++) {
        const hbt_job &j = jobs[k];
        if (j.kind != 0 && j.kind != 1) return fail(c, HBT_ERR_INVALID, "job kind must be 0 or 1");
        if (j.na < 0 || j.nb < 0) return fail(c, HBT_ERR_INVALID, "negative list size");
        if (j.kind == 0 && j.na >= 2) P_same += (u64)j.na * (u64)(j.na - 1) / 2;
        if (j.kind == 1) P_mixed += (u64)j.na * (u64)j.nb;
    }
    bool sequential = !batched_ok(c) || caps_may_bind(c, 0, P_same) || caps_may_bind(c, 1, P_mixed);
    if (sequential && batched_ok(c)) {
        TRY(drain_deferrals(c));
        std::vector<u64> ctr;
        TRY(read_counters(c, ctr));
        sequential = caps_may_bind(c, 0, P_same) || caps_may_bind(c, 1, P_mixed);
    }
    if (sequential && batched_ok(c) && !c->d.g.qinv) {
        // the numerator and denominator counters are separate families, so
        // the same-event jobs (each admitted on its own, in order) and the
        // mixed-event jobs (admitted together in their joint order) keep the
        // reference's order for the caps
        for (int k = 0; k < n_jobs; k++)
            if (jobs[k].kind == 0) TRY(hbt_bin_same_dev(c, jobs[k].na, &jobs[k].a));
        if (P_mixed > 0) {
            std::vector<FastJob> mj;
            for (const FastJob &f : fast_jobs_of(n_jobs, jobs))
                if (f.kind == 1) mj.push_back(f);
            c->st.pairs_mixed += P_mixed;
            if (caps_may_bind(c, 1, P_mixed)) {
                TRY(ordered_launch_mixed_jobs(c, mj));
                std::vector<u64> ctr;
                TRY(read_counters(c, ctr));
            } else {
                TRY(run_fast_jobs(c, mj));
                c->ub[1] += P_mixed;
            }
        }
        return HBT_OK;
    }
    if (sequential) {
        // one job at a time keeps the reference's order for the caps
        for (int k = 0; k < n_jobs; k++) {
            const hbt_job &j = jobs[k];
            if (j.kind == 0) {
                TRY(hbt_bin_same_dev(c, j.na, &j.a));
            } else {
                const hbt_soa4 a = {j.a.px, j.a.py, j.a.pz, j.a.E};
                const hbt_soa4 b = {j.b.px, j.b.py, j.b.pz, j.b.E};
                TRY(hbt_bin_mixed_dev(c, j.na, &a, j.nb, &b));
            }
        }
        return HBT_OK;
    }
    std::vector<FastJob> fj = fast_jobs_of(n_jobs, jobs);
    c->st.pairs_same += P_same;
    c->st.pairs_mixed += P_mixed;
    TRY(run_fast_jobs(c, fj));
    c->ub[0] += P_same;
    c->ub[1] += P_mixed;
    return HBT_OK;
}

hbt_status hbt_bin_batch(hbt_ctx *c, int32_t n_jobs, const hbt_job *jobs) {
    if (!c || n_jobs < 0 || (n_jobs > 0 && !jobs)) return HBT_ERR_INVALID;
    CU(cudaSetDevice(c->device));
    // stage every host column of the batch into one device buffer
    std::vector<const double *> src;
    std::vector<long long> len;
    for (int k = 0; k < n_jobs; k++) {
        const hbt_job &j = jobs[k];
        const double *a[8] = {j.a.px, j.a.py, j.a.pz, j.a.E, j.a.x, j.a.y, j.a.z, j.a.t};
        const int na = j.kind == 0 ? 8 : 4;
        for (int q = 0; q < na; q++) {
            src.push_back(a[q]);
            len.push_back(j.na);
        }
        if (j.kind == 1) {
            const double *b[4] = {j.b.px, j.b.py, j.b.pz, j.b.E};
            for (int q = 0; q < 4; q++) {
                src.push_back(b[q]);
                len.push_back(j.nb);
            }
        }
    }
    std::vector<const double *> dv(src.size());
    TRY(stage(c, src.data(), len.data(), (int)src.size(), dv.data()));
    std::vector<hbt_job> dj(jobs, jobs + n_jobs);
    size_t at = 0;
    for (int k = 0; k < n_jobs; k++) {
        hbt_job &j = dj[k];
        const double **a[8] = {&j.a.px, &j.a.py, &j.a.pz, &j.a.E, &j.a.x, &j.a.y, &j.a.z, &j.a.t};
        const int na = j.kind == 0 ? 8 : 4;
        for (int q = 0; q < na; q++) *a[q] = dv[at++];
        if (j.kind == 1) {
            const double **b[4] = {&j.b.px, &j.b.py, &j.b.pz, &j.b.E};
            for (int q = 0; q < 4; q++) *b[q] = dv[at++];
        }
    }
    return staged_done(c, hbt_bin_batch_dev(c, n_jobs, dj.data()));
}

hbt_status hbt_set_tuning(hbt_ctx *c, const hbt_tuning *t) {
    if (!c || !t) return HBT_ERR_INVALID;
    if (!tuning_valid(*t)) return fail(c, HBT_ERR_INVALID, "invalid tuning");
    c->tune = tuning_defaults(*t);
    return HBT_OK;
}

hbt_status hbt_get_tuning(hbt_ctx *c, hbt_tuning *t) {
    if (!c || !t) return HBT_ERR_INVALID;
    *t = c->tune;
    return HBT_OK;
}

hbt_status hbt_autotune_batch(hbt_ctx *c, int32_t n_jobs, const hbt_job *jobs, double max_pairs,
                              hbt_tuning *best, double *best_ms) {
    if (!c || n_jobs < 0 || (n_jobs > 0 && !jobs)) return HBT_ERR_INVALID;
    if (!batched_ok(c)) return fail(c, HBT_ERR_STATE, "the batched path is not in use");
    CU(cudaSetDevice(c->device));
    for (int k = 0; k < n_jobs; k++)
        if ((jobs[k].kind != 0 && jobs[k].kind != 1) || jobs[k].na < 0 || jobs[k].nb < 0)
            return fail(c, HBT_ERR_INVALID, "invalid job");
    // a sample of the batch: jobs in order up to max_pairs candidate pairs
    if (!(max_pairs > 0)) max_pairs = 2e9;
    std::vector<FastJob> all = fast_jobs_of(n_jobs, jobs), sample;
    double pairs = 0.0;
    for (const FastJob &f : all) {
        if (!sample.empty() && pairs >= max_pairs) break;
        sample.push_back(f);
        pairs += f.kind == 0 ? 0.5 * (double)f.na * (double)(f.na - 1) : (double)f.na * f.nb;
    }
    // scratch histograms of the same analysis
    hbt_ctx *t = nullptr;
    const hbt_status s = hbt::ctx_create(&c->prm, c->device, nullptr, &t);
    if (s != HBT_OK) return fail(c, s, "autotune: scratch context creation failed");
    std::unique_ptr<hbt_ctx, void (*)(hbt_ctx *)> guard(t, hbt_destroy);
    t->d.g.psi_ref = c->d.g.psi_ref;
    fill_screen(t);
    cudaEvent_t e0, e1;
    CU(cudaEventCreate(&e0));
    CU(cudaEventCreate(&e1));
    auto time_one = [&](const hbt_tuning &cand, double &ms) -> hbt_status {
        t->tune = cand;
        t->tune.use_graph = 0;
        double bestv = 1e300;
        for (int rep = 0; rep < 3; rep++) {  // the first run warms up
            CU(cudaEventRecord(e0, t->stream));
            TRY(run_fast_jobs(t, sample));
            CU(cudaEventRecord(e1, t->stream));
            CU(cudaEventSynchronize(e1));
            float m = 0.f;
            CU(cudaEventElapsedTime(&m, e0, e1));
            if (rep > 0) bestv = std::min(bestv, (double)m);
        }
        ms = bestv;
        return HBT_OK;
    };
    hbt_tuning cur = c->tune;
    double cur_ms = 0.0;
    hbt_status rs = time_one(cur, cur_ms);
    // coordinate search: sort cells, then CTAs per SM, then the item order,
    // then the merge chunk
    const double cells[][2] = {{0.01, 0.025}, {0.02, 0.05}, {0.04, 0.1}, {0.02, 0.1}, {0.04, 0.05},
                               {0.01, 0.05}};
    for (const auto &cl : cells) {
        if (rs != HBT_OK) break;
        hbt_tuning cand = cur;
        cand.cell_pt = cl[0];
        cand.cell_y = cl[1];
        if (cand.cell_pt == cur.cell_pt && cand.cell_y == cur.cell_y) continue;
        double ms = 0.0;
        rs = time_one(cand, ms);
        if (rs == HBT_OK && ms < cur_ms) {
            cur = cand;
            cur_ms = ms;
        }
    }
    for (int bps = 3; bps <= 6 && rs == HBT_OK; bps++) {
        hbt_tuning cand = cur;
        cand.blocks_per_sm = bps;
        if (cand.blocks_per_sm == cur.blocks_per_sm) continue;
        double ms = 0.0;
        rs = time_one(cand, ms);
        if (rs == HBT_OK && ms < cur_ms) {
            cur = cand;
            cur_ms = ms;
        }
    }
    if (c->d.precision == HBT_PRECISION_FP32W) {
        cur.order_items = 0;  // the FP32-weight form always runs in the cull's order
    } else {
        hbt_tuning cand = cur;
        cand.order_items = cur.order_items ? 0 : 1;
        double ms = 0.0;
        if (rs == HBT_OK) rs = time_one(cand, ms);
        if (rs == HBT_OK && ms < cur_ms) {
            cur = cand;
            cur_ms = ms;
        }
    }
    if (c->d.precision == HBT_PRECISION_FP32W)
        for (int chunk : {kMergeChunk / 2, kMergeChunk}) {
            if (rs != HBT_OK || chunk == cur.merge_chunk) continue;
            hbt_tuning cand = cur;
            cand.merge_chunk = chunk;
            double ms = 0.0;
            rs = time_one(cand, ms);
            if (rs == HBT_OK && ms < cur_ms) {
                cur = cand;
                cur_ms = ms;
            }
        }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rs != HBT_OK) return fail(c, rs, std::string("autotune: ") + hbt_last_error(t));
    cur.use_graph = c->tune.use_graph;
    c->tune = cur;
    if (best) *best = cur;
    if (best_ms) *best_ms = cur_ms;
    return HBT_OK;
}

hbt_status hbt_sync(hbt_ctx *c, uint64_t timeout_us) {
    if (!c) return HBT_ERR_INVALID;
    CU(cudaSetDevice(c->device));
    if (timeout_us == 0) {
        CU(cudaStreamSynchronize(c->stream));
    } else {
        const auto t0 = std::chrono::steady_clock::now();
        for (;;) {
            const cudaError_t e = cudaStreamQuery(c->stream);
            if (e == cudaSuccess) break;
            if (e != cudaErrorNotReady)
                return fail(c, HBT_ERR_CUDA, std::string("cudaStreamQuery: ") + cudaGetErrorString(e));
            const auto us = std::chrono::duration_cast<std::chrono::microseconds>(
                                std::chrono::steady_clock::now() - t0)
                                .count();
            if ((uint64_t)us >= timeout_us)
                return fail(c, HBT_ERR_TIMEOUT, "hbt_sync: work still running");
            std::this_thread::sleep_for(std::chrono::microseconds(50));
        }
    }
    u64 stats[hbt::STAT_N];
    CU(cudaMemcpy(stats, c->stats.p, sizeof(stats), cudaMemcpyDeviceToHost));
    if (stats[hbt::STAT_ERROR] != 0)
        return fail(c, HBT_ERR_DEVICE, "a kernel raised its error flag");
    return HBT_OK;
}

int64_t hbt_n_bins(const hbt_ctx *c) { return c ? (int64_t)c->d.g.n_slots * c->d.g.q3 : 0; }

hbt_status hbt_read_hist(hbt_ctx *c, double *num_count, double *q_out_sum, double *q_side_sum,
                         double *q_long_sum, double *num, double *den) {
    if (!c) return HBT_ERR_INVALID;
    CU(cudaSetDevice(c->device));
    TRY(drain_deferrals(c));
    TRY(hbt_sync(c, 0));
    const size_t nb = (size_t)hbt_n_bins(c);
    // each array is laid out as FP64 on the device (k_export), then copied
    // straight into the caller's array; two device buffers in turn keep the
    // next export running while a copy is in flight
    double *dst[6] = {q_out_sum, q_side_sum, q_long_sum, num, num_count, den};
    TRY(dalloc(c, c->exp, 2 * nb * sizeof(double)));
    int used = 0;
    for (int f = 0; f < 6; f++) {
        if (!dst[f]) continue;
        double *buf = ptr<double>(c->exp) + (size_t)(used++ & 1) * nb;
        CU(hbt::launch_export(c->d, f, buf, (long long)nb, c->stream));
        CU(cudaMemcpyAsync(dst[f], buf, nb * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    }
    CU(cudaStreamSynchronize(c->stream));
    c->st.launches += used;
    return HBT_OK;
}

hbt_status hbt_read_hist_wait(hbt_ctx *c) {
    if (!c) return HBT_ERR_INVALID;
    if (!c->read_pending) return HBT_OK;
    CU(cudaSetDevice(c->device));
    CU(cudaEventSynchronize(c->copy_ev));
    c->read_pending = false;
    if (*c->flag_host != 0) return fail(c, HBT_ERR_DEVICE, "a kernel raised its error flag");
    return HBT_OK;
}

hbt_status hbt_read_hist_async(hbt_ctx *c, double *num_count, double *q_out_sum,
                               double *q_side_sum, double *q_long_sum, double *num, double *den) {
    if (!c) return HBT_ERR_INVALID;
    CU(cudaSetDevice(c->device));
    TRY(hbt_read_hist_wait(c));  // one read in flight: the snapshot is reused
    TRY(drain_deferrals_async(c));
    if (!c->copy) {
        CU(cudaStreamCreateWithFlags(&c->copy, cudaStreamNonBlocking));
        CU(cudaEventCreateWithFlags(&c->snap_ev, cudaEventDisableTiming));
        CU(cudaEventCreateWithFlags(&c->copy_ev, cudaEventDisableTiming));
        CU(cudaMallocHost(&c->flag_host, sizeof(u64)));
    }
    const size_t nb = (size_t)hbt_n_bins(c);
    double *dst[6] = {q_out_sum, q_side_sum, q_long_sum, num, num_count, den};
    TRY(dalloc(c, c->snap, 6 * nb * sizeof(double) + sizeof(u64)));
    double *snap = ptr<double>(c->snap);
    u64 *flag = reinterpret_cast<u64 *>(snap + 6 * nb);
    // the snapshot is stream-ordered after everything binned so far
    int used = 0;
    for (int f = 0; f < 6; f++) {
        if (!dst[f]) continue;
        CU(hbt::launch_export(c->d, f, snap + (size_t)f * nb, (long long)nb, c->stream));
        used++;
    }
    CU(cudaMemcpyAsync(flag, ptr<u64>(c->stats) + hbt::STAT_ERROR, sizeof(u64),
                       cudaMemcpyDeviceToDevice, c->stream));
    CU(cudaEventRecord(c->snap_ev, c->stream));
    CU(cudaStreamWaitEvent(c->copy, c->snap_ev, 0));
    for (int f = 0; f < 6; f++)
        if (dst[f])
            CU(cudaMemcpyAsync(dst[f], snap + (size_t)f * nb, nb * sizeof(double),
                               cudaMemcpyDeviceToHost, c->copy));
    CU(cudaMemcpyAsync(c->flag_host, flag, sizeof(u64), cudaMemcpyDeviceToHost, c->copy));
    CU(cudaEventRecord(c->copy_ev, c->copy));
    c->read_pending = true;
    c->st.launches += used;
    return HBT_OK;
}

hbt_status hbt_read_qinv(hbt_ctx *c, double *qinv_sum, double *num, double *num_count,
                         double *den) {
    if (!c) return HBT_ERR_INVALID;
    CU(cudaSetDevice(c->device));
    TRY(hbt_sync(c, 0));
    const size_t nq = (size_t)c->d.g.n_KT * c->d.g.qnpts;
    std::vector<hbt::QiSums> s(nq);
    CU(cudaMemcpy(s.data(), c->qi_sums.p, nq * sizeof(hbt::QiSums), cudaMemcpyDeviceToHost));
    std::vector<u64> a(nq), b(nq);
    CU(cudaMemcpy(a.data(), c->qi_cnt.p, nq * sizeof(u64), cudaMemcpyDeviceToHost));
    CU(cudaMemcpy(b.data(), c->qi_den.p, nq * sizeof(u64), cudaMemcpyDeviceToHost));
    for (size_t k = 0; k < nq; k++) {
        if (qinv_sum) qinv_sum[k] = s[k].q;
        if (num) num[k] = s[k].w;
        if (num_count) num_count[k] = (double)a[k];
        if (den) den[k] = (double)b[k];
    }
    return HBT_OK;
}

hbt_status hbt_read_counters(hbt_ctx *c, uint64_t *num, uint64_t *den, uint64_t *num_qinv,
                             uint64_t *den_qinv) {
    if (!c) return HBT_ERR_INVALID;
    CU(cudaSetDevice(c->device));
    TRY(drain_deferrals(c));
    std::vector<u64> ctr;
    TRY(read_counters(c, ctr));
    const int ns = c->d.g.n_slots, nk = c->d.g.n_KT;
    for (int s = 0; s < ns; s++) {
        if (num) num[s] = ctr[s];
        if (den) den[s] = ctr[ns + s];
    }
    for (int k = 0; k < nk; k++) {
        if (num_qinv) num_qinv[k] = ctr[2 * ns + k];
        if (den_qinv) den_qinv[k] = ctr[2 * ns + nk + k];
    }
    return HBT_OK;
}

hbt_status hbt_inject_alloc_failure(hbt_ctx *c, int32_t n_ok) {
    if (!c || n_ok < -1) return HBT_ERR_INVALID;
    c->fail_after = n_ok;
    return HBT_OK;
}

hbt_status hbt_get_stats(hbt_ctx *c, hbt_stats *out) {
    if (!c || !out) return HBT_ERR_INVALID;
    CU(cudaSetDevice(c->device));
    TRY(hbt_sync(c, 0));
    u64 stats[hbt::STAT_N];
    CU(cudaMemcpy(stats, c->stats.p, sizeof(stats), cudaMemcpyDeviceToHost));
    *out = c->st;
    out->deferred_kphi += c->deferred_async;
    out->anomalies = stats[hbt::STAT_ANOMALY];
    long long cs = 0, cm = 0, ks = 0, km = 0;
    if (c->runner.tile_counts(cs, cm, ks, km)) {
        out->tiles_same = cs;
        out->tiles_mixed = cm;
        out->tiles_same_kept = ks;
        out->tiles_mixed_kept = km;
    }
    float sm = 0.f, mm = 0.f;
    if (c->tune.time_kernels && c->runner.kernel_times(sm, mm)) {
        out->same_kernel_ms = sm;
        out->mixed_kernel_ms = mm;
    }
    return HBT_OK;
}

}  // extern "C"

// Library-internal accessors (hbt_internal.h) for the serving loop.
namespace hbt {

const Device &ctx_device(const hbt_ctx *c) { return c->d; }

int ctx_persistent_grid(const hbt_ctx *c) { return c->persistent_grid; }

cudaStream_t ctx_stream(const hbt_ctx *c) { return c->own; }

void ctx_add_pairs(hbt_ctx *c, u64 same, u64 mixed) {
    c->st.pairs_same += same;
    c->st.pairs_mixed += mixed;
    c->ub[0] += same;
    c->ub[1] += mixed;
}

cudaError_t ctx_merge(hbt_ctx *c, cudaStream_t st) {
    if (c->d.precision != HBT_PRECISION_FP32W) return cudaSuccess;
    return launch_merge(c->d, st);
}

size_t ctx_device_bytes(const hbt_params &p) {
    const size_t slots = (size_t)p.n_KT * (p.azimuthal_flag == 1 ? p.n_Kphi : 1);
    const size_t nb = slots * p.qnpts * p.qnpts * p.qnpts, nq = (size_t)p.n_KT * p.qnpts;
    // bins, counts, the readback buffers, the q_inv bins, the deferrals
    size_t bytes = nb * (sizeof(Sums) + 2 * sizeof(u64) + 2 * sizeof(double)) +
                   nq * (sizeof(QiSums) + 2 * sizeof(u64)) + kDeferCap * sizeof(Deferral) + 4096;
    if (p.precision == HBT_PRECISION_FP32W) bytes += nb * (2 * sizeof(float4) + sizeof(Sums));
    return bytes;
}

bool ctx_batchable(const hbt_ctx *c) { return batched_ok(c) && !c->d.g.qinv; }

bool ctx_caps_may_bind(const hbt_ctx *c, int mixed, u64 P) { return caps_may_bind(c, mixed, P); }

}  // namespace hbt
