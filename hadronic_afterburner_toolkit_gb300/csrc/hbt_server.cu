// Serving loop (include/hbt_server.h): continuous batching of HBT requests
// of many analyses into the batched persistent pair-binning launches.
//
// Threads: callers submit and wait; one worker admits requests, uploads
// their particles, builds and issues rounds and retires them; one
// completion thread copies the results of finished requests out and frees
// their memory; one solo thread runs the requests that must go through the
// per-analysis path.  Streams:
// uploads and rotations on `upload_`, rounds on `rounds_`, each request's
// histograms live on its context's own stream.  All device memory of the
// requests is stream-ordered from one pool, so admitting and finishing
// requests never synchronises the device.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <climits>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <random>
#include <string>
#include <thread>
#include <vector>

#include "../../include/hbt_server.h"
#include "hbt_internal.h"
#include "hbt_runner.h"

namespace {

using hbt::u64;
using Clock = std::chrono::steady_clock;

double ms_between(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}

// One rotated partner list: rows [src, src + n) of the request's particle
// columns, rotated by (c, s), written to rows [dst, dst + n) of its partner
// columns.
struct Segment {
    long long dst, src, n;
    double c, s;
};

// Rotation of a mixed-event partner as the reference rotates it
// (src/HBT_correlation.cpp:495-523): px' = px cos - py sin,
// py' = px sin + py cos, pz and E unchanged.  This unit is compiled with
// --fmad=false, so each product rounds as the reference's CPU build does.
__global__ void k_rotate(const Segment *seg, const double *cols, long long n_rows, double *rot,
                         long long m_rows) {
    const Segment sg = seg[blockIdx.x];
    const double *px = cols, *py = cols + n_rows, *pz = cols + 2 * n_rows, *E = cols + 3 * n_rows;
    double *rx = rot, *ry = rot + m_rows, *rz = rot + 2 * m_rows, *rE = rot + 3 * m_rows;
    for (long long k = threadIdx.x; k < sg.n; k += blockDim.x) {
        const double x = px[sg.src + k], y = py[sg.src + k];
        rx[sg.dst + k] = x * sg.c - y * sg.s;
        ry[sg.dst + k] = x * sg.s + y * sg.c;
        rz[sg.dst + k] = pz[sg.src + k];
        rE[sg.dst + k] = E[sg.src + k];
    }
}

struct Request {
    uint64_t id = 0;
    hbt_params prm{};
    int n_events = 0, oversample = 0, partners = 0;
    std::vector<long long> off;  // event offsets after the rapidity cut
    std::vector<double> cols;    // [8][n] cut particles
    long long n = 0;             // cut particles
    long long m = 0;             // rows of all rotated partner lists
    std::vector<int> partner;    // [n_events][partners]
    std::vector<double> cphi, sphi;
    std::vector<long long> roff; // [n_events + 1] first partner row of each event
    double psi = 0.0;
    u64 pairs_same = 0, pairs_mixed = 0, anomalies = 0;
    size_t bytes = 0;

    // life cycle
    int state = HBT_JOB_QUEUED;
    int status = HBT_OK;
    bool solo = false;
    int rounds = 0;
    Clock::time_point t_submit, t_admit, t_done;

    // device state (worker / solo thread only)
    hbt_ctx *ctx = nullptr;
    double *dcols = nullptr, *drot = nullptr;
    cudaEvent_t ready = nullptr;
    bool waited = false;               // rounds_ waits on `ready`
    std::vector<hbt::FastJob> work;    // batched pair work
    std::vector<long long> work_tiles; // candidate tile pairs of each
    size_t next = 0;                   // first work item not issued

    // results
    long long nb = 0, nq = 0, ns = 0, nk = 0;
    std::vector<double> cnt, qo, qs, ql, num, den, qi_sum, qi_num, qi_cnt, qi_den;
    std::vector<uint64_t> c_num, c_den, c_qnum, c_qden;
};

struct Round {
    cudaEvent_t start = nullptr, end = nullptr;
    std::vector<Request *> finishing;
};

long long tiles_of(long long n) { return (n + 127) / 128; }

}  // namespace

struct hbt_server {
    hbt_server_config cfg{};
    int grid = 0;
    cudaMemPool_t pool = nullptr;
    cudaStream_t upload = nullptr, rounds = nullptr;
    hbt::BatchRunner runner;

    std::mutex mu;
    std::condition_variable cv_work;  // worker: new requests or stop
    std::condition_variable cv_done;  // waiters
    std::condition_variable cv_solo;
    std::condition_variable cv_complete;  // completion thread: finished rounds
    bool stop = false, worker_done = false;
    std::string err;
    uint64_t next_id = 1;
    std::map<uint64_t, std::unique_ptr<Request>> jobs;
    std::deque<Request *> queued;
    std::deque<Request *> solo_queue;
    // requests whose last round retired, with the round's status, waiting
    // for their results to be copied out (completion thread)
    struct Done {
        Request *q;
        hbt_status st;
        std::string err;
    };
    std::deque<Done> done_queue;

    // statistics (under mu)
    u64 submitted = 0, completed = 0, failed = 0, n_rounds = 0, pairs = 0;
    u64 bytes_in_use = 0, peak_bytes = 0;
    int active = 0, peak_active = 0;
    std::vector<double> latencies;
    double busy_ms = 0.0;

    // worker-only
    std::vector<Request *> batched;  // admitted, batched path, admission order
    std::deque<Round> in_flight;
    std::vector<cudaEvent_t> spare_events;

    std::thread worker, solo, completer;
};

namespace {

void set_err(hbt_server *s, const std::string &m) {
    std::lock_guard<std::mutex> lk(s->mu);
    s->err = m;
}

cudaEvent_t take_event(hbt_server *s, bool timing) {
    if (!timing && !s->spare_events.empty()) {
        cudaEvent_t e = s->spare_events.back();
        s->spare_events.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreateWithFlags(&e, timing ? cudaEventDefault : cudaEventDisableTiming);
    return e;
}

// Host part of a request: rapidity cut, event-plane angle, mixing draws.
hbt_status prepare(const hbt_request &r, Request &q, std::string &err) {
    if (!hbt::params_valid(r.params)) {
        err = "invalid hbt_params";
        return HBT_ERR_INVALID;
    }
    if (r.n_events < 1 || !r.event_offsets || r.event_offsets[0] != 0 || r.seed < 0 ||
        r.oversample < 0 || r.mixed_partners < 0) {
        err = "invalid request (events, offsets, seed, oversample or partners)";
        return HBT_ERR_INVALID;
    }
    for (int e = 0; e < r.n_events; e++)
        if (r.event_offsets[e + 1] < r.event_offsets[e]) {
            err = "event offsets must not decrease";
            return HBT_ERR_INVALID;
        }
    const long long total = r.event_offsets[r.n_events];
    const double *src[8] = {r.particles.px, r.particles.py, r.particles.pz, r.particles.E,
                            r.particles.x,  r.particles.y,  r.particles.z,  r.particles.t};
    if (total > 0)
        for (const double *p : src)
            if (!p) {
                err = "null particle column";
                return HBT_ERR_INVALID;
            }
    q.prm = r.params;
    q.n_events = r.n_events;
    q.oversample = r.oversample > 0 ? std::min(r.oversample, r.n_events) : r.n_events;
    q.partners = r.mixed_partners > 0 ? r.mixed_partners : r.n_events / 2 + 1;

    // event-plane angle of the buffer, all particles of its events
    // (calculate_flow_event_plane_angle(2), src/HBT_correlation.cpp:233-249)
    if (r.params.azimuthal_flag == 1) {
        double vr = 0.0, vi = 0.0;
        for (long long k = 0; k < total; k++) {
            const double phi = atan2(src[1][k], src[0][k]);
            vr += cos(2 * phi);
            vi += sin(2 * phi);
        }
        q.psi = atan2(vi, vr) / 2;
    }

    // rapidity cut of the gathers (src/HBT_correlation.cpp:254-285, 466-552)
    const double ycut_max = tanh(r.Krap_max), ycut_min = tanh(r.Krap_min);
    std::vector<long long> keep;
    keep.reserve(total);
    q.off.assign(r.n_events + 1, 0);
    for (int e = 0; e < r.n_events; e++) {
        for (long long k = r.event_offsets[e]; k < r.event_offsets[e + 1]; k++) {
            const double ratio = src[2][k] / src[3][k];
            if (ratio > ycut_min && ratio < ycut_max) keep.push_back(k);
        }
        q.off[e + 1] = (long long)keep.size();
    }
    q.n = (long long)keep.size();
    q.cols.resize((size_t)8 * q.n);
    for (int f = 0; f < 8; f++)
        for (long long k = 0; k < q.n; k++) q.cols[(size_t)f * q.n + k] = src[f][keep[k]];

    // same-event pairs per oversample group
    for (int g0 = 0; g0 < r.n_events; g0 += q.oversample) {
        const int g1 = std::min(g0 + q.oversample, r.n_events);
        const u64 n = (u64)(q.off[g1] - q.off[g0]);
        if (n >= 2) q.pairs_same += n * (n - 1) / 2;
    }

    // mixing draws in the reference's order (src/HBT_correlation.cpp:202-215
    // draws the partners of an event, then combine_and_bin_particle_pairs_
    // mixed_events draws their rotation angles, src/HBT_correlation.cpp:
    // 494-497): std::mt19937(seed), uniform_int_distribution<int> over
    // [0, INT_MAX], uniform_real_distribution<double> over [0, 1)
    std::mt19937 gen(static_cast<std::mt19937::result_type>(r.seed));
    std::uniform_real_distribution<double> uni(0.0, 1.0);
    std::uniform_int_distribution<int> uint_(0, INT_MAX);
    const int P = q.partners, nev = r.n_events;
    q.partner.assign((size_t)nev * P, 0);
    q.cphi.assign((size_t)nev * P, 1.0);
    q.sphi.assign((size_t)nev * P, 0.0);
    q.roff.assign(nev + 1, 0);
    for (int e = 0; e < nev; e++) {
        for (int k = 0; k < P; k++) {
            int id = uint_(gen) % nev;
            while (e == id && nev != 1) id = uint_(gen) % nev;
            q.partner[(size_t)e * P + k] = id;
        }
        long long rows = 0;
        for (int k = 0; k < P; k++) {
            const double rot = uni(gen) * 2 * M_PI;
            q.cphi[(size_t)e * P + k] = cos(rot);
            q.sphi[(size_t)e * P + k] = sin(rot);
            const int id = q.partner[(size_t)e * P + k];
            rows += q.off[id + 1] - q.off[id];
        }
        q.roff[e + 1] = q.roff[e] + rows;
        q.pairs_mixed += (u64)(q.off[e + 1] - q.off[e]) * (u64)rows;
    }
    q.m = q.roff[nev];

    q.nb = (long long)(r.params.azimuthal_flag == 1 ? r.params.n_KT * r.params.n_Kphi
                                                    : r.params.n_KT) *
           r.params.qnpts * r.params.qnpts * r.params.qnpts;
    q.ns = r.params.azimuthal_flag == 1 ? (long long)r.params.n_KT * r.params.n_Kphi
                                        : r.params.n_KT;
    q.nk = r.params.n_KT;
    q.nq = (long long)r.params.n_KT * r.params.qnpts;
    q.bytes = hbt::ctx_device_bytes(r.params) + ((size_t)8 * q.n + (size_t)4 * q.m) * 8 + 4096;
    return HBT_OK;
}

// Creates the request's context and device buffers and uploads its
// particles and rotated partner lists on the upload stream.
hbt_status admit(hbt_server *s, Request &q, std::string &err) {
    hbt_status st = hbt::ctx_create(&q.prm, s->cfg.device, s->pool, &q.ctx);
    if (st != HBT_OK) {
        err = "context creation failed";
        return st;
    }
    if (q.prm.azimuthal_flag == 1) hbt_set_psi_ref(q.ctx, q.psi);
    q.solo = !hbt::ctx_batchable(q.ctx) || hbt::ctx_caps_may_bind(q.ctx, 0, q.pairs_same) ||
             hbt::ctx_caps_may_bind(q.ctx, 1, q.pairs_mixed);
    const size_t cbytes = (size_t)8 * std::max(q.n, 1LL) * sizeof(double);
    const size_t rbytes = (size_t)4 * std::max(q.m, 1LL) * sizeof(double);
    if (cudaMallocFromPoolAsync(reinterpret_cast<void **>(&q.dcols), cbytes, s->pool, s->upload) !=
            cudaSuccess ||
        cudaMallocFromPoolAsync(reinterpret_cast<void **>(&q.drot), rbytes, s->pool, s->upload) !=
            cudaSuccess) {
        err = "device allocation of the particle buffers failed";
        return HBT_ERR_NOMEM;
    }
    if (q.n > 0 && cudaMemcpyAsync(q.dcols, q.cols.data(), (size_t)8 * q.n * sizeof(double),
                                   cudaMemcpyHostToDevice, s->upload) != cudaSuccess) {
        err = "particle upload failed";
        return HBT_ERR_CUDA;
    }
    // rotated partner lists
    std::vector<Segment> seg;
    const int P = q.partners;
    for (int e = 0; e < q.n_events; e++) {
        long long dst = q.roff[e];
        for (int k = 0; k < P; k++) {
            const int id = q.partner[(size_t)e * P + k];
            const long long n = q.off[id + 1] - q.off[id];
            if (n > 0)
                seg.push_back({dst, q.off[id], n, q.cphi[(size_t)e * P + k],
                               q.sphi[(size_t)e * P + k]});
            dst += n;
        }
    }
    if (!seg.empty()) {
        Segment *dseg = nullptr;
        if (cudaMallocFromPoolAsync(reinterpret_cast<void **>(&dseg), seg.size() * sizeof(Segment),
                                    s->pool, s->upload) != cudaSuccess ||
            cudaMemcpyAsync(dseg, seg.data(), seg.size() * sizeof(Segment),
                            cudaMemcpyHostToDevice, s->upload) != cudaSuccess) {
            err = "rotation table upload failed";
            return HBT_ERR_CUDA;
        }
        k_rotate<<<(unsigned)seg.size(), 256, 0, s->upload>>>(dseg, q.dcols, q.n, q.drot, q.m);
        if (cudaGetLastError() != cudaSuccess || cudaFreeAsync(dseg, s->upload) != cudaSuccess) {
            err = "rotation launch failed";
            return HBT_ERR_CUDA;
        }
    }
    q.ready = take_event(s, false);
    if (!q.ready || cudaEventRecord(q.ready, s->upload) != cudaSuccess) {
        err = "event record failed";
        return HBT_ERR_CUDA;
    }
    // host copies are no longer needed
    std::vector<double>().swap(q.cols);

    // pair work: same-event groups, then each event against its partners
    const hbt::Device &d = hbt::ctx_device(q.ctx);
    const double Q = std::max(std::fabs(d.g.q_lo), std::fabs(d.g.q_hi));
    for (int g0 = 0; g0 < q.n_events; g0 += q.oversample) {
        const int g1 = std::min(g0 + q.oversample, q.n_events);
        const long long a0 = q.off[g0], na = q.off[g1] - q.off[g0];
        if (na < 2) continue;
        hbt::FastJob j = {};
        j.kind = 0;
        j.na = na;
        for (int f = 0; f < 8; f++) j.a[f] = q.dcols + (size_t)f * q.n + a0;
        j.q_window = Q;
        j.boost = d.g.boost;
        q.work.push_back(j);
        const long long t = tiles_of(na);
        q.work_tiles.push_back(t * (t + 1) / 2);
    }
    for (int e = 0; e < q.n_events; e++) {
        const long long na = q.off[e + 1] - q.off[e], nb = q.roff[e + 1] - q.roff[e];
        if (na < 1 || nb < 1) continue;
        hbt::FastJob j = {};
        j.kind = 1;
        j.na = na;
        j.nb = nb;
        for (int f = 0; f < 4; f++) {
            j.a[f] = q.dcols + (size_t)f * q.n + q.off[e];
            j.b[f] = q.drot + (size_t)f * q.m + q.roff[e];
        }
        j.q_window = Q;
        j.boost = d.g.boost;
        q.work.push_back(j);
        q.work_tiles.push_back(tiles_of(na) * tiles_of(nb));
    }
    return HBT_OK;
}

// Copies the results to host memory and releases the device state.
hbt_status collect(hbt_server *s, Request &q, std::string &err) {
    hbt_status st = HBT_OK;
    q.cnt.resize(q.nb);
    q.qo.resize(q.nb);
    q.qs.resize(q.nb);
    q.ql.resize(q.nb);
    q.num.resize(q.nb);
    q.den.resize(q.nb);
    q.c_num.resize(q.ns);
    q.c_den.resize(q.ns);
    q.c_qnum.resize(q.nk);
    q.c_qden.resize(q.nk);
    if ((st = hbt_read_hist(q.ctx, q.cnt.data(), q.qo.data(), q.qs.data(), q.ql.data(),
                            q.num.data(), q.den.data())) != HBT_OK ||
        (st = hbt_read_counters(q.ctx, q.c_num.data(), q.c_den.data(), q.c_qnum.data(),
                                q.c_qden.data())) != HBT_OK) {
        err = hbt_last_error(q.ctx);
        return st;
    }
    hbt_stats hs;
    if ((st = hbt_get_stats(q.ctx, &hs)) != HBT_OK) {
        err = hbt_last_error(q.ctx);
        return st;
    }
    q.anomalies = hs.anomalies;
    if (q.prm.invariant_radius_flag == 1) {
        for (auto *v : {&q.qi_sum, &q.qi_num, &q.qi_cnt, &q.qi_den}) v->resize(q.nq);
        if ((st = hbt_read_qinv(q.ctx, q.qi_sum.data(), q.qi_num.data(), q.qi_cnt.data(),
                                q.qi_den.data())) != HBT_OK) {
            err = hbt_last_error(q.ctx);
            return st;
        }
    }
    return HBT_OK;
}

void release_device(hbt_server *s, Request &q) {
    cudaStream_t st = q.ctx ? hbt::ctx_stream(q.ctx) : s->upload;
    if (q.dcols) cudaFreeAsync(q.dcols, st);
    if (q.drot) cudaFreeAsync(q.drot, st);
    q.dcols = q.drot = nullptr;
    if (q.ctx) hbt_destroy(q.ctx);
    q.ctx = nullptr;
    if (q.ready) cudaEventDestroy(q.ready);
    q.ready = nullptr;
    q.work.clear();
    q.work.shrink_to_fit();
}

// Marks a request done (st == HBT_OK) or failed, frees its memory share.
void finish(hbt_server *s, Request &q, hbt_status st) {
    release_device(s, q);
    std::lock_guard<std::mutex> lk(s->mu);
    q.t_done = Clock::now();
    q.status = st;
    q.state = st == HBT_OK ? HBT_JOB_DONE : HBT_JOB_FAILED;
    s->bytes_in_use -= q.bytes;
    s->active--;
    if (st == HBT_OK) {
        s->completed++;
        s->pairs += q.pairs_same + q.pairs_mixed;
        s->latencies.push_back(ms_between(q.t_submit, q.t_done));
    } else {
        s->failed++;
    }
    s->cv_done.notify_all();
    s->cv_work.notify_all();  // memory and a slot are free for the queue
}

void solo_main(hbt_server *s) {
    cudaSetDevice(s->cfg.device);
    for (;;) {
        Request *q = nullptr;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            s->cv_solo.wait(lk, [&] { return s->stop || !s->solo_queue.empty(); });
            if (s->solo_queue.empty()) return;
            q = s->solo_queue.front();
            s->solo_queue.pop_front();
        }
        // the per-analysis entry points, in the reference's order
        hbt_status st = HBT_OK;
        std::string err;
        if (cudaStreamWaitEvent(hbt::ctx_stream(q->ctx), q->ready, 0) != cudaSuccess)
            st = HBT_ERR_CUDA;
        for (const hbt::FastJob &j : q->work) {
            if (st != HBT_OK) break;
            if (j.kind == 0) {
                const hbt_soa8 l = {j.a[0], j.a[1], j.a[2], j.a[3],
                                    j.a[4], j.a[5], j.a[6], j.a[7]};
                st = hbt_bin_same_dev(q->ctx, j.na, &l);
            } else {
                const hbt_soa4 a = {j.a[0], j.a[1], j.a[2], j.a[3]};
                const hbt_soa4 b = {j.b[0], j.b[1], j.b[2], j.b[3]};
                st = hbt_bin_mixed_dev(q->ctx, j.na, &a, j.nb, &b);
            }
            if (st != HBT_OK) err = hbt_last_error(q->ctx);
        }
        if (st == HBT_OK) st = collect(s, *q, err);
        if (st != HBT_OK) set_err(s, "request " + std::to_string(q->id) + ": " + err);
        finish(s, *q, st);
    }
}

// Copies out the results of requests whose last round retired and frees
// their device memory.
void completer_main(hbt_server *s) {
    cudaSetDevice(s->cfg.device);
    for (;;) {
        hbt_server::Done d;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            s->cv_complete.wait(lk, [&] { return s->worker_done || !s->done_queue.empty(); });
            if (s->done_queue.empty()) return;
            d = std::move(s->done_queue.front());
            s->done_queue.pop_front();
        }
        hbt_status st = d.st;
        std::string err = d.err;
        if (st == HBT_OK) {
            hbt::ctx_add_pairs(d.q->ctx, d.q->pairs_same, d.q->pairs_mixed);
            st = collect(s, *d.q, err);
        }
        if (st != HBT_OK) set_err(s, "request " + std::to_string(d.q->id) + ": " + err);
        finish(s, *d.q, st);
    }
}

// Completes the oldest round in flight (waits for it when `block`).
bool retire_round(hbt_server *s, bool block) {
    if (s->in_flight.empty()) return false;
    Round &r = s->in_flight.front();
    if (!block && cudaEventQuery(r.end) == cudaErrorNotReady) return false;
    const cudaError_t e = cudaEventSynchronize(r.end);
    float ms = 0.f;
    if (e == cudaSuccess) cudaEventElapsedTime(&ms, r.start, r.end);
    {
        // the completion thread copies the results out, so that the worker
        // goes on issuing rounds meanwhile
        std::lock_guard<std::mutex> lk(s->mu);
        for (Request *q : r.finishing)
            s->done_queue.push_back({q, e == cudaSuccess ? HBT_OK : HBT_ERR_CUDA,
                                     e == cudaSuccess ? "" : cudaGetErrorString(e)});
        if (!r.finishing.empty()) s->cv_complete.notify_one();
    }
    cudaEventDestroy(r.start);
    cudaEventDestroy(r.end);
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->busy_ms += ms;
    }
    s->in_flight.pop_front();
    return true;
}

// Builds and issues one round; false when no batched work is pending.
bool issue_round(hbt_server *s) {
    // kernel class of the oldest request with pending work
    Request *lead = nullptr;
    for (Request *q : s->batched)
        if (q->next < q->work.size()) {
            lead = q;
            break;
        }
    if (!lead) return false;
    const hbt::Device &ld = hbt::ctx_device(lead->ctx);
    const long long budget = s->cfg.round_tile_pairs;
    std::vector<hbt::FastJob> jobs;
    std::vector<hbt::Device> devs;
    std::vector<Request *> members;
    long long used = 0;
    for (Request *q : s->batched) {
        if (q->next >= q->work.size()) continue;
        const hbt::Device &d = hbt::ctx_device(q->ctx);
        if (d.g.azimuthal != ld.g.azimuthal || d.g.boost != ld.g.boost ||
            d.precision != ld.precision)
            continue;
        // whole work items in arrival order; an item larger than the budget
        // forms a round of its own
        const int dev = (int)devs.size();
        bool took = false;
        while (q->next < q->work.size()) {
            const long long t = q->work_tiles[q->next];
            if (used > 0 && used + t > budget) break;
            hbt::FastJob j = q->work[q->next];
            j.dev = dev;
            jobs.push_back(j);
            used += t;
            q->next++;
            took = true;
        }
        if (took) {
            devs.push_back(d);
            members.push_back(q);
            if (!q->waited) {
                cudaStreamWaitEvent(s->rounds, q->ready, 0);
                q->waited = true;
            }
            q->rounds++;
        }
        if (q->next < q->work.size()) break;  // the budget is reached
    }
    Round r;
    r.start = take_event(s, true);
    r.end = take_event(s, true);
    cudaEventRecord(r.start, s->rounds);
    std::string err;
    // rounds differ in shape: direct launches, no graph
    hbt::Tuning tu;
    tu.grid = 0;  // each persistent kernel at its own occupancy
    tu.chunk = ld.precision == HBT_PRECISION_FP32W ? (unsigned)ld.merge_chunk_blocks : 0u;
    tu.graph = false;
    const bool ok = s->runner.run_multi(jobs, devs, tu, s->rounds, err);
    cudaEventRecord(r.end, s->rounds);
    for (Request *q : members)
        if (!ok || q->next >= q->work.size()) r.finishing.push_back(q);
    if (!ok) {
        set_err(s, "round failed: " + err);
        for (Request *q : members) q->next = q->work.size();
    }
    // finished requests leave the batched list when their round retires
    s->batched.erase(std::remove_if(s->batched.begin(), s->batched.end(),
                                    [](Request *q) { return q->next >= q->work.size(); }),
                     s->batched.end());
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->n_rounds++;
    }
    s->in_flight.push_back(std::move(r));
    return true;
}

// Admits queued requests in arrival order while memory and slots allow.
void admit_queued(hbt_server *s) {
    for (;;) {
        Request *q = nullptr;
        {
            std::lock_guard<std::mutex> lk(s->mu);
            if (s->queued.empty()) return;
            Request *f = s->queued.front();
            if (s->active >= s->cfg.max_active ||
                s->bytes_in_use + f->bytes > s->cfg.memory_budget)
                return;
            s->queued.pop_front();
            q = f;
            s->active++;
            s->peak_active = std::max(s->peak_active, s->active);
            s->bytes_in_use += q->bytes;
            s->peak_bytes = std::max(s->peak_bytes, s->bytes_in_use);
            q->state = HBT_JOB_ACTIVE;
            q->t_admit = Clock::now();
        }
        std::string err;
        const hbt_status st = admit(s, *q, err);
        if (st != HBT_OK) {
            set_err(s, "request " + std::to_string(q->id) + ": " + err);
            finish(s, *q, st);
            continue;
        }
        if (q->solo) {
            std::lock_guard<std::mutex> lk(s->mu);
            s->solo_queue.push_back(q);
            s->cv_solo.notify_one();
        } else if (q->work.empty()) {
            // nothing to bin: results are the zero histograms
            cudaEventSynchronize(q->ready);
            std::lock_guard<std::mutex> lk(s->mu);
            s->done_queue.push_back({q, HBT_OK, ""});
            s->cv_complete.notify_one();
        } else {
            s->batched.push_back(q);
        }
    }
}

void worker_main(hbt_server *s) {
    cudaSetDevice(s->cfg.device);
    for (;;) {
        admit_queued(s);
        while (retire_round(s, false)) {
        }
        if ((int)s->in_flight.size() >= s->cfg.max_in_flight) {
            retire_round(s, true);
            continue;
        }
        if (issue_round(s)) continue;
        if (!s->in_flight.empty()) {
            retire_round(s, true);
            continue;
        }
        std::unique_lock<std::mutex> lk(s->mu);
        const bool can_admit =
            !s->queued.empty() && s->active < s->cfg.max_active &&
            s->bytes_in_use + s->queued.front()->bytes <= s->cfg.memory_budget;
        if (can_admit) continue;
        if (s->stop && s->active == 0) {
            // requests never admitted fail at shutdown
            for (Request *q : s->queued) {
                q->state = HBT_JOB_FAILED;
                q->status = HBT_ERR_STATE;
                s->failed++;
            }
            s->queued.clear();
            s->cv_done.notify_all();
            return;
        }
        s->cv_work.wait_for(lk, std::chrono::milliseconds(s->stop ? 1 : 50));
    }
}

Request *find(hbt_server *s, uint64_t id) {
    auto it = s->jobs.find(id);
    return it == s->jobs.end() ? nullptr : it->second.get();
}

double percentile(std::vector<double> v, double p) {
    if (v.empty()) return 0.0;
    std::sort(v.begin(), v.end());
    // nearest rank
    size_t k = (size_t)std::ceil(p / 100.0 * v.size());
    if (k < 1) k = 1;
    return v[std::min(k, v.size()) - 1];
}

}  // namespace

extern "C" {

hbt_status hbt_server_create(const hbt_server_config *cfg, hbt_server **out) {
    if (!cfg || !out) return HBT_ERR_INVALID;
    *out = nullptr;
    std::unique_ptr<hbt_server> s(new hbt_server());
    s->cfg = *cfg;
    if (s->cfg.max_active <= 0) s->cfg.max_active = 64;
    if (s->cfg.round_tile_pairs <= 0) s->cfg.round_tile_pairs = 65536;
    if (s->cfg.max_in_flight <= 0) s->cfg.max_in_flight = 2;
    if (cudaSetDevice(cfg->device) != cudaSuccess) return HBT_ERR_CUDA;
    if (s->cfg.memory_budget == 0) {
        size_t free_b = 0, total_b = 0;
        if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return HBT_ERR_CUDA;
        s->cfg.memory_budget = (uint64_t)(0.8 * (double)free_b);
    }
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = cfg->device;
    if (cudaMemPoolCreate(&s->pool, &props) != cudaSuccess) return HBT_ERR_CUDA;
    // keep freed memory in the pool for the next requests
    uint64_t keep = UINT64_MAX;
    cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &keep);
    if (cudaStreamCreateWithFlags(&s->upload, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&s->rounds, cudaStreamNonBlocking) != cudaSuccess)
        return HBT_ERR_CUDA;
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, cfg->device) != cudaSuccess)
        return HBT_ERR_CUDA;
    s->grid = sms * hbt::persistent_blocks_per_sm();
    hbt_server *raw = s.release();
    raw->worker = std::thread(worker_main, raw);
    raw->solo = std::thread(solo_main, raw);
    raw->completer = std::thread(completer_main, raw);
    *out = raw;
    return HBT_OK;
}

void hbt_server_destroy(hbt_server *s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    if (s->worker.joinable()) s->worker.join();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->worker_done = true;
        s->cv_solo.notify_all();
        s->cv_complete.notify_all();
    }
    if (s->solo.joinable()) s->solo.join();
    if (s->completer.joinable()) s->completer.join();
    cudaSetDevice(s->cfg.device);
    for (cudaEvent_t e : s->spare_events) cudaEventDestroy(e);
    if (s->upload) cudaStreamSynchronize(s->upload);
    if (s->rounds) cudaStreamSynchronize(s->rounds);
    if (s->upload) cudaStreamDestroy(s->upload);
    if (s->rounds) cudaStreamDestroy(s->rounds);
    if (s->pool) cudaMemPoolDestroy(s->pool);
    delete s;
}

const char *hbt_server_last_error(const hbt_server *s) {
    return s ? s->err.c_str() : "null server";
}

hbt_status hbt_server_submit(hbt_server *s, const hbt_request *req, uint64_t *job_id) {
    if (!s || !req || !job_id) return HBT_ERR_INVALID;
    std::unique_ptr<Request> q(new Request());
    q->t_submit = Clock::now();
    std::string err;
    const hbt_status st = prepare(*req, *q, err);
    if (st != HBT_OK) {
        set_err(s, err);
        return st;
    }
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) {
        s->err = "server is stopping";
        return HBT_ERR_STATE;
    }
    if (q->bytes > s->cfg.memory_budget) {
        s->err = "request needs more device memory than the server's budget";
        return HBT_ERR_NOMEM;
    }
    q->id = s->next_id++;
    *job_id = q->id;
    s->queued.push_back(q.get());
    s->jobs[q->id] = std::move(q);
    s->submitted++;
    s->cv_work.notify_all();
    return HBT_OK;
}

hbt_status hbt_server_wait(hbt_server *s, uint64_t job_id, uint64_t timeout_us) {
    if (!s) return HBT_ERR_INVALID;
    std::unique_lock<std::mutex> lk(s->mu);
    Request *q = find(s, job_id);
    if (!q) return HBT_ERR_INVALID;
    auto done = [&] { return q->state == HBT_JOB_DONE || q->state == HBT_JOB_FAILED; };
    if (timeout_us == 0)
        s->cv_done.wait(lk, done);
    else if (!s->cv_done.wait_for(lk, std::chrono::microseconds(timeout_us), done))
        return HBT_ERR_TIMEOUT;
    return q->state == HBT_JOB_DONE ? HBT_OK : (hbt_status)q->status;
}

hbt_status hbt_server_job_info(hbt_server *s, uint64_t job_id, hbt_job_info *out) {
    if (!s || !out) return HBT_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    Request *q = find(s, job_id);
    if (!q) return HBT_ERR_INVALID;
    memset(out, 0, sizeof(*out));
    out->state = q->state;
    out->status = q->status;
    out->solo = q->solo ? 1 : 0;
    out->rounds = q->rounds;
    if (q->state != HBT_JOB_QUEUED) out->queue_ms = ms_between(q->t_submit, q->t_admit);
    if (q->state == HBT_JOB_DONE || q->state == HBT_JOB_FAILED)
        out->latency_ms = ms_between(q->t_submit, q->t_done);
    out->pairs_same = q->pairs_same;
    out->pairs_mixed = q->pairs_mixed;
    out->device_bytes = q->bytes;
    out->psi_ref = q->psi;
    out->n_bins = q->nb;
    out->anomalies = q->anomalies;
    return HBT_OK;
}

hbt_status hbt_server_mixing(hbt_server *s, uint64_t job_id, int32_t *partners_per_event,
                             int32_t *partners, double *cos_phi, double *sin_phi) {
    if (!s) return HBT_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    Request *q = find(s, job_id);
    if (!q) return HBT_ERR_INVALID;
    if (partners_per_event) *partners_per_event = q->partners;
    const size_t n = q->partner.size();
    for (size_t k = 0; k < n; k++) {
        if (partners) partners[k] = q->partner[k];
        if (cos_phi) cos_phi[k] = q->cphi[k];
        if (sin_phi) sin_phi[k] = q->sphi[k];
    }
    return HBT_OK;
}

hbt_status hbt_server_read_hist(hbt_server *s, uint64_t job_id, double *num_count,
                                double *q_out_sum, double *q_side_sum, double *q_long_sum,
                                double *num, double *den) {
    if (!s) return HBT_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    Request *q = find(s, job_id);
    if (!q) return HBT_ERR_INVALID;
    if (q->state != HBT_JOB_DONE) return HBT_ERR_STATE;
    const std::vector<double> *src[6] = {&q->cnt, &q->qo, &q->qs, &q->ql, &q->num, &q->den};
    double *dst[6] = {num_count, q_out_sum, q_side_sum, q_long_sum, num, den};
    for (int k = 0; k < 6; k++)
        if (dst[k]) std::copy(src[k]->begin(), src[k]->end(), dst[k]);
    return HBT_OK;
}

hbt_status hbt_server_read_qinv(hbt_server *s, uint64_t job_id, double *qinv_sum, double *num,
                                double *num_count, double *den) {
    if (!s) return HBT_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    Request *q = find(s, job_id);
    if (!q) return HBT_ERR_INVALID;
    if (q->state != HBT_JOB_DONE) return HBT_ERR_STATE;
    const std::vector<double> *src[4] = {&q->qi_sum, &q->qi_num, &q->qi_cnt, &q->qi_den};
    double *dst[4] = {qinv_sum, num, num_count, den};
    for (int k = 0; k < 4; k++)
        if (dst[k]) {
            if (src[k]->empty())
                std::fill(dst[k], dst[k] + q->nq, 0.0);
            else
                std::copy(src[k]->begin(), src[k]->end(), dst[k]);
        }
    return HBT_OK;
}

hbt_status hbt_server_read_counters(hbt_server *s, uint64_t job_id, uint64_t *num,
                                    uint64_t *den, uint64_t *num_qinv, uint64_t *den_qinv) {
    if (!s) return HBT_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    Request *q = find(s, job_id);
    if (!q) return HBT_ERR_INVALID;
    if (q->state != HBT_JOB_DONE) return HBT_ERR_STATE;
    const std::vector<uint64_t> *src[4] = {&q->c_num, &q->c_den, &q->c_qnum, &q->c_qden};
    uint64_t *dst[4] = {num, den, num_qinv, den_qinv};
    for (int k = 0; k < 4; k++)
        if (dst[k]) std::copy(src[k]->begin(), src[k]->end(), dst[k]);
    return HBT_OK;
}

hbt_status hbt_server_release(hbt_server *s, uint64_t job_id) {
    if (!s) return HBT_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    Request *q = find(s, job_id);
    if (!q) return HBT_ERR_INVALID;
    if (q->state != HBT_JOB_DONE && q->state != HBT_JOB_FAILED) return HBT_ERR_STATE;
    s->jobs.erase(job_id);
    return HBT_OK;
}

hbt_status hbt_server_get_stats(hbt_server *s, hbt_server_stats *out) {
    if (!s || !out) return HBT_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    memset(out, 0, sizeof(*out));
    out->submitted = s->submitted;
    out->completed = s->completed;
    out->failed = s->failed;
    out->rounds = s->n_rounds;
    out->pairs = s->pairs;
    out->bytes_in_use = s->bytes_in_use;
    out->peak_bytes = s->peak_bytes;
    out->active = s->active;
    out->queued = (int32_t)s->queued.size();
    out->peak_active = s->peak_active;
    out->p50_ms = percentile(s->latencies, 50.0);
    out->p99_ms = percentile(s->latencies, 99.0);
    double sum = 0.0, mx = 0.0;
    for (double v : s->latencies) {
        sum += v;
        mx = std::max(mx, v);
    }
    out->mean_ms = s->latencies.empty() ? 0.0 : sum / s->latencies.size();
    out->max_ms = mx;
    out->gpu_busy_ms = s->busy_ms;
    return HBT_OK;
}

hbt_status hbt_server_reset_stats(hbt_server *s) {
    if (!s) return HBT_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    s->latencies.clear();
    s->completed = s->failed = s->n_rounds = s->pairs = 0;
    s->submitted = 0;
    s->peak_bytes = s->bytes_in_use;
    s->peak_active = s->active;
    s->busy_ms = 0.0;
    return HBT_OK;
}

}  // extern "C"
