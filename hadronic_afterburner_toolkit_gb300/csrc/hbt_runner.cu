// BatchRunner: device tables and scratch of the batched pair binning.
#include "hbt_runner.h"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace hbt {

BatchRunner::~BatchRunner() {
    if (exec_) cudaGraphExecDestroy(exec_);
    for (cudaEvent_t e : marks_)
        if (e) cudaEventDestroy(e);
    Buf *all[] = {&lists_, &jobs_, &offs_, &table_, &keys_, &vals_, &sort_temp_, &boxes_,
                  &items_, &counters_, &devs_, &item_order_, &item_sort_temp_};
    for (Buf *b : all)
        if (b->p) cudaFree(b->p);
}

bool BatchRunner::grow(Buf &b, size_t bytes, std::string &err) {
    if (b.p && b.bytes >= bytes) return true;
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.bytes = 0;
    // a cached graph refers to the old buffers
    key_.clear();
    last_key_.clear();
    if (bytes == 0) return true;
    // a little headroom so slowly growing batches do not reallocate each time
    const size_t want = bytes + bytes / 8;
    if (cudaMalloc(&b.p, want) != cudaSuccess) {
        err = "cudaMalloc of batch scratch failed";
        b.p = nullptr;
        return false;
    }
    b.bytes = want;
    return true;
}

bool BatchRunner::run(const std::vector<FastJob> &jobs, const Device &d, const Tuning &t,
                      cudaStream_t st, std::string &err, int mode) {
    return run_impl(jobs, d, nullptr, nullptr, 0, t, st, err, mode);
}

bool BatchRunner::run_multi(const std::vector<FastJob> &jobs, const std::vector<Device> &devs,
                            const Tuning &t, cudaStream_t st, std::string &err) {
    if (devs.empty()) {
        err = "no analyses in the batch";
        return false;
    }
    for (const FastJob &j : jobs)
        if (j.dev < 0 || j.dev >= (int)devs.size()) {
            err = "job refers to a missing analysis";
            return false;
        }
    for (const Device &x : devs)
        if (x.g.azimuthal != devs[0].g.azimuthal || x.g.boost != devs[0].g.boost ||
            x.precision != devs[0].precision || x.g.qinv != devs[0].g.qinv) {
            err = "analyses of one batch must share azimuthal_flag, boost, precision and "
                  "invariant_radius_flag";
            return false;
        }
    if (!grow(devs_, devs.size() * sizeof(Device), err)) return false;
    if (cudaMemcpyAsync(devs_.p, devs.data(), devs.size() * sizeof(Device),
                        cudaMemcpyHostToDevice, st) != cudaSuccess) {
        err = "uploading the analysis descriptors failed";
        return false;
    }
    return run_impl(jobs, devs[0], static_cast<const Device *>(devs_.p), devs.data(),
                    (int)devs.size(), t, st, err, MODE_FAST);
}

// The graph captured for one set of launch arguments stays valid while they
// are unchanged: the batch tables it reads are re-uploaded before each
// launch, into the same buffers.
bool BatchRunner::tile_counts(long long &cand_same, long long &cand_mixed, long long &kept_same,
                              long long &kept_mixed) {
    cand_same = last_same_;
    cand_mixed = last_mixed_;
    kept_same = kept_mixed = 0;
    if (!counters_.p || last_pairs_ == 0) return last_pairs_ == 0;
    unsigned n[2] = {0, 0};
    if (cudaMemcpyAsync(n, counters_.p, sizeof(n), cudaMemcpyDeviceToHost, last_stream_) !=
            cudaSuccess ||
        cudaStreamSynchronize(last_stream_) != cudaSuccess)
        return false;
    kept_same = std::min<long long>(n[0], last_same_);
    kept_mixed = std::min<long long>(n[1], last_mixed_);
    return true;
}

bool BatchRunner::kernel_times(float &same_ms, float &mixed_ms) {
    same_ms = mixed_ms = 0.f;
    if (!timed_ || cudaEventSynchronize(marks_[3]) != cudaSuccess) return false;
    return cudaEventElapsedTime(&same_ms, marks_[0], marks_[1]) == cudaSuccess &&
           cudaEventElapsedTime(&mixed_ms, marks_[2], marks_[3]) == cudaSuccess;
}

cudaError_t BatchRunner::launch(const Device &d, const BatchDev &b, const Device *devs_host,
                                int n_devs, const Tuning &t, cudaStream_t st, int mode) {
    cudaEvent_t *marks = nullptr;
    if (t.time_kernels) {
        for (cudaEvent_t &e : marks_)
            if (!e && cudaEventCreate(&e) != cudaSuccess) return cudaErrorMemoryAllocation;
        marks = marks_;
    }
    timed_ = marks != nullptr;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (!t.graph || st == nullptr || cudaStreamIsCapturing(st, &cap) != cudaSuccess ||
        cap != cudaStreamCaptureStatusNone) {
        last_reuse_ = -1;
        return run_batch(d, b, t.grid, t.chunk, devs_host, n_devs, st, marks, mode);
    }
    std::vector<unsigned char> key;
    auto put = [&](const void *p, size_t n) {
        const unsigned char *c = static_cast<const unsigned char *>(p);
        key.insert(key.end(), c, c + n);
    };
    put(&d, sizeof(d));
    put(&b, sizeof(b));
    put(&t.grid, sizeof(t.grid));
    put(&t.chunk, sizeof(t.chunk));
    put(&n_devs, sizeof(n_devs));
    put(&timed_, sizeof(timed_));
    put(&mode, sizeof(mode));
    if (n_devs > 0) put(devs_host, sizeof(Device) * n_devs);
    if (exec_ && key == key_) {
        last_reuse_ = 1;
        return cudaGraphLaunch(exec_, st);
    }
    if (key != last_key_) {
        // a new shape: run directly; capture if it comes again
        last_key_.swap(key);
        last_reuse_ = -1;
        return run_batch(d, b, t.grid, t.chunk, devs_host, n_devs, st, marks, mode);
    }
    cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return e;
    const cudaError_t run_e = run_batch(d, b, t.grid, t.chunk, devs_host, n_devs, st, marks, mode);
    cudaGraph_t g = nullptr;
    e = cudaStreamEndCapture(st, &g);
    if (run_e != cudaSuccess || e != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        key_.clear();
        return run_e != cudaSuccess ? run_e : e;
    }
    bool updated = false;
    if (exec_) {
        cudaGraphExecUpdateResultInfo info;
        updated = cudaGraphExecUpdate(exec_, g, &info) == cudaSuccess;
        if (!updated) {
            cudaGetLastError();  // clear the update's error
            cudaGraphExecDestroy(exec_);
            exec_ = nullptr;
        }
    }
    if (!updated) e = cudaGraphInstantiate(&exec_, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        exec_ = nullptr;
        key_.clear();
        return e;
    }
    key_.swap(key);
    last_reuse_ = 0;
    return cudaGraphLaunch(exec_, st);
}

bool BatchRunner::run_impl(const std::vector<FastJob> &jobs, const Device &d,
                           const Device *devs_dev, const Device *devs_host, int n_devs,
                           const Tuning &t, cudaStream_t st, std::string &err, int mode) {
    std::vector<BatchList> lists;
    std::vector<BatchJob> bj;
    std::vector<long long> list_off, tile_off, pair_off;
    long long total = 0, tiles = 0, pairs = 0, same_pairs = 0, mixed_pairs = 0;
    auto add_list = [&](const double *const *src, int ncols, long long n) {
        BatchList l = {};
        for (int f = 0; f < 8; f++) l.src[f] = f < ncols ? src[f] : nullptr;
        l.n = n;
        l.off = total;
        l.tiles = (n + 127) / 128;
        l.tile_off = tiles;
        l.ncols = ncols;
        list_off.push_back(total);
        tile_off.push_back(tiles);
        total += n;
        tiles += l.tiles;
        lists.push_back(l);
        return (int)lists.size() - 1;
    };
    for (const FastJob &j : jobs) {
        BatchJob b = {};
        b.kind = j.kind;
        if (j.kind == 0) {
            if (j.na < 2) continue;
            b.la = b.lb = add_list(j.a, 8, j.na);
            const long long t = lists[b.la].tiles;
            b.n_pairs = t * (t + 1) / 2;
            same_pairs += b.n_pairs;
        } else {
            if (j.na < 1 || j.nb < 1) continue;
            b.la = add_list(j.a, 4, j.na);
            b.lb = add_list(j.b, 4, j.nb);
            b.n_pairs = lists[b.la].tiles * lists[b.lb].tiles;
            mixed_pairs += b.n_pairs;
        }
        b.pair_off = pairs;
        b.dev = j.dev;
        b.qt2_max = 2.0 * j.q_window * j.q_window * (1.0 + 1e-6) + 1e-300;
        b.ql_max = j.q_window * (1.0 + 1e-6) + 1e-300;
        b.boost = j.boost;
        b.qinv = j.qinv;
        b.row_base = j.row_base;
        pair_off.push_back(pairs);
        pairs += b.n_pairs;
        bj.push_back(b);
    }
    last_pairs_ = pairs;
    last_same_ = same_pairs;
    last_mixed_ = mixed_pairs;
    last_stream_ = st;
    if (bj.empty()) return true;
    if (same_pairs > 0xffffffffLL || mixed_pairs > 0xffffffffLL || total > 0x7fffffffLL) {
        err = "batch too large (tile pairs or particles)";
        return false;
    }
    const size_t sort_bytes = batch_sort_temp_bytes(total);
    if (!grow(lists_, lists.size() * sizeof(BatchList), err) ||
        !grow(jobs_, bj.size() * sizeof(BatchJob), err) ||
        !grow(offs_, (2 * lists.size() + bj.size()) * sizeof(long long), err) ||
        !grow(table_, (size_t)8 * total * sizeof(double), err) ||
        !grow(keys_, (size_t)2 * total * sizeof(unsigned long long), err) ||
        !grow(vals_, (size_t)3 * total * sizeof(unsigned), err) ||
        !grow(sort_temp_, sort_bytes, err) || !grow(boxes_, (size_t)tiles * sizeof(Box), err) ||
        !grow(items_, (size_t)pairs * sizeof(Item), err) ||
        !grow(counters_, 4 * sizeof(unsigned), err))
        return false;
    if (t.order_items && same_pairs > 0 &&
        (!grow(item_order_, (size_t)4 * same_pairs * sizeof(unsigned), err) ||
         !grow(item_sort_temp_, item_sort_temp_bytes(same_pairs), err)))
        return false;
    std::vector<long long> offs(list_off);
    offs.insert(offs.end(), tile_off.begin(), tile_off.end());
    offs.insert(offs.end(), pair_off.begin(), pair_off.end());
    if (cudaMemcpyAsync(lists_.p, lists.data(), lists.size() * sizeof(BatchList),
                        cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemcpyAsync(jobs_.p, bj.data(), bj.size() * sizeof(BatchJob), cudaMemcpyHostToDevice,
                        st) != cudaSuccess ||
        cudaMemcpyAsync(offs_.p, offs.data(), offs.size() * sizeof(long long),
                        cudaMemcpyHostToDevice, st) != cudaSuccess) {
        err = "uploading the batch tables failed";
        return false;
    }
    BatchDev b;
    memset(&b, 0, sizeof(b));  // padding too: the bytes key the cached graph
    const long long *o = static_cast<const long long *>(offs_.p);
    b.lists = static_cast<const BatchList *>(lists_.p);
    b.jobs = static_cast<const BatchJob *>(jobs_.p);
    b.list_off = o;
    b.tile_off = o + lists.size();
    b.pair_off = o + 2 * lists.size();
    b.n_lists = (int)lists.size();
    b.n_jobs = (int)bj.size();
    b.total = total;
    b.total_tiles = tiles;
    b.total_pairs = pairs;
    b.cap = total;
    b.table = static_cast<double *>(table_.p);
    b.keys_in = static_cast<unsigned long long *>(keys_.p);
    b.keys_out = b.keys_in + total;
    b.vals_in = static_cast<unsigned *>(vals_.p);
    b.vals_out = b.vals_in + total;
    b.orig = b.vals_in + 2 * total;
    b.sort_temp = sort_temp_.p;
    b.sort_temp_bytes = sort_temp_.bytes;
    b.boxes = static_cast<Box *>(boxes_.p);
    b.items = static_cast<Item *>(items_.p);
    b.same_cap = (unsigned)same_pairs;
    b.mixed_cap = (unsigned)mixed_pairs;
    b.n_items = static_cast<unsigned *>(counters_.p);
    b.item_next = b.n_items + 2;
    b.p_extent = 1024 * t.cell_pt / 2;
    b.inv_cell_pt = 1.0 / t.cell_pt;
    b.y_extent = 1024 * t.cell_y / 2;
    b.inv_cell_y = 1.0 / t.cell_y;
    b.devs = devs_dev;
    b.n_devs = n_devs;
    b.order_items = t.order_items && same_pairs > 0 ? 1 : 0;
    if (b.order_items) {
        unsigned *o = static_cast<unsigned *>(item_order_.p);
        b.item_key_in = o;
        b.item_key_out = o + same_pairs;
        b.item_pos_in = o + 2 * same_pairs;
        b.item_pos_out = o + 3 * same_pairs;
        b.item_sort_temp = item_sort_temp_.p;
        b.item_sort_temp_bytes = item_sort_temp_.bytes;
    }
    const cudaError_t e = launch(d, b, devs_host, n_devs, t, st, mode);
    if (e != cudaSuccess) {
        err = std::string("batch launch failed: ") + cudaGetErrorString(e);
        return false;
    }
    return true;
}

}  // namespace hbt
