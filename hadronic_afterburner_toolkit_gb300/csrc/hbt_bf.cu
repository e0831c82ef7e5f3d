// Balance-function pair binning (include/hbt_bf.h).
//
// One CTA per event pair (job): the particles of list A in registers (one
// per thread), those of list B staged through shared memory in tiles of
// 128.  Every pair is binned in FP32 with rigorous error bounds (bin32);
// the pairs within those bounds of a bin edge or a cut run the reference's
// FP64 expressions (bin64, src/BalanceFunction.cpp:136-160 and :183-204;
// this unit is compiled with --fmad=false), so every bin is the
// reference's.  Counts go to a shared-memory histogram of Bnpts x 20,
// whose non-zero bins are added to the global histogram when the job is
// done.  The bins are few and every pair lands in one, so privatising the
// histogram in shared memory turns the pair rate's worth of global atomics
// into one per non-zero bin and job.
#include <algorithm>
#include <cmath>
#include <map>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/hbt_bf.h"

namespace {

constexpr int kTile = 128;
constexpr int kNphi = HBT_BF_NPHI;

// Resident CTAs per SM the kernel is compiled for (register budget).
#ifndef HBT_BF_MIN_BLOCKS
#define HBT_BF_MIN_BLOCKS 10
#endif

// A job with its particle ranges resolved in the concatenated arrays.
struct BfJob {
    long long a0, a1, b0, b1;
    double rotation;
    int hist, mixed;
};

// The reference's binning constants (src/BalanceFunction.cpp:29-35) and
// the reciprocals the screen multiplies by.
struct BfConst {
    double drap, Brap_min, dphi, Bphi_min;
    double inv_drap, inv_dphi;
    int Bnpts;
};

// The reference's FP64 binning of one pair (src/BalanceFunction.cpp
// :183-204; the same-event loop :136-157 has no rotation term, and adding
// a zero rotation changes no value): the flat bin, or -1 when skipped.
__device__ __forceinline__ int bin64(const BfConst &c, double pa, double ya, double pb, double yb,
                                     int mixed, double rot) {
    const double d = mixed ? (pa - pb) + rot : pa - pb;
    int ip = static_cast<int>(floor((d - c.Bphi_min) / c.dphi)) % kNphi;
    if (ip < 0) ip += kNphi;
    const double dy = ya - yb;
    if (fabs(dy) < 1e-10) return -1;
    if (dy < c.Brap_min) return -1;
    const int iy = static_cast<int>((dy - c.Brap_min) / c.drap);
    if (iy >= 0 && iy < c.Bnpts) return iy * kNphi + ip;
    return -1;
}

// A pair the FP32 screen leaves undecided, from the particles' FP64 values
// in global memory: equal rapidities (a particle with itself, when the two
// lists hold the same species) give dy = 0, which the reference skips;
// everything else runs the reference's expressions.  Out of line: it runs
// for about one pair in a thousand and keeps the loop's registers free.
__device__ __noinline__ int bin_slow(const BfConst &c, const double *phi, const double *y,
                                     long long ia, long long ib, int mixed, double rot) {
    const double ya = y[ia], yb = y[ib];
    if (ya == yb && fabs(ya) < INFINITY) return -1;
    return bin64(c, phi[ia], ya, phi[ib], yb, mixed, rot);
}

// The screen.  A pair's bins are the floors of two quotients,
//   T_phi = (phi_a - phi_b + rot - Bphi_min) / dphi   (taken mod 20),
//   T_y   = (y_a - y_b - Brap_min) / drap              (T_y < 0 is the
//           reference's dy < Brap_min cut),
// each the difference of a term of particle a and a term of particle b.
// The terms are computed once per particle in FP64, the phi term reduced
// mod 20 into [0, 20), and rounded to FP32 (error <= u |term|, u = 2^-24),
// so a pair costs one FP32 subtraction per quotient (error <= u (|term a| +
// |term b|)).  Each term carries a bound: 2.0001 u |term| for those
// roundings, 2^-46 times the magnitudes it was made of for the FP64
// arithmetic here and in the reference's own quotient, and on particle a
// 2e-7 for the FP32 rounding of 1 - bound.  When the fraction of both FP32
// differences clears the summed bounds, their floors are the reference's.
// A term of magnitude >= 1e9 (or NaN) becomes NaN: every pair of that
// particle then fails the screen and takes the FP64 path.
constexpr double kU64 = 0x1p-24;
constexpr float kU = 0x1p-24f;

__device__ __forceinline__ double wrap20(double x) {
    double r = x - 20.0 * floor(x * 0.05);
    if (r < 0.0) r += 20.0;
    if (r >= 20.0) r -= 20.0;
    return r;
}

__device__ __forceinline__ float4 pack_terms(double xp, double mp, double xy, double my,
                                             double slack) {
    if (!(fabs(xp) < 1e9 && fabs(xy) < 1e9)) return make_float4(NAN, 0.f, NAN, 0.f);
    const float tp = (float)wrap20(xp), ty = (float)xy;
    const float ep = (float)(2.0001 * kU64 * fabs((double)tp) + 0x1p-46 * (mp + 40.0) + slack);
    const float ey = (float)(2.0001 * kU64 * fabs((double)ty) + 0x1p-46 * my + slack);
    return make_float4(tp, ep, ty, ey);
}

// Particle a's terms as the pair loop uses them: the azimuthal term plus
// 19.5 and the rapidity term minus 0.5 (both shifts in FP64 before the
// rounding to FP32, inside the bound), so that rint of a pair's difference
// is the floor of the unshifted one (plus 20 for the azimuth: a column in
// [0, 40) of a histogram whose columns c and c + 20 are the same bin), and
// each bound as its distance to a half-integer, 0.5 - bound.
__device__ __forceinline__ float4 pack_terms_a(double xp, double mp, double xy, double my) {
    if (!(fabs(xp) < 1e9 && fabs(xy) < 1e9)) return make_float4(NAN, 0.f, NAN, 0.f);
    const double sp = wrap20(xp) + 19.5, sy = xy - 0.5;
    const float tp = (float)sp, ty = (float)sy;
    const double ep = 2.0001 * kU64 * fabs((double)tp) + 0x1p-46 * (mp + 60.0) + 2e-7;
    const double ey = 2.0001 * kU64 * fabs((double)ty) + 0x1p-46 * (my + 1.0) + 2e-7;
    return make_float4(tp, (float)(0.5 - ep), ty, (float)(0.5 - ey));
}

// Particle a: (phi + rot - Bphi_min) / dphi and (y - Brap_min) / drap,
// shifted (pack_terms_a).
__device__ __forceinline__ float4 terms_a(const BfConst &c, double phi, double y, double rot) {
    return pack_terms_a(((phi + rot) - c.Bphi_min) * c.inv_dphi,
                        (fabs(phi) + fabs(rot) + fabs(c.Bphi_min)) * c.inv_dphi,
                        (y - c.Brap_min) * c.inv_drap, (fabs(y) + fabs(c.Brap_min)) * c.inv_drap);
}

// Particle b: phi / dphi and y / drap.
__device__ __forceinline__ float4 terms_b(const BfConst &c, double phi, double y) {
    return pack_terms(phi * c.inv_dphi, fabs(phi) * c.inv_dphi, y * c.inv_drap,
                      fabs(y) * c.inv_drap, 0.0);
}

// The |dy| < 1e-10 cut: |dy| from FP32 copies errs by at most u (|y_a| +
// |y_b| + |dy|); the pair certainly passes when |dy| exceeds 7 u per
// magnitude plus 1.0001e-10 (1e-10f itself rounds above 1e-10).
__device__ __forceinline__ float2 dy_terms(double y, float slack) {
    const float fy = (float)y;
    return make_float2(fy, 7.0f * kU * fabsf(fy) + slack);
}

// Every particle's b terms, once per call.
__global__ void k_bf_terms(long long n, const double *phi, const double *y, BfConst c,
                           float4 *tb, float2 *yb) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        tb[i] = terms_b(c, phi[i], y[i]);
        yb[i] = dy_terms(y[i], 0.f);
    }
}

// One work item per (job, tile of up to 128 particles of list A): a job of
// n_a particles is ceil(n_a / 128) items, so the grid holds several waves
// of similar items instead of one CTA per event pair.  A's terms sit in
// registers (one particle per thread), B's are staged through shared memory
// 128 at a time; the histogram is privatised in shared memory and its
// non-zero bins are added to the global one when the item is done.
__global__ void __launch_bounds__(kTile, HBT_BF_MIN_BLOCKS)
    k_bf(const BfJob *jobs, const int2 *items, long long n_items, const double *phi,
         const double *y, const float4 *tb, const float2 *yb, BfConst c,
         unsigned long long *hist, unsigned long long *n_slow) {
    extern __shared__ unsigned sh[];  // [Bnpts][2 kNphi]: columns c and c + 20 are bin c
    __shared__ float4 sb[kTile];
    __shared__ float2 sd[kTile];
    __shared__ BfJob sj;
    const int nbins = c.Bnpts * kNphi, nsh = 2 * nbins;
    unsigned slow = 0;
    for (long long it = blockIdx.x; it < n_items; it += gridDim.x) {
        const int2 item = items[it];
        for (int k = threadIdx.x; k < nsh; k += blockDim.x) sh[k] = 0u;
        if (threadIdx.x == 0) sj = jobs[item.x];
        __syncthreads();
        const long long ia = sj.a0 + item.y + threadIdx.x;
        const bool have = ia < sj.a1;
        float4 A = make_float4(0.f, 0.f, 0.f, 0.f);
        float2 Ay = make_float2(0.f, 0.f);
        if (have) {
            A = terms_a(c, phi[ia], y[ia], sj.mixed ? sj.rotation : 0.0);
            Ay = dy_terms(y[ia], 1.0001e-10f);
        }
        for (long long b = sj.b0; b < sj.b1; b += kTile) {
            if (b + threadIdx.x < sj.b1) {
                sb[threadIdx.x] = tb[b + threadIdx.x];
                sd[threadIdx.x] = yb[b + threadIdx.x];
            }
            __syncthreads();
            const int nb = (int)min((long long)kTile, sj.b1 - b);
            if (have) {
#pragma unroll 2
                for (int j = 0; j < nb; j++) {
                    const float4 B = sb[j];
                    const float2 By = sd[j];
                    // shifted differences: rint gives the floors (the azimuth
                    // + 20); certain when their distance to the rint is
                    // below 0.5 - bound
                    const float tp = A.x - B.x, ty = A.z - B.z;
                    const float kp = rintf(tp), ky = rintf(ty);
                    int k;
                    if (fabsf(tp - kp) < A.y - B.y && fabsf(ty - ky) < A.w - B.w &&
                        fabsf(Ay.x - By.x) > Ay.y + By.y) {
                        // tp in (-0.5, 39.5): column kp in [0, 39]; a row ky
                        // beyond [0, Bnpts) puts k outside the histogram
                        // (|ty| < 2^23 here, so k fits an int)
                        k = (int)__fmaf_rn(ky, 2.0f * kNphi, kp);
                    } else {
                        const int k20 = bin_slow(c, phi, y, ia, b + j, sj.mixed, sj.rotation);
                        k = k20 < 0 ? -1 : (k20 / kNphi) * (2 * kNphi) + k20 % kNphi;
                        slow++;
                    }
                    if ((unsigned)k < (unsigned)nsh) atomicAdd(&sh[k], 1u);
                }
            }
            __syncthreads();
        }
        unsigned long long *h = hist + (long long)sj.hist * nbins;
        for (int k = threadIdx.x; k < nbins; k += blockDim.x) {
            const int r = k / kNphi, col = k - r * kNphi;
            const unsigned v = sh[r * 2 * kNphi + col] + sh[r * 2 * kNphi + col + kNphi];
            if (v) atomicAdd(h + k, (unsigned long long)v);
        }
        __syncthreads();
    }
    for (int o = 16; o > 0; o >>= 1) slow += __shfl_xor_sync(0xffffffffu, slow, o);
    if ((threadIdx.x & 31) == 0 && slow) atomicAdd(n_slow, (unsigned long long)slow);
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

}  // namespace

struct hbt_bf_ctx {
    hbt_bf_params p;
    int device = 0;
    cudaStream_t stream = nullptr;
    BfConst c;
    Buf hist, jobs, items, phi, y, tb, yb, counter;
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
    hbt_bf_stats stats{};
    std::string err;
};

namespace {

hbt_status bf_fail(hbt_bf_ctx *c, hbt_status s, const std::string &m) {
    if (c) c->err = m;
    return s;
}

}  // namespace

extern "C" {

hbt_status hbt_bf_create(const hbt_bf_params *p, int device, hbt_bf_ctx **out) {
    if (!p || !out) return HBT_ERR_INVALID;
    *out = nullptr;
    // the shared-memory histogram holds Bnpts x 40 counts (at most 96 KB)
    if (p->Bnpts < 2 || p->Bnpts * kNphi * 4 > 48 * 1024) return HBT_ERR_INVALID;
    hbt_bf_ctx *c = new hbt_bf_ctx();
    c->p = *p;
    c->device = device;
    // the reference's expressions (src/BalanceFunction.cpp:29-35)
    c->c.drap = 2. * std::abs(p->Brap_max) / (p->Bnpts - 1);
    c->c.Brap_min = -std::abs(p->Brap_max) - 0.5 * c->c.drap;
    c->c.dphi = 2. * M_PI / kNphi;
    c->c.Bphi_min = -M_PI / 2.;
    c->c.Bnpts = p->Bnpts;
    c->c.inv_drap = 1.0 / c->c.drap;
    c->c.inv_dphi = 1.0 / c->c.dphi;
    if (cudaSetDevice(device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&c->ev[0]) != cudaSuccess || cudaEventCreate(&c->ev[1]) != cudaSuccess ||
        cudaEventCreate(&c->ev[2]) != cudaSuccess ||
        !grow(c->hist, (size_t)8 * p->Bnpts * kNphi * sizeof(unsigned long long)) ||
        !grow(c->counter, sizeof(unsigned long long)) ||
        cudaFuncSetAttribute(k_bf, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             p->Bnpts * 2 * kNphi * (int)sizeof(unsigned)) != cudaSuccess) {
        hbt_bf_destroy(c);
        return HBT_ERR_CUDA;
    }
    const hbt_status s = hbt_bf_reset(c);
    if (s != HBT_OK) {
        hbt_bf_destroy(c);
        return s;
    }
    *out = c;
    return HBT_OK;
}

void hbt_bf_destroy(hbt_bf_ctx *c) {
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (Buf *b : {&c->hist, &c->jobs, &c->items, &c->phi, &c->y, &c->tb, &c->yb, &c->counter})
        if (b->p) cudaFree(b->p);
    for (cudaEvent_t e : c->ev)
        if (e) cudaEventDestroy(e);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

const char *hbt_bf_last_error(const hbt_bf_ctx *c) { return c ? c->err.c_str() : "null context"; }

hbt_status hbt_bf_reset(hbt_bf_ctx *c) {
    if (!c) return HBT_ERR_INVALID;
    if (cudaSetDevice(c->device) != cudaSuccess ||
        cudaMemsetAsync(c->hist.p, 0, (size_t)8 * c->p.Bnpts * kNphi * 8, c->stream) != cudaSuccess ||
        cudaStreamSynchronize(c->stream) != cudaSuccess)
        return bf_fail(c, HBT_ERR_CUDA, "clearing the histograms failed");
    return HBT_OK;
}

hbt_status hbt_bf_bin(hbt_bf_ctx *c, int32_t n_lists, const hbt_bf_list *lists, int32_t n_jobs,
                      const hbt_bf_job *jobs) {
    if (!c || n_lists < 0 || n_jobs < 0 || (n_lists > 0 && !lists) || (n_jobs > 0 && !jobs))
        return HBT_ERR_INVALID;
    if (n_jobs == 0) return HBT_OK;
    if (cudaSetDevice(c->device) != cudaSuccess) return bf_fail(c, HBT_ERR_CUDA, "cudaSetDevice");
    // concatenate the lists (a list passed again with the same arrays, as the
    // mixed-event pool is when it is the buffer itself, shares the first
    // copy), resolve every job's particle ranges
    std::vector<long long> base(n_lists, 0);
    std::vector<int> copy_of(n_lists, -1);
    std::map<std::tuple<const void *, const void *, const void *, int32_t>, int> first;
    long long total = 0;
    for (int l = 0; l < n_lists; l++) {
        const hbt_bf_list &L = lists[l];
        if (L.n_events < 0 || (L.n_events > 0 && !L.offsets))
            return bf_fail(c, HBT_ERR_INVALID, "list without offsets");
        const long long n = L.n_events > 0 ? L.offsets[L.n_events] : 0;
        if (n > 0 && (!L.phi || !L.y)) return bf_fail(c, HBT_ERR_INVALID, "list without columns");
        const auto key = std::make_tuple(static_cast<const void *>(L.offsets),
                                         static_cast<const void *>(L.phi),
                                         static_cast<const void *>(L.y), L.n_events);
        const auto seen = first.emplace(key, l);
        if (!seen.second) copy_of[l] = seen.first->second;
        if (copy_of[l] >= 0) {
            base[l] = base[copy_of[l]];
        } else {
            base[l] = total;
            total += n;
        }
    }
    long long pairs = 0;
    std::vector<BfJob> dj(n_jobs);
    for (int k = 0; k < n_jobs; k++) {
        const hbt_bf_job &J = jobs[k];
        if (J.hist < 0 || J.hist > 7 || J.la < 0 || J.la >= n_lists || J.lb < 0 ||
            J.lb >= n_lists || J.ea < 0 || J.ea >= lists[J.la].n_events || J.eb < 0 ||
            J.eb >= lists[J.lb].n_events)
            return bf_fail(c, HBT_ERR_INVALID, "job out of range");
        const int64_t *oa = lists[J.la].offsets, *ob = lists[J.lb].offsets;
        dj[k] = BfJob{base[J.la] + oa[J.ea], base[J.la] + oa[J.ea + 1], base[J.lb] + ob[J.eb],
                      base[J.lb] + ob[J.eb + 1], J.rotation, J.hist, J.mixed ? 1 : 0};
        pairs += (oa[J.ea + 1] - oa[J.ea]) * (ob[J.eb + 1] - ob[J.eb]);
    }
    std::vector<int2> items;
    for (int k = 0; k < n_jobs; k++)
        if (dj[k].b1 > dj[k].b0)
            for (long long a = 0; a < dj[k].a1 - dj[k].a0; a += kTile)
                items.push_back(make_int2(k, (int)a));
    if (items.empty()) {
        c->stats = hbt_bf_stats{};
        return HBT_OK;
    }
    if (!grow(c->jobs, dj.size() * sizeof(BfJob)) || !grow(c->items, items.size() * sizeof(int2)) ||
        !grow(c->phi, total * sizeof(double)) || !grow(c->y, total * sizeof(double)) ||
        !grow(c->tb, total * sizeof(float4)) || !grow(c->yb, total * sizeof(float2)))
        return bf_fail(c, HBT_ERR_NOMEM, "device allocation failed");
    cudaError_t e = cudaEventRecord(c->ev[0], c->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(c->jobs.p, dj.data(), dj.size() * sizeof(BfJob),
                            cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(c->items.p, items.data(), items.size() * sizeof(int2),
                            cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(c->counter.p, 0, sizeof(unsigned long long), c->stream);
    for (int l = 0; l < n_lists && e == cudaSuccess; l++) {
        const long long n = lists[l].n_events > 0 ? lists[l].offsets[lists[l].n_events] : 0;
        if (n == 0 || copy_of[l] >= 0) continue;
        e = cudaMemcpyAsync(static_cast<double *>(c->phi.p) + base[l], lists[l].phi,
                            n * sizeof(double), cudaMemcpyHostToDevice, c->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(static_cast<double *>(c->y.p) + base[l], lists[l].y,
                                n * sizeof(double), cudaMemcpyHostToDevice, c->stream);
    }
    if (e == cudaSuccess) e = cudaEventRecord(c->ev[1], c->stream);
    if (e != cudaSuccess) return bf_fail(c, HBT_ERR_CUDA, "upload failed");
    const double *dphi_p = static_cast<const double *>(c->phi.p);
    const double *dy_p = static_cast<const double *>(c->y.p);
    if (total > 0)
        k_bf_terms<<<(unsigned)std::min<long long>((total + 255) / 256, 152LL * 16), 256, 0,
                     c->stream>>>(total, dphi_p, dy_p, c->c, static_cast<float4 *>(c->tb.p),
                                  static_cast<float2 *>(c->yb.p));
    const long long n_items = (long long)items.size();
    const long long grid = std::min<long long>(n_items, 1LL << 30);
    k_bf<<<(unsigned)grid, kTile, (size_t)c->p.Bnpts * 2 * kNphi * sizeof(unsigned), c->stream>>>(
        static_cast<const BfJob *>(c->jobs.p), static_cast<const int2 *>(c->items.p), n_items,
        dphi_p, dy_p, static_cast<const float4 *>(c->tb.p), static_cast<const float2 *>(c->yb.p),
        c->c, static_cast<unsigned long long *>(c->hist.p),
        static_cast<unsigned long long *>(c->counter.p));
    if ((e = cudaGetLastError()) != cudaSuccess)
        return bf_fail(c, HBT_ERR_CUDA, std::string("k_bf: ") + cudaGetErrorString(e));
    unsigned long long slow = 0;
    if ((e = cudaEventRecord(c->ev[2], c->stream)) != cudaSuccess ||
        (e = cudaMemcpyAsync(&slow, c->counter.p, sizeof slow, cudaMemcpyDeviceToHost,
                             c->stream)) != cudaSuccess)
        return bf_fail(c, HBT_ERR_CUDA, cudaGetErrorString(e));
    // the host arrays may be reused once the copies are done
    if ((e = cudaStreamSynchronize(c->stream)) != cudaSuccess)
        return bf_fail(c, HBT_ERR_CUDA, cudaGetErrorString(e));
    float up = 0.f, ker = 0.f;
    cudaEventElapsedTime(&up, c->ev[0], c->ev[1]);
    cudaEventElapsedTime(&ker, c->ev[1], c->ev[2]);
    c->stats.pairs = pairs;
    c->stats.bytes_uploaded = (int64_t)(dj.size() * sizeof(BfJob) + items.size() * sizeof(int2) +
                                        2 * total * sizeof(double));
    c->stats.fp64_pairs = (int64_t)slow;
    c->stats.upload_ms = up;
    c->stats.kernel_ms = ker;
    return HBT_OK;
}

hbt_status hbt_bf_get_stats(const hbt_bf_ctx *c, hbt_bf_stats *out) {
    if (!c || !out) return HBT_ERR_INVALID;
    *out = c->stats;
    return HBT_OK;
}

hbt_status hbt_bf_read(hbt_bf_ctx *c, int32_t hist, double *out) {
    if (!c || hist < 0 || hist > 7 || !out) return HBT_ERR_INVALID;
    const size_t nb = (size_t)c->p.Bnpts * kNphi;
    std::vector<unsigned long long> v(nb);
    if (cudaSetDevice(c->device) != cudaSuccess ||
        cudaMemcpyAsync(v.data(), static_cast<unsigned long long *>(c->hist.p) + hist * nb,
                        nb * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                        c->stream) != cudaSuccess ||
        cudaStreamSynchronize(c->stream) != cudaSuccess)
        return bf_fail(c, HBT_ERR_CUDA, "reading the histogram failed");
    for (size_t k = 0; k < nb; k++) out[k] = (double)v[k];
    return HBT_OK;
}

}  // extern "C"
