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
#include <string>
#include <vector>

#include "../../include/hbt_bf.h"

namespace {

constexpr int kTile = 128;
constexpr int kNphi = HBT_BF_NPHI;

// A job with its particle ranges resolved in the concatenated arrays.
struct BfJob {
    long long a0, a1, b0, b1;
    double rotation;
    int hist, mixed;
};

// The reference's binning constants (src/BalanceFunction.cpp:29-35) and
// their FP32 copies for the screen.
struct BfConst {
    double drap, Brap_min, dphi, Bphi_min;
    int Bnpts;
    float f_Brap_min, f_inv_drap, f_Bphi_min, f_inv_dphi;
};

constexpr float kU = 5.9604645e-8f;  // 2^-24

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

// The same decision from FP32 copies with rigorous error bounds (u =
// 2^-24 per rounding, every input rounded once from FP64, bounds widened by
// a factor for the FP32 constants and the reference's own FP64 rounding):
// the bin, -1 (skipped) or -2 (undecided: the caller runs bin64).
__device__ __forceinline__ int bin32(const BfConst &c, float pa, float ya, float pb, float yb,
                                     int mixed, float rot) {
    const float s1 = pa - pb;
    const float d = mixed ? s1 + rot : s1;
    const float ed = 3.0f * kU * (fabsf(d) + fabsf(pa) + fabsf(pb) + fabsf(rot));
    const float t = (d - c.f_Bphi_min) * c.f_inv_dphi;
    const float et = (ed + 3.0f * kU * (fabsf(d) + fabsf(c.f_Bphi_min))) * c.f_inv_dphi * 1.01f +
                     3.0f * kU * fabsf(t) + 1e-6f;
    const float kp = floorf(t), fp = t - kp;
    if (!(fp > et) || !(fp < 1.0f - et)) return -2;
    const float dy = ya - yb;
    const float ey = 3.0f * kU * (fabsf(ya) + fabsf(yb) + fabsf(dy)) + 1e-12f;
    const float ady = fabsf(dy);
    // 1e-10f rounds above 1e-10: both tests keep a relative margin
    if (ady + ey < 0.9999e-10f) return -1;  // |dy| < 1e-10 for certain
    if (!(ady - ey > 1.0001e-10f)) return -2;
    const float eb = ey + 3.0f * kU * fabsf(c.f_Brap_min);
    if (dy + eb < c.f_Brap_min) return -1;  // dy < Brap_min for certain
    if (!(dy - eb > c.f_Brap_min)) return -2;
    const float ty = (dy - c.f_Brap_min) * c.f_inv_drap;
    const float ety = (eb + 3.0f * kU * fabsf(dy - c.f_Brap_min)) * c.f_inv_drap * 1.01f +
                      3.0f * kU * fabsf(ty) + 1e-6f;
    const float ky = floorf(ty), fy = ty - ky;
    if (!(fy > ety) || !(fy < 1.0f - ety)) return -2;
    const int iy = (int)ky;
    if (iy < 0 || iy >= c.Bnpts) return -1;
    int ip = ((int)kp) % kNphi;
    if (ip < 0) ip += kNphi;
    return iy * kNphi + ip;
}

__global__ void __launch_bounds__(kTile) k_bf(const BfJob *jobs, long long n_jobs,
                                              const double *phi, const double *y, BfConst c,
                                              unsigned long long *hist) {
    extern __shared__ unsigned sh[];  // [Bnpts][kNphi]
    __shared__ double sphi[kTile], sy[kTile];
    __shared__ float fphi[kTile], fy[kTile];
    const int nbins = c.Bnpts * kNphi;
    for (long long job = blockIdx.x; job < n_jobs; job += gridDim.x) {
        for (int k = threadIdx.x; k < nbins; k += blockDim.x) sh[k] = 0u;
        __syncthreads();
        const BfJob J = jobs[job];
        const float frot = (float)J.rotation;
        for (long long a = J.a0; a < J.a1; a += kTile) {
            const long long ia = a + threadIdx.x;
            const bool have = ia < J.a1;
            const double pa = have ? phi[ia] : 0.0, ya = have ? y[ia] : 0.0;
            const float fpa = (float)pa, fya = (float)ya;
            for (long long b = J.b0; b < J.b1; b += kTile) {
                __syncthreads();
                if (b + threadIdx.x < J.b1) {
                    sphi[threadIdx.x] = phi[b + threadIdx.x];
                    sy[threadIdx.x] = y[b + threadIdx.x];
                    fphi[threadIdx.x] = (float)sphi[threadIdx.x];
                    fy[threadIdx.x] = (float)sy[threadIdx.x];
                }
                __syncthreads();
                const int nb = (int)min((long long)kTile, J.b1 - b);
                if (!have) continue;
                for (int j = 0; j < nb; j++) {
                    int k = bin32(c, fpa, fya, fphi[j], fy[j], J.mixed, frot);
                    if (k == -2) k = bin64(c, pa, ya, sphi[j], sy[j], J.mixed, J.rotation);
                    if (k >= 0) atomicAdd(&sh[k], 1u);
                }
            }
        }
        __syncthreads();
        unsigned long long *h = hist + (long long)J.hist * nbins;
        for (int k = threadIdx.x; k < nbins; k += blockDim.x)
            if (sh[k]) atomicAdd(h + k, (unsigned long long)sh[k]);
        __syncthreads();
    }
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
    Buf hist, jobs, phi, y;
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
    // the shared-memory histogram holds Bnpts x 20 counts (48 KB default)
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
    c->c.f_Brap_min = (float)c->c.Brap_min;
    c->c.f_inv_drap = (float)(1.0 / c->c.drap);
    c->c.f_Bphi_min = (float)c->c.Bphi_min;
    c->c.f_inv_dphi = (float)(1.0 / c->c.dphi);
    if (cudaSetDevice(device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
        !grow(c->hist, (size_t)8 * p->Bnpts * kNphi * sizeof(unsigned long long))) {
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
    for (Buf *b : {&c->hist, &c->jobs, &c->phi, &c->y})
        if (b->p) cudaFree(b->p);
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
    // concatenate the lists, resolve every job's particle ranges
    std::vector<long long> base(n_lists + 1, 0);
    for (int l = 0; l < n_lists; l++) {
        const hbt_bf_list &L = lists[l];
        if (L.n_events < 0 || (L.n_events > 0 && !L.offsets))
            return bf_fail(c, HBT_ERR_INVALID, "list without offsets");
        const long long n = L.n_events > 0 ? L.offsets[L.n_events] : 0;
        if (n > 0 && (!L.phi || !L.y)) return bf_fail(c, HBT_ERR_INVALID, "list without columns");
        base[l + 1] = base[l] + n;
    }
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
    }
    const long long total = base[n_lists];
    if (!grow(c->jobs, dj.size() * sizeof(BfJob)) || !grow(c->phi, total * sizeof(double)) ||
        !grow(c->y, total * sizeof(double)))
        return bf_fail(c, HBT_ERR_NOMEM, "device allocation failed");
    cudaError_t e = cudaMemcpyAsync(c->jobs.p, dj.data(), dj.size() * sizeof(BfJob),
                                    cudaMemcpyHostToDevice, c->stream);
    for (int l = 0; l < n_lists && e == cudaSuccess; l++) {
        const long long n = base[l + 1] - base[l];
        if (n == 0) continue;
        e = cudaMemcpyAsync(static_cast<double *>(c->phi.p) + base[l], lists[l].phi,
                            n * sizeof(double), cudaMemcpyHostToDevice, c->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(static_cast<double *>(c->y.p) + base[l], lists[l].y,
                                n * sizeof(double), cudaMemcpyHostToDevice, c->stream);
    }
    if (e != cudaSuccess) return bf_fail(c, HBT_ERR_CUDA, "upload failed");
    const long long grid = std::min<long long>(n_jobs, 152LL * 32);
    k_bf<<<(unsigned)grid, kTile, (size_t)c->p.Bnpts * kNphi * sizeof(unsigned), c->stream>>>(
        static_cast<const BfJob *>(c->jobs.p), n_jobs, static_cast<const double *>(c->phi.p),
        static_cast<const double *>(c->y.p), c->c, static_cast<unsigned long long *>(c->hist.p));
    if ((e = cudaGetLastError()) != cudaSuccess)
        return bf_fail(c, HBT_ERR_CUDA, std::string("k_bf: ") + cudaGetErrorString(e));
    // the host arrays may be reused once the copies are done
    if ((e = cudaStreamSynchronize(c->stream)) != cudaSuccess)
        return bf_fail(c, HBT_ERR_CUDA, cudaGetErrorString(e));
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
