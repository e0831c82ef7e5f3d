// hbt_bin_mixed_rotated_noalloc: mixed-event binning that allocates no memory.
//
// Some callers cannot call cudaMalloc: a host framework that owns the whole
// device memory budget through its own pool (a cudaMalloc from a library
// would fail or fragment that pool), or a time-critical loop that must not
// pay for an allocation's implicit device synchronisation.  They already hold
// their particle arrays and histogram in device memory and need only the
// binning.  This entry point serves them: the caller passes every input and
// the output; the one piece of scratch the operation needs - the partner
// list after its random rotation - lives in a file-scope __device__ array of
// fixed size instead of being allocated.
//
// Behaviour and limits
//  - Rotates the partner pool (px, py) by (cos_phi, sin_phi) exactly as the
//    reference rotates a mixed event (src/HBT_correlation.cpp:522-523, no
//    fused multiply-add) into the scratch array, then bins list1 x rotated
//    pool into `den` with the screened mixed-event kernel.  Counts are
//    identical to hbt_bin_mixed_dev on the same rotated list.
//  - At most HBT_NOALLOC_MAX_POOL pool particles per call; larger pools are
//    rejected with HBT_ERR_INVALID and a message.
//  - azimuthal_flag and invariant_radius_flag must be 0, and no
//    needed_number_of_pairs cap is applied (every surviving pair is counted).
//  - The scratch array is held by every GPU that loads the library until the
//    process exits.  All calls share it and it keeps the last call's
//    contents; the counter words are cleared at the start of each call.
//    Calls that overlap on the GPU (different streams, or different host
//    threads on the same device) race on it; order them on one stream.
//  - The first call on a device looks up the array's device address
//    (cudaGetSymbolAddress) with that device current; make that first call
//    before any stream capture.
#include <cmath>
#include <cstdio>
#include <mutex>

#include "../../include/hbt_gpu.h"
#include "hbt_engine.cuh"

namespace hbt {
namespace {

constexpr long long kPool = HBT_NOALLOC_MAX_POOL;
// rotated px, py, pz, E (kPool doubles each) followed by the stats words
constexpr size_t kScratchBytes = (size_t)4 * kPool * sizeof(double) + STAT_N * sizeof(u64);

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// Device address of the scratch array, per device (looked up once).
constexpr int kMaxDevices = 64;
unsigned char *g_scratch_addr[kMaxDevices] = {nullptr};
std::mutex g_scratch_mutex;

__global__ void k_rotate(long long n, const double *px, const double *py, const double *pz,
                         const double *E, double cph, double sph, double *out) {
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const double x = px[k], y = py[k];
    out[k] = x * cph - y * sph;               // compiled with --fmad=false
    out[kPool + k] = x * sph + y * cph;
    out[2 * kPool + k] = pz[k];
    out[3 * kPool + k] = E[k];
}

int fail(char *errbuf, size_t errlen, int status, const char *msg) {
    if (errbuf && errlen > 0) snprintf(errbuf, errlen, "%s", msg);
    return status;
}

}  // namespace
}  // namespace hbt

extern "C" hbt_status hbt_bin_mixed_rotated_noalloc(const hbt_params *p, int64_t n1,
                                                    const hbt_soa4 *list1, int64_t n2,
                                                    const hbt_soa4 *pool, double cos_phi,
                                                    double sin_phi, uint64_t *den,
                                                    void *stream, char *errbuf, size_t errlen) {
    using namespace hbt;
    if (errbuf && errlen > 0) errbuf[0] = '\0';
    if (!p || !list1 || !pool || !den || n1 < 0 || n2 < 0)
        return (hbt_status)fail(errbuf, errlen, HBT_ERR_INVALID, "null argument or negative size");
    if (n2 > kPool) {
        char msg[160];
        snprintf(msg, sizeof(msg),
                 "pool of %lld particles exceeds HBT_NOALLOC_MAX_POOL = %lld",
                 (long long)n2, kPool);
        return (hbt_status)fail(errbuf, errlen, HBT_ERR_INVALID, msg);
    }
    if (p->azimuthal_flag != 0 || p->invariant_radius_flag != 0)
        return (hbt_status)fail(errbuf, errlen, HBT_ERR_INVALID,
                                "azimuthal_flag and invariant_radius_flag must be 0");
    if (p->qnpts < 2 || p->qnpts > 1024 || p->n_KT < 2 || p->n_KT > 255)
        return (hbt_status)fail(errbuf, errlen, HBT_ERR_INVALID, "qnpts or n_KT out of range");
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
        return (hbt_status)fail(errbuf, errlen, HBT_ERR_CUDA, "cudaGetDevice failed");
    unsigned char *scratch = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_scratch_mutex);
        if (!g_scratch_addr[dev]) {
            void *addr = nullptr;
            const cudaError_t e = cudaGetSymbolAddress(&addr, g_noalloc_scratch);
            if (e != cudaSuccess)
                return (hbt_status)fail(errbuf, errlen, HBT_ERR_CUDA,
                                        "cudaGetSymbolAddress of the scratch array failed");
            g_scratch_addr[dev] = static_cast<unsigned char *>(addr);
        }
        scratch = g_scratch_addr[dev];
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    double *rot = reinterpret_cast<double *>(scratch);
    u64 *stats = reinterpret_cast<u64 *>(scratch + (size_t)4 * kPool * sizeof(double));
    if (cudaMemsetAsync(stats, 0, STAT_N * sizeof(u64), st) != cudaSuccess)
        return (hbt_status)fail(errbuf, errlen, HBT_ERR_CUDA, "clearing the scratch counters failed");
    if (n1 == 0 || n2 == 0) return HBT_OK;

    // constants with the reference's expressions (src/HBT_correlation.cpp:25-61)
    Device d = {};
    Grid &g = d.g;
    g.qnpts = p->qnpts;
    g.n_KT = p->n_KT;
    g.n_Kphi = p->n_Kphi > 0 ? p->n_Kphi : 1;
    g.n_slots = p->n_KT;
    g.azimuthal = 0;
    g.qinv = 0;
    g.boost = p->long_comoving_boost == 1;
    g.q3 = (long long)p->qnpts * p->qnpts * p->qnpts;
    g.delta_q = (p->q_max - p->q_min) / (p->qnpts - 1);
    g.q_lo = p->q_min - g.delta_q / 2. + 1e-8;
    g.q_hi = p->q_max + g.delta_q / 2. - 1e-8;
    g.q_base = p->q_min - g.delta_q / 2.;
    g.KT_min = p->KT_min;
    g.dKT = (p->KT_max - p->KT_min) / (p->n_KT - 1);
    g.KT_min_sq = p->KT_min * p->KT_min;
    g.KT_max_sq = p->KT_max * p->KT_max;
    g.dKphi = 2 * M_PI / g.n_Kphi;
    g.two_pi = 2. * M_PI;
    g.hbarC_inv = 1. / 0.197327053;
    // FP32 screen constants and the bounds on their rounding
    Screen &s = d.s;
    auto f = [](double v) { return static_cast<float>(v); };
    auto slack = [](double v, float v32) { return std::fabs(v - static_cast<double>(v32)); };
    const double lo4 = 4.0 * g.KT_min_sq, hi4 = 4.0 * g.KT_max_sq;
    s.kt_lo4 = f(lo4);
    s.kt_hi4 = f(hi4);
    s.kt_slack = f(std::fmax(slack(lo4, s.kt_lo4), slack(hi4, s.kt_hi4)) + 1e-7 * hi4);
    s.lo = f(g.q_lo);
    s.hi = f(g.q_hi);
    s.win_slack = f(std::fmax(slack(g.q_lo, s.lo), slack(g.q_hi, s.hi)) + 1e-12);
    s.base = f(g.q_base);
    s.inv_dq = f(1.0 / g.delta_q);
    s.t_slack = f(slack(g.q_base, s.base) / g.delta_q + 4.0 * 5.96e-8 * g.qnpts + 1e-9);
    s.KT_min = f(g.KT_min);
    s.inv_dKT = f(1.0 / g.dKT);
    s.kt_t_slack = f(slack(g.KT_min, s.KT_min) / g.dKT + 4.0 * 5.96e-8 * g.n_KT + 1e-9);
    s.two_pi = f(g.two_pi);
    s.inv_dKphi = f(1.0 / g.dKphi);
    s.qnpts = g.qnpts;
    s.n_KT = g.n_KT;
    s.n_Kphi = g.n_Kphi;
    fill_prefilter(s);
    d.h.den = reinterpret_cast<u64 *>(den);
    d.stats = stats;

    k_rotate<<<(unsigned)((n2 + 255) / 256), 256, 0, st>>>(n2, pool->px, pool->py, pool->pz,
                                                         pool->E, cos_phi, sin_phi, rot);
    if (cudaGetLastError() != cudaSuccess)
        return (hbt_status)fail(errbuf, errlen, HBT_ERR_CUDA, "rotation kernel launch failed");
    const double *l1[4] = {list1->px, list1->py, list1->pz, list1->E};
    const double *l2[4] = {rot, rot + kPool, rot + 2 * kPool, rot + 3 * kPool};
    if (launch_mixed_fast(d, n1, l1, n2, l2, st) != cudaSuccess)
        return (hbt_status)fail(errbuf, errlen, HBT_ERR_CUDA, "binning kernel launch failed");
    return HBT_OK;
}
