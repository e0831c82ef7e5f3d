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
//    before any stream capture.  The address is kept per device together
//    with the CUDA context it was looked up in, and looked up again when the
//    device's current context changes (after cudaDeviceReset, or when the
//    host framework tears down and re-creates the primary context).
//  - The pool must already carry the rapidity cut the reference applies to
//    partner particles before rotating them (src/HBT_correlation.cpp:
//    509-511); list1 likewise (:474-476).  Pairs the reference would index
//    out of bounds (an LCMS component NaN because K_perp == 0) are skipped
//    and not reported here; hbt_get_stats of a context counts them.
#include <cuda.h>

#include <cmath>
#include <cstdio>
#include <mutex>

#include "../../include/hbt_gpu.h"
#include "hbt_engine.cuh"
#include "hbt_internal.h"

namespace hbt {
namespace {

constexpr long long kPool = HBT_NOALLOC_MAX_POOL;
// rotated px, py, pz, E (kPool doubles each) followed by the stats words
constexpr size_t kScratchBytes = (size_t)4 * kPool * sizeof(double) + STAT_N * sizeof(u64);

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// Device address of the scratch array, per device, with the unique id of
// the CUDA context it was looked up in (0: unknown).
constexpr int kMaxDevices = 64;
unsigned char *g_scratch_addr[kMaxDevices] = {nullptr};
unsigned long long g_scratch_ctx[kMaxDevices] = {0};
std::mutex g_scratch_mutex;

// Unique id of the calling thread's current CUDA context (cuCtxGetId, which
// never repeats within a process, unlike a context handle), through the
// driver entry points the runtime hands out; 0 when it cannot be had, in
// which case the address is looked up on every call.
unsigned long long current_context_id() {
    typedef CUresult (*GetCurrent)(CUcontext *);
    typedef CUresult (*GetId)(CUcontext, unsigned long long *);
    static GetCurrent cur = nullptr;
    static GetId id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr, *q = nullptr;
        cudaDriverEntryPointQueryResult r1, r2;
        // the two entry points as CUDA 12.0 defined them (cuCtxGetId first
        // appeared there)
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault,
                                             &r1) == cudaSuccess &&
            r1 == cudaDriverEntryPointSuccess &&
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &q, 12000, cudaEnableDefault, &r2) ==
                cudaSuccess &&
            r2 == cudaDriverEntryPointSuccess) {
            cur = reinterpret_cast<GetCurrent>(p);
            id = reinterpret_cast<GetId>(q);
        } else {
            cudaGetLastError();
        }
    });
    CUcontext ctx = nullptr;
    unsigned long long v = 0;
    if (!cur || !id || cur(&ctx) != CUDA_SUCCESS || !ctx || id(ctx, &v) != CUDA_SUCCESS)
        return 0;
    return v;
}

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
    // an error left by earlier work on this thread is reported as such, not
    // as a failure of this call's launches
    const cudaError_t prior = cudaGetLastError();
    if (prior != cudaSuccess) {
        char msg[200];
        snprintf(msg, sizeof(msg), "a CUDA error from earlier work was pending: %s",
                 cudaGetErrorString(prior));
        return (hbt_status)fail(errbuf, errlen, HBT_ERR_CUDA, msg);
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
        return (hbt_status)fail(errbuf, errlen, HBT_ERR_CUDA, "cudaGetDevice failed");
    unsigned char *scratch = nullptr;
    {
        // once per device (and again if the device's context was re-created)
        const unsigned long long ctx = current_context_id();
        std::lock_guard<std::mutex> lock(g_scratch_mutex);
        if (!g_scratch_addr[dev] || ctx == 0 || ctx != g_scratch_ctx[dev]) {
            void *addr = nullptr;
            const cudaError_t e = cudaGetSymbolAddress(&addr, g_noalloc_scratch);
            if (e != cudaSuccess)
                return (hbt_status)fail(errbuf, errlen, HBT_ERR_CUDA,
                                        "cudaGetSymbolAddress of the scratch array failed");
            g_scratch_addr[dev] = static_cast<unsigned char *>(addr);
            g_scratch_ctx[dev] = ctx;
        }
        scratch = g_scratch_addr[dev];
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    double *rot = reinterpret_cast<double *>(scratch);
    u64 *stats = reinterpret_cast<u64 *>(scratch + (size_t)4 * kPool * sizeof(double));
    if (cudaMemsetAsync(stats, 0, STAT_N * sizeof(u64), st) != cudaSuccess)
        return (hbt_status)fail(errbuf, errlen, HBT_ERR_CUDA, "clearing the scratch counters failed");
    if (n1 == 0 || n2 == 0) return HBT_OK;

    // the engine's constants and FP32 screen for these parameters, as
    // hbt_create derives them
    hbt_params prm = *p;
    if (prm.n_Kphi < 1) prm.n_Kphi = 1;  // unused without K_phi bins
    Device d = {};
    grid_from_params(prm, d.g);
    screen_from_grid(d.g, d.s);
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
