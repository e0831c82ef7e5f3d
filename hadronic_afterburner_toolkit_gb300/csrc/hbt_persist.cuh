// Persistent pair-binning kernels of the batched path: CTAs pull
// (job, i-tile, j-tile) items from the culled queues that hbt_batch.cu
// builds and run the screened tile-pair bodies of hbt_tile.cuh on them.
// The kernel templates are instantiated in three translation units,
// compiled in parallel: hbt_persist_fast.cu (fast binning),
// hbt_persist_caps.cu (the two passes of ordered cap admission) and
// hbt_persist_qinv.cu (fast binning with the q_inv histograms).
#pragma once

#include "hbt_batch.cuh"
#include "hbt_tile.cuh"

namespace hbt {

// Launchers, one family per translation unit (same-event items
// [base, end) of the queue; mixed-event items all at once).
cudaError_t persistent_same_fast(const Device &d, const BatchDev &b, unsigned base, unsigned end,
                                 int grid, cudaStream_t st);
cudaError_t persistent_mixed_fast(const Device &d, const BatchDev &b, int grid, cudaStream_t st);
cudaError_t persistent_same_ordered(const Device &d, const BatchDev &b, unsigned base,
                                    unsigned end, int grid, cudaStream_t st, int mode);
cudaError_t persistent_mixed_ordered(const Device &d, const BatchDev &b, int grid,
                                     cudaStream_t st, int mode);
cudaError_t persistent_same_qinv(const Device &d, const BatchDev &b, unsigned base, unsigned end,
                                 int grid, cudaStream_t st);
cudaError_t persistent_mixed_qinv(const Device &d, const BatchDev &b, int grid, cudaStream_t st);
// Dispatch on the admission mode and the q_inv histograms.
cudaError_t persistent_same(const Device &d, const BatchDev &b, unsigned base, unsigned end,
                            int grid, cudaStream_t st, int mode);
cudaError_t persistent_mixed(const Device &d, const BatchDev &b, int grid, cudaStream_t st,
                             int mode);

namespace persist {

using namespace tile;

// Serving many analyses in one launch (MANY): the job's engine descriptor,
// its entry of b.devs, copied into shared memory.  A launch of one analysis
// reads the descriptor from its kernel parameter instead: its fields are
// then constant-bank operands, where a reference that may point to either
// the parameter or shared memory made every field a generic load (the
// same-event kernel took 141 ms per central group that way, 121 ms
// without).
__device__ __forceinline__ void load_device(const BatchDev &b, const BatchJob &job, Device &dsm) {
    const int *src = reinterpret_cast<const int *>(b.devs + job.dev);
    int *dst = reinterpret_cast<int *>(&dsm);
    for (int k = threadIdx.x; k < (int)(sizeof(Device) / sizeof(int)); k += blockDim.x)
        dst[k] = src[k];
    __syncthreads();
}

// Resident CTAs per SM (register budget 65536 / (128 x CTAs); shared
// memory allows 5 of the FP64 and double-float forms' 38.4 KB): measured on
// GB300, the FP64 form of the same-event kernel is fastest at 5 (96
// registers, no spills: 141.0 ms kernel per central group against 144.6 ms
// at 4 with 124 registers; at 3, 164 registers, it took 173.6 ms), the
// double-float form at 5 too (96 registers: 119.8 ms kernel against 123.1
// ms at 4 with 128, with the descriptor read from the kernel parameter), the
// FP32-weight form at 6 (80 registers: 94.0 ms, against 97.4 ms at 5 and,
// before the descriptor change, 127.8 ms at 7 with 72) and the mixed-event
// kernel at 6 (12.6 ms, against 13.0 ms at 5 and 18.3 ms at 7).
#ifndef HBT_FP64_SAME_CTAS
#define HBT_FP64_SAME_CTAS 5  // compile-time choice for the FP64 form (-D to measure others)
#endif
#ifndef HBT_DF64_SAME_CTAS
#define HBT_DF64_SAME_CTAS 5  // the same for the double-float form
#endif
#ifndef HBT_FP32W_SAME_CTAS
#define HBT_FP32W_SAME_CTAS 6  // and for the FP32-weight form
#endif
template <int PREC>
struct SameCtas {
    static constexpr int value =
        PREC == 1 ? HBT_FP32W_SAME_CTAS : (PREC == 2 ? HBT_DF64_SAME_CTAS : HBT_FP64_SAME_CTAS);
};
#ifndef HBT_MIXED_CTAS
#define HBT_MIXED_CTAS 6  // the mixed-event kernel's
#endif
constexpr int kMixedCtas = HBT_MIXED_CTAS;

// Same-event items [base, min(end, queued)) pulled by persistent CTAs.
// MODE: fast binning, or one pass of ordered cap admission; MANY: the items
// of many analyses (b.devs), fast binning only.
template <bool AZ, bool BOOST, int PREC, int MODE, bool QINV, bool MANY>
__global__ void __launch_bounds__(FT, SameCtas<PREC>::value) k_persistent_same(Device d, BatchDev b, unsigned base,
                                                           unsigned end) {
    __shared__ SmemFor<QINV> sm;
    __shared__ unsigned item;
    __shared__ double2 cs[COS_TABLE];
    if (PREC == 0) fill_cos_table(cs);
    if (PREC == 2) fill_df_table(reinterpret_cast<float4 *>(cs));
    const unsigned stop = min(end, min(b.n_items[0], b.same_cap));
    for (;;) {
        if (threadIdx.x == 0) item = base + atomicAdd(b.item_next, 1u);
        __syncthreads();
        const unsigned k = item;
        if (k >= stop) break;
        const Item it = b.items[b.order_items ? b.item_pos_out[k] : k];
        const BatchJob &job = b.jobs[it.job];
        const BatchList &la = b.lists[job.la];
        const double *c[8];
#pragma unroll
        for (int f = 0; f < 8; f++) c[f] = b.table + (long long)f * b.cap + la.off;
        if constexpr (MANY) {
            __shared__ Device dsm;
            load_device(b, job, dsm);
            same_tile_pair<AZ, BOOST, PREC, MODE, QINV>(dsm, sm, cs, c, b.orig + la.off, la.n,
                                                        (long long)it.ti * FT,
                                                        (long long)it.tj * FT);
        } else {
            same_tile_pair<AZ, BOOST, PREC, MODE, QINV>(d, sm, cs, c, b.orig + la.off, la.n,
                                                        (long long)it.ti * FT,
                                                        (long long)it.tj * FT);
        }
        __syncthreads();
    }
}

// Mixed-event items, all in one launch.
template <bool AZ, bool BOOST, int MODE, bool QINV, bool MANY>
__global__ void __launch_bounds__(FT, kMixedCtas) k_persistent_mixed(Device d, BatchDev b) {
    __shared__ TileSmem sm;
    __shared__ unsigned item;
    const unsigned stop = min(b.n_items[1], b.mixed_cap);
    for (;;) {
        if (threadIdx.x == 0) item = atomicAdd(b.item_next + 1, 1u);
        __syncthreads();
        const unsigned k = item;
        if (k >= stop) break;
        const Item it = b.items[b.same_cap + k];
        const BatchJob &job = b.jobs[it.job];
        const BatchList &la = b.lists[job.la], &lb = b.lists[job.lb];
        const double *c1[4], *c2[4];
#pragma unroll
        for (int f = 0; f < 4; f++) {
            c1[f] = b.table + (long long)f * b.cap + la.off;
            c2[f] = b.table + (long long)f * b.cap + lb.off;
        }
        if constexpr (MANY) {
            __shared__ Device dsm;
            load_device(b, job, dsm);
            mixed_tile_pair<AZ, BOOST, MODE, QINV>(dsm, sm, c1, la.n, c2, lb.n,
                                                   (long long)it.ti * FT, (long long)it.tj * FT,
                                                   b.orig + la.off, b.orig + lb.off,
                                                   job.row_base);
        } else {
            mixed_tile_pair<AZ, BOOST, MODE, QINV>(d, sm, c1, la.n, c2, lb.n,
                                                   (long long)it.ti * FT, (long long)it.tj * FT,
                                                   b.orig + la.off, b.orig + lb.off,
                                                   job.row_base);
        }
        __syncthreads();
    }
}

inline int sm_count() {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
            sms = 152;
    }
    return sms;
}

// grid > 0: that many CTAs; otherwise one CTA per resident slot.
template <class K>
int persistent_grid(K kernel, int grid) {
    if (grid > 0) return grid;
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, FT, 0) != cudaSuccess || nb < 1)
        nb = 4;
    return sm_count() * nb;
}

// The kernel for one analysis, or (b.devs, fast binning only) for many.
template <bool AZ, bool BOOST, int PREC, int MODE, bool QINV>
cudaError_t launch_same_items(const Device &d, const BatchDev &b, unsigned base, unsigned end,
                              int grid, cudaStream_t st) {
    if (b.devs) {
        if constexpr (MODE == MODE_FAST) {
            grid = persistent_grid(k_persistent_same<AZ, BOOST, PREC, MODE, QINV, true>, grid);
            k_persistent_same<AZ, BOOST, PREC, MODE, QINV, true><<<grid, FT, 0, st>>>(d, b, base,
                                                                                     end);
            return cudaGetLastError();
        }
        return cudaErrorNotSupported;
    }
    grid = persistent_grid(k_persistent_same<AZ, BOOST, PREC, MODE, QINV, false>, grid);
    k_persistent_same<AZ, BOOST, PREC, MODE, QINV, false><<<grid, FT, 0, st>>>(d, b, base, end);
    return cudaGetLastError();
}

template <bool AZ, bool BOOST, int MODE, bool QINV>
cudaError_t launch_mixed_items(const Device &d, const BatchDev &b, int grid, cudaStream_t st) {
    if (b.devs) {
        if constexpr (MODE == MODE_FAST) {
            grid = persistent_grid(k_persistent_mixed<AZ, BOOST, MODE, QINV, true>, grid);
            k_persistent_mixed<AZ, BOOST, MODE, QINV, true><<<grid, FT, 0, st>>>(d, b);
            return cudaGetLastError();
        }
        return cudaErrorNotSupported;
    }
    grid = persistent_grid(k_persistent_mixed<AZ, BOOST, MODE, QINV, false>, grid);
    k_persistent_mixed<AZ, BOOST, MODE, QINV, false><<<grid, FT, 0, st>>>(d, b);
    return cudaGetLastError();
}

// The same-event kernel of the context's flags and precision form for one
// admission mode.  The COUNT pass only counts decided pairs per row, the
// same in every form, so it runs the FP64 form's kernel.
template <int MODE, bool QINV>
cudaError_t launch_same_mode(const Device &d, const BatchDev &b, unsigned base, unsigned end,
                             int grid, cudaStream_t st) {
    const bool az = d.g.azimuthal, boost = d.g.boost;
    // the forms this mode instantiates: FP64 only for COUNT
    constexpr int P1 = MODE == MODE_COUNT ? 0 : 1, P2 = MODE == MODE_COUNT ? 0 : 2;
    const int prec = MODE == MODE_COUNT ? 0 : d.precision;
#define HBT_P(AZ_, BO_, PR_) \
    return launch_same_items<AZ_, BO_, PR_, MODE, QINV>(d, b, base, end, grid, st)
    if (prec == 0) {
        if (az && boost) HBT_P(true, true, 0);
        if (az) HBT_P(true, false, 0);
        if (boost) HBT_P(false, true, 0);
        HBT_P(false, false, 0);
    }
    if (prec == 1) {
        if (az && boost) HBT_P(true, true, P1);
        if (az) HBT_P(true, false, P1);
        if (boost) HBT_P(false, true, P1);
        HBT_P(false, false, P1);
    }
    if (az && boost) HBT_P(true, true, P2);
    if (az) HBT_P(true, false, P2);
    if (boost) HBT_P(false, true, P2);
    HBT_P(false, false, P2);
#undef HBT_P
}

template <int MODE, bool QINV>
cudaError_t launch_mixed_mode(const Device &d, const BatchDev &b, int grid, cudaStream_t st) {
    const bool az = d.g.azimuthal, boost = d.g.boost;
    if (az && boost) return launch_mixed_items<true, true, MODE, QINV>(d, b, grid, st);
    if (az) return launch_mixed_items<true, false, MODE, QINV>(d, b, grid, st);
    if (boost) return launch_mixed_items<false, true, MODE, QINV>(d, b, grid, st);
    return launch_mixed_items<false, false, MODE, QINV>(d, b, grid, st);
}

}  // namespace persist
}  // namespace hbt
