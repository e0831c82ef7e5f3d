// Batched, culled, persistent pair binning.
//
// A batch is a list of jobs: same-event jobs (all pairs i < j of one list)
// and mixed-event jobs (list 1 x list 2).  When no pair cap can bind, the
// order of the pairs does not matter, and the batch is run as:
//
//  1. k_keys + CUB radix sort + k_gather: every list is reordered by a
//     Morton key of (p_x, p_y, rapidity) cells into a sorted particle table,
//     so that 128-particle tiles are compact in momentum space;
//  2. k_boxes: per tile, the ranges of p_x, p_y, rapidity y and the
//     smallest m_T = sqrt(E^2 - p_z^2);
//  3. k_cull: every tile pair of every job is kept unless no pair in it can
//     pass the q windows.  The test is rigorous: the reference's q_out and
//     q_side satisfy q_out^2 + q_side^2 = q_x^2 + q_y^2, and both lie within
//     Q = max(|lo|, |hi|) of the window, so a pair needs |q_T|^2 <= 2 Q^2;
//     with the longitudinal boost
//       q_long = 2 m_T1 m_T2 sinh(y1 - y2) / sqrt(m_T1^2 + m_T2^2 +
//                2 m_T1 m_T2 cosh(y1 - y2)),
//     which grows with m_T1, m_T2 and |y1 - y2|, so its smallest value over
//     two tiles bounds |q_long| from below; without the boost q_long = q_z.
//     Each bound carries a 1e-6 relative margin for rounding;
//  4. k_persistent_same / k_persistent_mixed: persistent CTAs (5 per SM)
//     pull (job, i-tile, j-tile) items from the culled same-event and
//     mixed-event queues and run the screened tile-pair bodies of
//     hbt_tile.cuh.  The FP32-weight form runs the same-event queue in
//     chunks and merges the FP32 partials between them.
#include <cub/device/device_radix_sort.cuh>

#include "hbt_batch.cuh"
#include "hbt_tile.cuh"

namespace hbt {
namespace {

using namespace tile;

// Morton interleave of three 10-bit cell coordinates.
__device__ __forceinline__ unsigned spread10(unsigned v) {
    v &= 0x3ffu;
    v = (v | (v << 16)) & 0x030000ffu;
    v = (v | (v << 8)) & 0x0300f00fu;
    v = (v | (v << 4)) & 0x030c30c3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

__device__ __forceinline__ int find_range(const long long *off, int n, long long g) {
    // largest k with off[k] <= g (off is non-decreasing, off[0] == 0)
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (off[mid] <= g)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ unsigned cell(double v, double origin, double inv_h) {
    const double c = (v - origin) * inv_h;
    if (!(c > 0.0)) return 0u;
    if (c >= 1023.0) return 1023u;
    return (unsigned)c;
}

__global__ void k_keys(BatchDev b) {
    for (long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x; g < b.total;
         g += (long long)gridDim.x * blockDim.x) {
        const int L = find_range(b.list_off, b.n_lists, g);
        const BatchList &l = b.lists[L];
        const long long k = g - l.off;
        const double px = l.src[0][k], py = l.src[1][k], pz = l.src[2][k], E = l.src[3][k];
        const double y = 0.5 * log((E + pz) / (E - pz));
        const unsigned key = spread10(cell(px, -b.p_extent, b.inv_cell_pt)) |
                             (spread10(cell(py, -b.p_extent, b.inv_cell_pt)) << 1) |
                             (spread10(cell(y == y ? y : 0.0, -b.y_extent, b.inv_cell_y)) << 2);
        b.keys_in[g] = ((unsigned long long)L << 32) | key;
        b.vals_in[g] = (unsigned)g;
    }
}

__global__ void k_gather(BatchDev b) {
    for (long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x; s < b.total;
         s += (long long)gridDim.x * blockDim.x) {
        const int L = (int)(b.keys_out[s] >> 32);
        const BatchList &l = b.lists[L];
        const long long k = (long long)b.vals_out[s] - l.off;
        for (int f = 0; f < l.ncols; f++) b.table[(long long)f * b.cap + s] = l.src[f][k];
        b.orig[s] = (unsigned)k;  // position in the caller's list (pair orientation)
    }
}

// One warp per tile: momentum-space box of its particles.
__global__ void k_boxes(BatchDev b) {
    const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= b.total_tiles) return;
    const int L = find_range(b.tile_off, b.n_lists, warp);
    const BatchList &l = b.lists[L];
    const long long t = warp - l.tile_off;
    const long long s0 = l.off + t * FT, s1 = min(l.off + (t + 1) * FT, l.off + l.n);
    double x0 = 1e300, x1 = -1e300, y0 = 1e300, y1 = -1e300, Y0 = 1e300, Y1 = -1e300, m0 = 1e300;
    double z0 = 1e300, z1 = -1e300;
    for (long long s = s0 + lane; s < s1; s += 32) {
        const double px = b.table[s], py = b.table[b.cap + s];
        const double pz = b.table[2 * b.cap + s], E = b.table[3 * b.cap + s];
        const double y = 0.5 * log((E + pz) / (E - pz));
        const double m2 = (E - pz) * (E + pz);
        x0 = fmin(x0, px);
        x1 = fmax(x1, px);
        y0 = fmin(y0, py);
        y1 = fmax(y1, py);
        z0 = fmin(z0, pz);
        z1 = fmax(z1, pz);
        if (y == y) {
            Y0 = fmin(Y0, y);
            Y1 = fmax(Y1, y);
        } else {
            Y0 = -1e300;  // not a physical momentum: never cull on rapidity
            Y1 = 1e300;
        }
        m0 = fmin(m0, m2 > 0.0 ? sqrt(m2) : 0.0);
    }
    for (int o = 16; o > 0; o >>= 1) {
        x0 = fmin(x0, __shfl_xor_sync(0xffffffffu, x0, o));
        x1 = fmax(x1, __shfl_xor_sync(0xffffffffu, x1, o));
        y0 = fmin(y0, __shfl_xor_sync(0xffffffffu, y0, o));
        y1 = fmax(y1, __shfl_xor_sync(0xffffffffu, y1, o));
        Y0 = fmin(Y0, __shfl_xor_sync(0xffffffffu, Y0, o));
        Y1 = fmax(Y1, __shfl_xor_sync(0xffffffffu, Y1, o));
        m0 = fmin(m0, __shfl_xor_sync(0xffffffffu, m0, o));
        z0 = fmin(z0, __shfl_xor_sync(0xffffffffu, z0, o));
        z1 = fmax(z1, __shfl_xor_sync(0xffffffffu, z1, o));
    }
    if (lane == 0) b.boxes[warp] = Box{x0, x1, y0, y1, Y0, Y1, m0, z0, z1};
}

// Can a pair with one particle in box a and one in box b pass the windows?
__device__ __forceinline__ bool boxes_may_pair(const BatchJob &b, const Box &a, const Box &c) {
    const double gx = fmax(0.0, fmax(a.x0 - c.x1, c.x0 - a.x1));
    const double gy = fmax(0.0, fmax(a.y0 - c.y1, c.y0 - a.y1));
    if (gx * gx + gy * gy > b.qt2_max) return false;
    if (b.boost) {
        const double gY = fmax(0.0, fmax(a.Y0 - c.Y1, c.Y0 - a.Y1));
        if (gY > 0.0) {
            const double m1 = a.m0, m2 = c.m0;
            const double f = 2.0 * m1 * m2 * sinh(gY) /
                             sqrt(m1 * m1 + m2 * m2 + 2.0 * m1 * m2 * cosh(gY));
            if (f > b.ql_max) return false;
        }
    } else {
        // q_long = q_z
        const double gz = fmax(0.0, fmax(a.z0 - c.z1, c.z0 - a.z1));
        if (gz > b.ql_max) return false;
    }
    return true;
}

// Culled queues: same-event items at items[0, same_cap), mixed-event items
// at items[same_cap, same_cap + mixed_cap); n_items[0] / n_items[1] count them.
__global__ void k_cull(BatchDev b) {
    for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < b.total_pairs;
         p += (long long)gridDim.x * blockDim.x) {
        const int J = find_range(b.pair_off, b.n_jobs, p);
        const BatchJob &job = b.jobs[J];
        const long long k = p - job.pair_off;
        long long ti, tj;
        if (job.kind == 0) {
            tri_tile(k, ti, tj);
        } else {
            const long long ta = b.lists[job.la].tiles;
            ti = k % ta;
            tj = k / ta;
        }
        const Box &A = b.boxes[b.lists[job.la].tile_off + ti];
        const Box &B = b.boxes[b.lists[job.lb].tile_off + tj];
        if (boxes_may_pair(job, A, B)) {
            const Item it = Item{(unsigned)J, (unsigned)ti, (unsigned)tj};
            if (job.kind == 0) {
                const unsigned slot = atomicAdd(b.n_items, 1u);
                if (slot < b.same_cap) b.items[slot] = it;
            } else {
                const unsigned slot = atomicAdd(b.n_items + 1, 1u);
                if (slot < b.mixed_cap) b.items[b.same_cap + slot] = it;
            }
        }
    }
}

// Engine descriptor of an item: the launch's own, or (serving many
// analyses) the job's entry of b.devs copied into shared memory.
__device__ __forceinline__ const Device &item_device(const Device &d, const BatchDev &b,
                                                    const BatchJob &job, Device &dsm) {
    if (!b.devs) return d;
    const int *src = reinterpret_cast<const int *>(b.devs + job.dev);
    int *dst = reinterpret_cast<int *>(&dsm);
    for (int k = threadIdx.x; k < (int)(sizeof(Device) / sizeof(int)); k += blockDim.x)
        dst[k] = src[k];
    __syncthreads();
    return dsm;
}

// Resident CTAs per SM (register budget 65536 / (128 x CTAs)): measured on
// GB300, the FP64 form of the same-event kernel is fastest at 5 (its FP64
// values need the registers), the double-float form at 4 (118 registers, no
// spills: 167 ms per central group, against 194 ms at 5 and 234 ms at 6,
// where its 80 registers spill in the pair loop), the FP32-weight form and
// the mixed-event kernel at 6.
template <int PREC>
struct SameCtas {
    static constexpr int value = PREC == 1 ? 6 : (PREC == 2 ? 4 : 5);
};
constexpr int kMixedCtas = 6;

// Same-event items [base, min(end, queued)) pulled by persistent CTAs.
// MODE: fast binning, or one pass of ordered cap admission.
template <bool AZ, bool BOOST, int PREC, int MODE>
__global__ void __launch_bounds__(FT, SameCtas<PREC>::value) k_persistent_same(Device d, BatchDev b, unsigned base,
                                                           unsigned end) {
    __shared__ TileSmem sm;
    __shared__ Device dsm;
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
        const Item it = b.items[k];
        const BatchJob &job = b.jobs[it.job];
        const Device &dd = item_device(d, b, job, dsm);
        const BatchList &la = b.lists[job.la];
        const double *c[8];
#pragma unroll
        for (int f = 0; f < 8; f++) c[f] = b.table + (long long)f * b.cap + la.off;
        same_tile_pair<AZ, BOOST, PREC, MODE>(dd, sm, cs, c, b.orig + la.off, la.n,
                                              (long long)it.ti * FT, (long long)it.tj * FT);
        __syncthreads();
    }
}

// Mixed-event items, all in one launch.
template <bool AZ, bool BOOST, int MODE>
__global__ void __launch_bounds__(FT, kMixedCtas) k_persistent_mixed(Device d, BatchDev b) {
    __shared__ TileSmem sm;
    __shared__ Device dsm;
    __shared__ unsigned item;
    const unsigned stop = min(b.n_items[1], b.mixed_cap);
    for (;;) {
        if (threadIdx.x == 0) item = atomicAdd(b.item_next + 1, 1u);
        __syncthreads();
        const unsigned k = item;
        if (k >= stop) break;
        const Item it = b.items[b.same_cap + k];
        const BatchJob &job = b.jobs[it.job];
        const Device &dd = item_device(d, b, job, dsm);
        const BatchList &la = b.lists[job.la], &lb = b.lists[job.lb];
        const double *c1[4], *c2[4];
#pragma unroll
        for (int f = 0; f < 4; f++) {
            c1[f] = b.table + (long long)f * b.cap + la.off;
            c2[f] = b.table + (long long)f * b.cap + lb.off;
        }
        mixed_tile_pair<AZ, BOOST, MODE>(dd, sm, c1, la.n, c2, lb.n, (long long)it.ti * FT,
                                         (long long)it.tj * FT, b.orig + la.off,
                                         b.orig + lb.off);
        __syncthreads();
    }
}

int sm_count() {
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

template <bool AZ, bool BOOST, int PREC, int MODE>
cudaError_t launch_same_items(const Device &d, const BatchDev &b, unsigned base, unsigned end,
                              int grid, cudaStream_t st) {
    grid = persistent_grid(k_persistent_same<AZ, BOOST, PREC, MODE>, grid);
    k_persistent_same<AZ, BOOST, PREC, MODE><<<grid, FT, 0, st>>>(d, b, base, end);
    return cudaGetLastError();
}

template <bool AZ, bool BOOST, int MODE>
cudaError_t launch_mixed_items(const Device &d, const BatchDev &b, int grid, cudaStream_t st) {
    grid = persistent_grid(k_persistent_mixed<AZ, BOOST, MODE>, grid);
    k_persistent_mixed<AZ, BOOST, MODE><<<grid, FT, 0, st>>>(d, b);
    return cudaGetLastError();
}

// The same-event kernel for a precision form and admission mode.  The
// COUNT pass only counts decided pairs per row, the same in every form, so
// it runs the FP64 form's kernel.
template <int MODE>
cudaError_t launch_same_mode(const Device &d, const BatchDev &b, unsigned base, unsigned end,
                             int grid, cudaStream_t st) {
    const bool az = d.g.azimuthal, boost = d.g.boost;
    // the forms this mode instantiates: FP64 only for COUNT
    constexpr int P1 = MODE == MODE_COUNT ? 0 : 1, P2 = MODE == MODE_COUNT ? 0 : 2;
    const int prec = MODE == MODE_COUNT ? 0 : d.precision;
#define HBT_P(AZ_, BO_, PR_) return launch_same_items<AZ_, BO_, PR_, MODE>(d, b, base, end, grid, st)
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

template <int MODE>
cudaError_t launch_mixed_mode(const Device &d, const BatchDev &b, int grid, cudaStream_t st) {
    const bool az = d.g.azimuthal, boost = d.g.boost;
    if (az && boost) return launch_mixed_items<true, true, MODE>(d, b, grid, st);
    if (az) return launch_mixed_items<true, false, MODE>(d, b, grid, st);
    if (boost) return launch_mixed_items<false, true, MODE>(d, b, grid, st);
    return launch_mixed_items<false, false, MODE>(d, b, grid, st);
}

}  // namespace

int persistent_blocks_per_sm() {
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_persistent_same<true, true, 0, MODE_FAST>, FT,
                                                      0) != cudaSuccess)
        return 4;
    return nb > 0 ? nb : 1;
}

size_t batch_sort_temp_bytes(long long cap) {
    size_t bytes = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, bytes, (const unsigned long long *)nullptr,
                                    (unsigned long long *)nullptr, (const unsigned *)nullptr,
                                    (unsigned *)nullptr, (int)cap, 0, 64);
    return bytes;
}

cudaError_t run_batch(const Device &d, const BatchDev &b, int grid, unsigned chunk,
                      const Device *host_devs, int n_host_devs, cudaStream_t st,
                      cudaEvent_t *marks, int mode) {
    cudaError_t e;
    const int gs = 152 * 8;
    if (b.total > 0) {
        k_keys<<<gs, 256, 0, st>>>(b);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        int end_bit = 32;
        while (end_bit < 64 && (1LL << (end_bit - 32)) < b.n_lists) end_bit++;
        size_t bytes = b.sort_temp_bytes;
        e = cub::DeviceRadixSort::SortPairs(b.sort_temp, bytes, b.keys_in, b.keys_out, b.vals_in,
                                            b.vals_out, (int)b.total, 0, end_bit, st);
        if (e != cudaSuccess) return e;
        k_gather<<<gs, 256, 0, st>>>(b);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        k_boxes<<<(unsigned)((b.total_tiles * 32 + 255) / 256), 256, 0, st>>>(b);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    if ((e = cudaMemsetAsync(b.n_items, 0, 2 * sizeof(unsigned), st)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(b.item_next, 0, 2 * sizeof(unsigned), st)) != cudaSuccess) return e;
    if (b.total_pairs > 0) {
        k_cull<<<gs, 256, 0, st>>>(b);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    // the COUNT pass bins nothing: no FP32 partials to merge
    const int prec = mode == MODE_COUNT ? 0 : d.precision;
    // same-event items (chunked for the FP32-weight form)
    const unsigned upper = b.same_cap;
    if (chunk == 0 || prec != 1) chunk = upper;
    if (marks && (e = cudaEventRecord(marks[0], st)) != cudaSuccess) return e;
    for (unsigned base = 0; base < upper; base += chunk) {
        const unsigned end =
            (unsigned)min((unsigned long long)base + chunk, (unsigned long long)upper);
        if (base > 0 && (e = cudaMemsetAsync(b.item_next, 0, sizeof(unsigned), st)) != cudaSuccess)
            return e;
        if (mode == MODE_COUNT)
            e = launch_same_mode<MODE_COUNT>(d, b, base, end, grid, st);
        else if (mode == MODE_ORDER)
            e = launch_same_mode<MODE_ORDER>(d, b, base, end, grid, st);
        else
            e = launch_same_mode<MODE_FAST>(d, b, base, end, grid, st);
        if (e != cudaSuccess) return e;
        if (prec == 1 && !b.devs) {
            if ((e = launch_merge(d, st, b.n_items, base)) != cudaSuccess) return e;
        } else if (prec == 1) {
            for (int k = 0; k < n_host_devs; k++)
                if ((e = launch_merge(host_devs[k], st, b.n_items, base)) != cudaSuccess) return e;
        }
    }
    if (marks && (e = cudaEventRecord(marks[1], st)) != cudaSuccess) return e;
    if (marks && (e = cudaEventRecord(marks[2], st)) != cudaSuccess) return e;
    // mixed-event items
    if (b.mixed_cap > 0) {
        if (mode == MODE_COUNT)
            e = launch_mixed_mode<MODE_COUNT>(d, b, grid, st);
        else if (mode == MODE_ORDER)
            e = launch_mixed_mode<MODE_ORDER>(d, b, grid, st);
        else
            e = launch_mixed_mode<MODE_FAST>(d, b, grid, st);
        if (e != cudaSuccess) return e;
    }
    if (marks && (e = cudaEventRecord(marks[3], st)) != cudaSuccess) return e;
    return cudaSuccess;
}

}  // namespace hbt
