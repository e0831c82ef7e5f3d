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
//     With q_inv histograms the LCMS q_long bound alone also keeps a tile
//     pair (boxes_may_pair).  Each bound carries a 1e-6 relative margin for
//     rounding;
//  4. k_persistent_same / k_persistent_mixed (hbt_persist.cuh): persistent
//     CTAs (4 to 6 per SM) pull (job, i-tile, j-tile) items from the culled
//     same-event and mixed-event queues and run the screened tile-pair
//     bodies of hbt_tile.cuh.  The FP32-weight form runs the same-event
//     queue in chunks and merges the FP32 partials between them.
#include <cub/device/device_radix_sort.cuh>

#include "hbt_batch.cuh"
#include "hbt_persist.cuh"
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
    double z0 = 1e300, z1 = -1e300, mm0 = 1e300, mm1 = -1e300;
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
        const double mm = m2 - (px * px + py * py);
        if (mm == mm) {
            mm0 = fmin(mm0, mm);
            mm1 = fmax(mm1, mm);
        } else {
            mm0 = -1e300;  // never treated as one mass
            mm1 = 1e300;
        }
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
        mm0 = fmin(mm0, __shfl_xor_sync(0xffffffffu, mm0, o));
        mm1 = fmax(mm1, __shfl_xor_sync(0xffffffffu, mm1, o));
    }
    if (lane == 0) b.boxes[warp] = Box{x0, x1, y0, y1, Y0, Y1, m0, z0, z1, mm0, mm1};
}

// Can a pair with one particle in box a and one in box b pass the windows?
// The 3-D windows bound q_x^2 + q_y^2 and |q_long|; the LCMS q_long of two
// particles with transverse masses m_1, m_2 and rapidity gap dy is
// 2 m_1 m_2 sinh(dy) / sqrt(m_1^2 + m_2^2 + 2 m_1 m_2 cosh(dy)), which
// grows with dy, m_1 and m_2, so the boxes' smallest m_T and gap bound it
// from below.  With q_inv histograms a pair may also pass the q_inv window:
// for two particles of one mass q.K = 0, so in the LCMS
// q_inv^2 = q_out^2 (1 - beta_T^2) + q_side^2 + q_long^2 >= q_long^2, and
// only the q_long bound culls (tiles whose masses differ keep every pair).
__device__ __forceinline__ bool boxes_may_pair(const BatchJob &b, const Box &a, const Box &c) {
    const double gY = fmax(0.0, fmax(a.Y0 - c.Y1, c.Y0 - a.Y1));
    double qlong_lcms = 0.0;  // lower bound of |q_long| in the LCMS
    if (gY > 0.0) {
        const double m1 = a.m0, m2 = c.m0;
        qlong_lcms = 2.0 * m1 * m2 * sinh(gY) /
                     sqrt(m1 * m1 + m2 * m2 + 2.0 * m1 * m2 * cosh(gY));
    }
    const double gx = fmax(0.0, fmax(a.x0 - c.x1, c.x0 - a.x1));
    const double gy = fmax(0.0, fmax(a.y0 - c.y1, c.y0 - a.y1));
    bool pass3 = !(gx * gx + gy * gy > b.qt2_max);
    if (b.boost) {
        pass3 = pass3 && !(qlong_lcms > b.ql_max);
    } else {
        // q_long = q_z
        const double gz = fmax(0.0, fmax(a.z0 - c.z1, c.z0 - a.z1));
        pass3 = pass3 && !(gz > b.ql_max);
    }
    if (pass3 || !b.qinv) return pass3;
    const double lo = fmin(a.mm0, c.mm0), hi = fmax(a.mm1, c.mm1);
    if (!(hi - lo <= 1e-9 * fabs(hi))) return true;
    return !(qlong_lcms > b.ql_max);
}

// Momentum-space region of a tile pair's pairs: K = (p_1 + p_2) / 2 at the
// boxes' centres, in K_T cells of 1/32 GeV (up to 2 GeV) and 32 azimuthal
// sectors, above the analysis index (serving).  Items of one region update
// the same few histogram slots.
__device__ __forceinline__ unsigned region_key(const BatchJob &job, const Box &a, const Box &c) {
    const double kx = 0.25 * (a.x0 + a.x1 + c.x0 + c.x1);
    const double ky = 0.25 * (a.y0 + a.y1 + c.y0 + c.y1);
    const double kt = sqrt(kx * kx + ky * ky);
    const unsigned kc = kt < 2.0 ? (unsigned)(kt * 32.0) : 63u;
    double ph = atan2(ky, kx) * (16.0 / 3.141592653589793) + 16.0;  // [0, 32]
    const unsigned pc = ph >= 0.0 && ph < 32.0 ? (unsigned)ph : 0u;
    // (below 0x1FFFFF, so that no key equals the unused entries' 0xffffffff)
    const unsigned dev = job.dev < 0x1FFFFE ? (unsigned)job.dev : 0x1FFFFEu;
    return (dev << 11) | (kc << 5) | pc;
}

// Ordered cap admission: the 3-D slots already at their cap (of the pass's
// counter family) and the grid constants that map a tile pair to the slots
// its pairs can reach.  full == nullptr: no slot test.
struct SlotCull {
    const unsigned char *full;
    double KT_min, dKT, KT_min_sq, KT_max_sq, psi, dKphi, two_pi;
    int n_KT, n_Kphi, az;
};

// Can the pairs of boxes a and c reach only slots already at their cap?
// K = (p_1 + p_2) / 2 lies in the rectangle of the boxes' mean p_x, p_y
// ranges: its K_T range (nearest and farthest points) gives the K_T bins the
// reference can assign (K_perp^2 in [KT_min^2, KT_max^2], src/HBT_correlation.cpp
// :323-366), its angle range the K_phi bins (:408-422), each widened by a
// margin far above rounding.  A rectangle that holds the origin is never
// skipped (its pairs may have K_perp = 0, counted as anomalies).  Admission
// admits nothing more in a full slot, so such a tile pair needs neither the
// count nor the order pass.
__device__ bool slots_all_full(const SlotCull &sc, const Box &a, const Box &c) {
    const double x0 = 0.5 * (a.x0 + c.x0), x1 = 0.5 * (a.x1 + c.x1);
    const double y0 = 0.5 * (a.y0 + c.y0), y1 = 0.5 * (a.y1 + c.y1);
    if (x0 <= 0.0 && x1 >= 0.0 && y0 <= 0.0 && y1 >= 0.0) return false;
    const double nx = x0 > 0.0 ? x0 : (x1 < 0.0 ? x1 : 0.0);
    const double ny = y0 > 0.0 ? y0 : (y1 < 0.0 ? y1 : 0.0);
    const double fx = fmax(fabs(x0), fabs(x1)), fy = fmax(fabs(y0), fabs(y1));
    const double k2lo = (nx * nx + ny * ny) * (1.0 - 1e-9), k2hi = (fx * fx + fy * fy) * (1.0 + 1e-9);
    if (k2hi < sc.KT_min_sq || k2lo > sc.KT_max_sq) return true;  // no pair in the K_T window
    const double klo = sqrt(fmax(k2lo, sc.KT_min_sq)), khi = sqrt(fmin(k2hi, sc.KT_max_sq));
    const int i0 = max(0, (int)floor((klo - sc.KT_min) / sc.dKT - 1e-6));
    const int i1 = min(sc.n_KT - 1, (int)floor((khi - sc.KT_min) / sc.dKT + 1e-6));
    if (!sc.az) {
        for (int k = i0; k <= i1; k++)
            if (!sc.full[k]) return false;
        return true;
    }
    // the angle range around the centre's direction (under pi: the
    // rectangle does not hold the origin), as bins modulo n_Kphi
    const double cth = atan2(0.5 * (y0 + y1), 0.5 * (x0 + x1));
    const double cx[4] = {x0, x1, x0, x1}, cy[4] = {y0, y0, y1, y1};
    double lo = 0.0, hi = 0.0;
    for (int q = 0; q < 4; q++) {
        const double da = remainder(atan2(cy[q], cx[q]) - cth, sc.two_pi);
        lo = fmin(lo, da);
        hi = fmax(hi, da);
    }
    double u = cth + lo - 1e-6 - sc.psi;
    u -= sc.two_pi * floor(u / sc.two_pi);
    const int p0 = (int)floor(u / sc.dKphi);
    const int p1 = (int)floor((u + hi - lo + 2e-6) / sc.dKphi);
    const int np = min(sc.n_Kphi, p1 - p0 + 1);
    for (int k = i0; k <= i1; k++)
        for (int t = 0; t < np; t++) {
            const int ip = ((p0 + t) % sc.n_Kphi + sc.n_Kphi) % sc.n_Kphi;  // u may round below 0
            if (!sc.full[k * sc.n_Kphi + ip]) return false;
        }
    return true;
}

// Culled queues: same-event items at items[0, same_cap), mixed-event items
// at items[same_cap, same_cap + mixed_cap); n_items[0] / n_items[1] count them.
__global__ void k_cull(BatchDev b, SlotCull sc) {
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
        if (boxes_may_pair(job, A, B) && !(sc.full && !job.qinv && slots_all_full(sc, A, B))) {
            const Item it = Item{(unsigned)J, (unsigned)ti, (unsigned)tj};
            if (job.kind == 0) {
                const unsigned slot = atomicAdd(b.n_items, 1u);
                if (slot < b.same_cap) {
                    b.items[slot] = it;
                    if (b.order_items) {
                        b.item_key_in[slot] = region_key(job, A, B);
                        b.item_pos_in[slot] = slot;
                    }
                }
            } else {
                const unsigned slot = atomicAdd(b.n_items + 1, 1u);
                if (slot < b.mixed_cap) b.items[b.same_cap + slot] = it;
            }
        }
    }
}

}  // namespace

cudaError_t persistent_same(const Device &d, const BatchDev &b, unsigned base, unsigned end,
                            int grid, cudaStream_t st, int mode) {
    if (d.g.qinv)
        return mode == MODE_FAST ? persistent_same_qinv(d, b, base, end, grid, st)
                                 : cudaErrorNotSupported;
    if (mode == MODE_FAST) return persistent_same_fast(d, b, base, end, grid, st);
    return persistent_same_ordered(d, b, base, end, grid, st, mode);
}

cudaError_t persistent_mixed(const Device &d, const BatchDev &b, int grid, cudaStream_t st,
                             int mode) {
    if (d.g.qinv)
        return mode == MODE_FAST ? persistent_mixed_qinv(d, b, grid, st) : cudaErrorNotSupported;
    if (mode == MODE_FAST) return persistent_mixed_fast(d, b, grid, st);
    return persistent_mixed_ordered(d, b, grid, st, mode);
}

size_t item_sort_temp_bytes(long long n) {
    size_t bytes = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, bytes, (const unsigned *)nullptr,
                                    (unsigned *)nullptr, (const unsigned *)nullptr,
                                    (unsigned *)nullptr, (int)n, 0, 32);
    return bytes;
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
    if (b.order_items && b.same_cap > 0 &&
        (e = cudaMemsetAsync(b.item_key_in, 0xff, (size_t)b.same_cap * sizeof(unsigned), st)) !=
            cudaSuccess)
        return e;
    if (b.total_pairs > 0) {
        SlotCull sc = {};
        if (mode != MODE_FAST && d.caps.slot_full && !b.devs) {
            sc.full = d.caps.slot_full;
            sc.KT_min = d.g.KT_min;
            sc.dKT = d.g.dKT;
            sc.KT_min_sq = d.g.KT_min_sq;
            sc.KT_max_sq = d.g.KT_max_sq;
            sc.psi = d.g.psi_ref;
            sc.dKphi = d.g.dKphi;
            sc.two_pi = d.g.two_pi;
            sc.n_KT = d.g.n_KT;
            sc.n_Kphi = d.g.n_Kphi;
            sc.az = d.g.azimuthal;
        }
        k_cull<<<gs, 256, 0, st>>>(b, sc);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    if (b.order_items && b.same_cap > 0) {
        // unused entries keep the key 0xffffffff and sort behind the queue
        size_t bytes = b.item_sort_temp_bytes;
        e = cub::DeviceRadixSort::SortPairs(b.item_sort_temp, bytes, b.item_key_in,
                                            b.item_key_out, b.item_pos_in, b.item_pos_out,
                                            (int)b.same_cap, 0, 32, st);
        if (e != cudaSuccess) return e;
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
        e = persistent_same(d, b, base, end, grid, st, mode);
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
        e = persistent_mixed(d, b, grid, st, mode);
        if (e != cudaSuccess) return e;
    }
    if (marks && (e = cudaEventRecord(marks[3], st)) != cudaSuccess) return e;
    return cudaSuccess;
}

}  // namespace hbt
