// Grid launches of the screened tile-pair kernels (hbt_tile.cuh) for one
// list or one list pair, plus the merge of the FP32-weight partial sums.
//
//   k_same_screened   one CTA per triangular (i-tile <= j-tile) pair
//   k_mixed_screened  one CTA per (list-1 tile, list-2 tile)
//   k_merge_partials  FP32 partial bins -> FP64 bins, Kahan-compensated
//
// The batched, culled, persistent form of the same tile bodies is in
// hbt_batch.cu.
#include "hbt_tile.cuh"

namespace hbt {
namespace {

using namespace tile;

template <bool AZ, bool BOOST, int PREC>
__global__ void __launch_bounds__(FT) k_same_screened(Device d, long long n, Cols8 c) {
    __shared__ TileSmem sm;
    __shared__ double2 cs[COS_TABLE];
    if (PREC == 0) fill_cos_table(cs);
    if (PREC == 2) fill_df_table(reinterpret_cast<float4 *>(cs));
    long long ti, tj;
    tri_tile((long long)blockIdx.x + d.block_offset, ti, tj);
    same_tile_pair<AZ, BOOST, PREC>(d, sm, cs, c.p, nullptr, n, ti * FT, tj * FT);
}

template <bool AZ, bool BOOST>
__global__ void __launch_bounds__(FT) k_mixed_screened(Device d, long long n1, Cols4 l1,
                                                       long long n2, Cols4 l2, long long tiles1) {
    __shared__ TileSmem sm;
    const long long ti = blockIdx.x % tiles1, tj = blockIdx.x / tiles1;
    mixed_tile_pair<AZ, BOOST>(d, sm, l1.p, n1, l2.p, n2, ti * FT, tj * FT);
}

}  // namespace

// FP32 partial sums -> FP64 bins with Kahan compensation; partials cleared.
__global__ void __launch_bounds__(256) k_merge_partials(Device d, long long nbins,
                                                        const unsigned *n_items,
                                                        unsigned chunk_base) {
    // a chunk of the batched queue past its culled length binned nothing
    if (n_items && chunk_base >= *n_items) return;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < nbins;
         k += (long long)gridDim.x * blockDim.x) {
        const float4 p = d.part[k], r = d.part_b[k];
        if (p.x == 0.0f && p.y == 0.0f && p.z == 0.0f && p.w == 0.0f && r.x == 0.0f &&
            r.y == 0.0f && r.z == 0.0f && r.w == 0.0f)
            continue;
        Sums s = d.h.sums[k];
        Sums c = d.comp[k];
        // the two partials' sum in FP64 (exact unless their exponents differ
        // by more than 28)
        const double in[4] = {(double)p.x + (double)r.x, (double)p.y + (double)r.y,
                              (double)p.z + (double)r.z, (double)p.w + (double)r.w};
        double *sv[4] = {&s.qo, &s.qs, &s.ql, &s.w};
        double *cv[4] = {&c.qo, &c.qs, &c.ql, &c.w};
#pragma unroll
        for (int f = 0; f < 4; f++) {
            const double y = in[f] - *cv[f];
            const double t = *sv[f] + y;
            *cv[f] = (t - *sv[f]) - y;
            *sv[f] = t;
        }
        d.h.sums[k] = s;
        d.comp[k] = c;
        d.part[k] = make_float4(0.f, 0.f, 0.f, 0.f);
        d.part_b[k] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
}

cudaError_t launch_merge(const Device &d, cudaStream_t st, const unsigned *n_items,
                         unsigned chunk_base) {
    const long long nbins = (long long)d.g.n_slots * d.g.q3;
    k_merge_partials<<<(unsigned)min((nbins + 255) / 256, 152LL * 16), 256, 0, st>>>(
        d, nbins, n_items, chunk_base);
    return cudaGetLastError();
}

cudaError_t launch_same_fast(const Device &d0, long long n, const double *const *c8,
                             cudaStream_t st) {
    if (n < 2) return cudaSuccess;
    const long long nt = (n + FT - 1) / FT;
    const long long blocks = nt * (nt + 1) / 2;
    Cols8 c;
    for (int f = 0; f < 8; f++) c.p[f] = c8[f];
    const bool az = d0.g.azimuthal, boost = d0.g.boost;
    const int prec = d0.precision;
    // FP32 partials are merged every `chunk` CTAs to bound the number of
    // terms an FP32 partial bin accumulates
    long long chunk = prec == 1 ? (d0.merge_chunk_blocks > 0 ? d0.merge_chunk_blocks : blocks)
                                : blocks;
    chunk = min(chunk, 0x7fffffffLL);
    for (long long b0 = 0; b0 < blocks; b0 += chunk) {
        Device d = d0;
        d.block_offset = b0;
        const unsigned nb = (unsigned)min(chunk, blocks - b0);
#define HBT_SAME(AZ_, BO_, PR_) k_same_screened<AZ_, BO_, PR_><<<nb, FT, 0, st>>>(d, n, c)
        if (prec == 0) {
            if (az && boost) HBT_SAME(true, true, 0);
            else if (az) HBT_SAME(true, false, 0);
            else if (boost) HBT_SAME(false, true, 0);
            else HBT_SAME(false, false, 0);
        } else if (prec == 1) {
            if (az && boost) HBT_SAME(true, true, 1);
            else if (az) HBT_SAME(true, false, 1);
            else if (boost) HBT_SAME(false, true, 1);
            else HBT_SAME(false, false, 1);
        } else {
            if (az && boost) HBT_SAME(true, true, 2);
            else if (az) HBT_SAME(true, false, 2);
            else if (boost) HBT_SAME(false, true, 2);
            else HBT_SAME(false, false, 2);
        }
#undef HBT_SAME
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        if (prec == 1) {
            e = launch_merge(d0, st);
            if (e != cudaSuccess) return e;
        }
    }
    return cudaSuccess;
}

cudaError_t launch_mixed_fast(const Device &d, long long n1, const double *const *l1,
                              long long n2, const double *const *l2, cudaStream_t st) {
    if (n1 < 1 || n2 < 1) return cudaSuccess;
    const long long t1 = (n1 + FT - 1) / FT, t2 = (n2 + FT - 1) / FT;
    const long long blocks = t1 * t2;
    if (blocks > 0x7fffffffLL) return cudaErrorInvalidValue;
    Cols4 a, b;
    for (int f = 0; f < 4; f++) {
        a.p[f] = l1[f];
        b.p[f] = l2[f];
    }
    const bool az = d.g.azimuthal, boost = d.g.boost;
    if (az && boost)
        k_mixed_screened<true, true><<<(unsigned)blocks, FT, 0, st>>>(d, n1, a, n2, b, t1);
    else if (az)
        k_mixed_screened<true, false><<<(unsigned)blocks, FT, 0, st>>>(d, n1, a, n2, b, t1);
    else if (boost)
        k_mixed_screened<false, true><<<(unsigned)blocks, FT, 0, st>>>(d, n1, a, n2, b, t1);
    else
        k_mixed_screened<false, false><<<(unsigned)blocks, FT, 0, st>>>(d, n1, a, n2, b, t1);
    return cudaGetLastError();
}

}  // namespace hbt
