// Device evaluation of the table-driven FP64 functions and of the
// double-float cos of the pair kernels (include/hbt_check.h).
#include "../../include/hbt_check.h"
#include "hbt_math.cuh"
#include "hbt_tile.cuh"

namespace {

// df_cos of each argument split into (hi, lo) FP32 parts, as the
// double-float pair kernels split their columns.
__global__ void k_check_dfcos(long long n, const double *x, double *out) {
    __shared__ float4 t[hbt::tile::DF_TABLE];
    hbt::tile::fill_df_table(t);
    __syncthreads();
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const float2 s = hbt::tile::split(x[i]);
        out[i] = hbt::tile::df_cos(t, hbt::tile::FF{s.x, s.y});
    }
}

__global__ void k_check_math(int which, CosScale k, long long n, const double *x, double *out) {
    __shared__ double2 cs[COS_TABLE];
    __shared__ double et[EXP_TABLE];
    fill_cos_table(cs);
    fill_exp_table(et);
    __syncthreads();
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        double v;
        if (which == HBT_CHECK_COS || which == HBT_CHECK_COS_PHASE)
            v = table_cos(cs, k, x[i]);
        else
            v = table_exp(et, x[i]);
        out[i] = v;
    }
}

}  // namespace

extern "C" hbt_status hbt_check_math(int device, int32_t which, int64_t n, const double *x,
                                     double *out) {
    if (n < 0 || (n > 0 && (!x || !out)) ||
        which < HBT_CHECK_COS || which > HBT_CHECK_COS_PHASE)
        return HBT_ERR_INVALID;
    if (n == 0) return HBT_OK;
    if (cudaSetDevice(device) != cudaSuccess) return HBT_ERR_CUDA;
    double *d = nullptr;
    if (cudaMalloc(&d, 2 * n * sizeof(double)) != cudaSuccess) return HBT_ERR_NOMEM;
    cudaError_t e = cudaMemcpy(d, x, n * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        const long long blocks = (n + 255) / 256 < 1024 ? (n + 255) / 256 : 1024;
        if (which == HBT_CHECK_DFCOS)
            k_check_dfcos<<<(unsigned)blocks, 256>>>(n, d, d + n);
        else
            k_check_math<<<(unsigned)blocks, 256>>>(
                which, make_cos_scale(which == HBT_CHECK_COS_PHASE ? 1.0 / hbt::kHbarC : 1.0), n,
                d, d + n);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(out, d + n, n * sizeof(double), cudaMemcpyDeviceToHost);
    cudaFree(d);
    return e == cudaSuccess ? HBT_OK : HBT_ERR_CUDA;
}
