// Throughput probes used by the benchmark to measure, on the GPU it runs
// on, the peak rates the HBT kernels are bound by: the FP64 and FP32 fused
// multiply-add issue rate (each thread runs 8 independent FMA chains in
// registers and writes one value, so the memory traffic is one store per
// thread), the rates of the FP64 divide, square root and cosine the
// reference's per-pair chain uses (the same 8-chain layout), and the rate
// of FP64 atomic adds to scattered addresses of an array larger than L2
// (the histogram updates).
#include <cuda_runtime.h>

namespace {

template <typename T>
__global__ void __launch_bounds__(256) k_fma(T *out, int iters, T a, T b) {
    T x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
    T x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (int k = 0; k < iters; k++) {
        x0 = x0 * a + b;
        x1 = x1 * a + b;
        x2 = x2 * a + b;
        x3 = x3 * a + b;
        x4 = x4 * a + b;
        x5 = x5 * a + b;
        x6 = x6 * a + b;
        x7 = x7 * a + b;
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

template <typename T>
int run(int blocks, int iters, float *ms, double *flops) {
    T *out = nullptr;
    if (cudaMalloc(&out, (size_t)blocks * 256 * sizeof(T)) != cudaSuccess) return 1;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    k_fma<T><<<blocks, 256>>>(out, iters / 8 + 1, (T)0.999, (T)0.001);  // warm-up
    cudaEventRecord(e0);
    k_fma<T><<<blocks, 256>>>(out, iters, (T)0.999, (T)0.001);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(ms, e0, e1);
    *flops = 2.0 * 8.0 * (double)iters * blocks * 256.0;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    const cudaError_t err = cudaGetLastError();
    cudaFree(out);
    return err == cudaSuccess ? 0 : 2;
}

// Chains of one FP64 operation: op 0 divide (x = 1 / (x + 1.5)), 1 square
// root (x = sqrt(x + 0.25)), 2 cosine (x = cos(x + 0.5)), each step the
// operation plus one add; the values stay bounded and away from special
// cases, so every step takes the operation's ordinary path.
template <int OP>
__global__ void __launch_bounds__(256) k_op64(double *out, int iters) {
    double x[8];
#pragma unroll
    for (int c = 0; c < 8; c++) x[c] = 0.25 + 0.01 * (threadIdx.x & 7) + 0.03 * c;
    for (int k = 0; k < iters; k++) {
#pragma unroll
        for (int c = 0; c < 8; c++) {
            if (OP == 0) x[c] = 1.0 / (x[c] + 1.5);
            if (OP == 1) x[c] = sqrt(x[c] + 0.25);
            if (OP == 2) x[c] = cos(x[c] + 0.5);
        }
    }
    double s = 0.0;
#pragma unroll
    for (int c = 0; c < 8; c++) s += x[c];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <int OP>
int run_op(int blocks, int iters, float *ms, double *ops) {
    double *out = nullptr;
    if (cudaMalloc(&out, (size_t)blocks * 256 * sizeof(double)) != cudaSuccess) return 1;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    k_op64<OP><<<blocks, 256>>>(out, iters / 8 + 1);  // warm-up
    cudaEventRecord(e0);
    k_op64<OP><<<blocks, 256>>>(out, iters);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(ms, e0, e1);
    *ops = 8.0 * (double)iters * blocks * 256.0;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    const cudaError_t err = cudaGetLastError();
    cudaFree(out);
    return err == cudaSuccess ? 0 : 2;
}

// FP64 atomic adds at pseudo-random positions of a 2^log2 array: each
// thread walks its own xorshift-multiply sequence, `iters` adds.
__global__ void __launch_bounds__(256) k_atomic(double *h, unsigned long long mask, int iters) {
    unsigned long long x = (blockIdx.x * 256ull + threadIdx.x + 1) * 0x9E3779B97F4A7C15ull;
    for (int k = 0; k < iters; k++) {
        x ^= x >> 31;
        x *= 0xBF58476D1CE4E5B9ull;
        x ^= x >> 29;
        atomicAdd(h + (x & mask), 1.0);
    }
}

}  // namespace

extern "C" {

// Scattered FP64 atomic-add throughput over 2^log2 doubles: returns 0 and
// the elapsed ms and the number of atomics.
int hbt_probe_atomic(int blocks, int iters, int log2, float *ms, double *ops) {
    if (log2 < 10 || log2 > 31) return 1;
    double *h = nullptr;
    const size_t n = (size_t)1 << log2;
    if (cudaMalloc(&h, n * sizeof(double)) != cudaSuccess) return 1;
    cudaMemset(h, 0, n * sizeof(double));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    k_atomic<<<blocks, 256>>>(h, n - 1, iters / 8 + 1);  // warm-up
    cudaEventRecord(e0);
    k_atomic<<<blocks, 256>>>(h, n - 1, iters);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(ms, e0, e1);
    *ops = (double)iters * blocks * 256.0;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    const cudaError_t err = cudaGetLastError();
    cudaFree(h);
    return err == cudaSuccess ? 0 : 2;
}

// FP64 FMA throughput: returns 0 and the elapsed ms and flop count.
int hbt_probe_fp64(int blocks, int iters, float *ms, double *flops) {
    return run<double>(blocks, iters, ms, flops);
}

// FP32 FMA throughput.
int hbt_probe_fp32(int blocks, int iters, float *ms, double *flops) {
    return run<float>(blocks, iters, ms, flops);
}

// FP64 divide (op 0), square root (1) or cosine (2) throughput, each
// operation with one add: returns 0 and the elapsed ms and operation count.
int hbt_probe_op64(int op, int blocks, int iters, float *ms, double *ops) {
    if (op == 0) return run_op<0>(blocks, iters, ms, ops);
    if (op == 1) return run_op<1>(blocks, iters, ms, ops);
    if (op == 2) return run_op<2>(blocks, iters, ms, ops);
    return 1;
}

}  // extern "C"
